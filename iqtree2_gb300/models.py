"""Host-side substitution-model inputs for the likelihood engine.

The engine consumes a reversible model through the same three arrays IQ-TREE 2
reads from ``ModelSubst`` (``getEigenvalues/getEigenvectors/
getInverseEigenvectors``, model/modelsubst.h:360-372) plus the discrete rate
categories of ``RateHeterogeneity`` (``getRate/getProp``,
model/rategamma.h:106,120) and the eigen-space tip vectors built by
``PhyloTree::computeTipPartialLikelihood`` (tree/phylotreesse.cpp:354-375).
This module builds those arrays for the models the benchmarks use: GTR (DNA),
LG (protein) and GY94 (codon), with +G discrete gamma rates.

The eigen-decomposition follows the reversible path of
``ModelMarkov::decomposeRateMatrix`` (model/modelmarkov.cpp:1450-1560):
symmetrise Q with sqrt(pi), solve the symmetric eigenproblem (eigenvalues
ascending), then U = diag(1/sqrt(pi)) V and U^-1 = V^T diag(sqrt(pi)).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np
from scipy import special

# aln->STATE_UNKNOWN per alphabet (alignment/alignment.cpp:738-745).
STATE_UNKNOWN = {4: 18, 20: 23, 61: 61}

_DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")

# Standard genetic code in TCAG order (first, second, third base).
_CODE_TCAG = "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG"
_TCAG_OF_ACGT = (2, 1, 3, 0)  # A C G T -> index in TCAG


def _codon_aa(n1, n2, n3):
    t = _TCAG_OF_ACGT
    return _CODE_TCAG[t[n1] * 16 + t[n2] * 4 + t[n3]]


def sense_codons():
    """Sense codons in IQ-TREE's order (nt1*16+nt2*4+nt3, ACGT), stops removed."""
    out = []
    for c in range(64):
        n1, n2, n3 = c // 16, (c // 4) % 4, c % 4
        if _codon_aa(n1, n2, n3) != "*":
            out.append((n1, n2, n3))
    return out


def normalize_rate_matrix(R, pi):
    """Q = R diag(pi) with zero row sums, scaled to one substitution per unit time.

    Mirrors the ``normalize_matrix`` branch of decomposeRateMatrix
    (model/modelmarkov.cpp:1504-1512): the scale factor is computed from the
    off-diagonal row sums before the diagonal is set.
    """
    R = np.array(R, dtype=np.float64)
    pi = np.asarray(pi, dtype=np.float64)
    Q = R * pi[None, :]
    np.fill_diagonal(Q, 0.0)
    row = Q.sum(axis=1)
    Q -= np.diag(row)
    Q *= 1.0 / float(row @ pi)
    return Q


def eigen_decompose(Q, pi):
    """(eval, U, U^-1) of a reversible Q in the reference's storage convention."""
    pi = np.asarray(pi, dtype=np.float64)
    s = np.sqrt(pi)
    S = (s[:, None] * Q) / s[None, :]
    S = 0.5 * (S + S.T)
    w, V = np.linalg.eigh(S)
    U = V / s[:, None]
    Uinv = V.T * s[None, :]
    return (np.ascontiguousarray(w), np.ascontiguousarray(U), np.ascontiguousarray(Uinv))


def gamma_rates_mean(alpha, ncat):
    """Discrete-gamma category rates by the mean method (Yang 1994).

    Restates ``RateGamma::computeRatesMean`` (model/rategamma.cpp:157-170):
    cut points are Gamma(alpha, alpha) quantiles; each rate is ncat times the
    Gamma(alpha+1) probability mass between consecutive cut points.
    """
    if ncat == 1:
        return np.ones(1), np.ones(1)
    k = np.arange(1, ncat)
    cuts = special.gammaincinv(alpha, k / ncat) / alpha
    mass = special.gammainc(alpha + 1.0, cuts * alpha)
    rates = np.empty(ncat)
    rates[0] = mass[0] * ncat
    rates[-1] = (1.0 - mass[-1]) * ncat
    rates[1:-1] = (mass[1:] - mass[:-1]) * ncat
    rates *= ncat / rates.sum()
    props = np.full(ncat, 1.0 / ncat)
    return rates, props


def gamma_invar_rates(alpha, p_invar, ncat):
    """+I+G: rates and proportions of the variable-site categories.

    Restates ``RateGammaInvar`` (model/rategammainvar.cpp:25-42 sets every
    rate to 1/(1-p_inv) before ``RateGamma::computeRates``, which rescales the
    discrete-gamma rates to that sum, model/rategamma.cpp:98-141) and its
    ``getProp`` = (1-p_inv)/ncat (model/rategammainvar.h:69).
    """
    rates, _ = gamma_rates_mean(alpha, ncat)
    return rates / (1.0 - p_invar), np.full(ncat, (1.0 - p_invar) / ncat)


def free_rates(rates, props):
    """+R (FreeRate) categories from given weights and rates: weights
    normalised to sum 1, rates divided by sum(prop * rate) so the mean rate is
    1 (the ``RateFree`` constructor, model/ratefree.cpp:38-75)."""
    r = np.asarray(rates, np.float64)
    p = np.asarray(props, np.float64)
    p = p / p.sum()
    return r / float(p @ r), p


def invariant_site_lh(patterns, pi, p_invar, nstates):
    """Per-pattern +I term (``ptn_invar``): p_inv times the summed frequency of
    the states every taxon of the pattern allows.

    Restates ``Alignment::computeConst`` (alignment/alignment.cpp:925-1012:
    the intersection of the taxa's state sets, ``getAppearance``
    :4769-4800) and ``PhyloTree::computePtnInvar``
    (tree/phylotreesse.cpp:549-610): a pattern of one state s gives
    p_inv * pi[s], an all-unknown pattern p_inv, an ambiguous intersection
    (DNA masks, protein B/Z/J) the sum over its states, an empty one 0.
    """
    app = tip_vectors(nstates)[np.asarray(patterns)]  # (taxa, patterns, states): which states each code allows
    common = np.prod(app, axis=0)
    return p_invar * (common @ np.asarray(pi, np.float64))


def variable_patterns(patterns, freq, nstates):
    """The patterns +ASC accepts: drops every pattern whose taxa share an
    allowed state (``is_invariant`` of alignment/alignment.cpp:1017-1019; the
    reference refuses +ASC on an alignment that has any,
    model/modelfactory.cpp:686-704)."""
    app = tip_vectors(nstates)[np.asarray(patterns)]
    keep = np.prod(app, axis=0).sum(axis=1) == 0
    return np.ascontiguousarray(np.asarray(patterns)[:, keep]), np.ascontiguousarray(np.asarray(freq)[keep])


def asc_lewis_patterns(patterns, freq, nstates, pi=None):
    """Appends +ASC's unobserved constant patterns: for every state s (with
    frequency >= 1e-8), the pattern of all taxa in s unless it is observed
    (``Alignment::getUnobservedConstPatterns`` ASC_VARIANT,
    alignment/alignment.cpp:4143-4156; rare states dropped as in
    model/modelfactory.cpp:679-682), with weight 0. Returns (patterns, freq,
    nconst, nsite) for ``Engine.set_asc`` and the oracle."""
    pats = np.asarray(patterns)
    seen = {tuple(col) for col in pats.T}
    extra = [s for s in range(nstates)
             if (pi is None or pi[s] >= 1e-8) and tuple([s] * pats.shape[0]) not in seen]
    cols = np.array([[s] * pats.shape[0] for s in extra], dtype=pats.dtype).T.reshape(pats.shape[0], len(extra))
    out = np.ascontiguousarray(np.concatenate([pats, cols], axis=1))
    f = np.concatenate([np.asarray(freq, np.float64), np.zeros(len(extra))])
    return out, f, len(extra), float(np.asarray(freq).sum())


def asc_informative_patterns(ntaxa, nstates, limit=200000):
    """Every uninformative pattern, the unobserved patterns of the +ASC
    correction for informative sites (ASC_INFORMATIVE, Lewis's formula over
    them; alignment/alignment.cpp:4104-4138, 4181-4192): for each repeat state
    r and each subset T of the other states (in bitmask order) with |T| <
    ntaxa - 1, or |T| = ntaxa - 1 when r = 0, every placement of T's states
    (in order) on distinct taxa (taxa tuples in lexicographic order), all other
    taxa in state r. Returns uint8 (ntaxa, count)."""
    from itertools import permutations
    out = []
    for r in range(nstates):
        rest = [s for s in range(nstates) if s != r]
        for mask in range(1 << len(rest)):
            T = [rest[i] for i in range(len(rest)) if mask & (1 << i)]
            if not (len(T) < ntaxa - 1 or (len(T) == ntaxa - 1 and r == 0)):
                continue
            for pos in permutations(range(ntaxa), len(T)):
                col = np.full(ntaxa, r, np.uint8)
                col[list(pos)] = T
                out.append(col)
                if len(out) > limit:
                    raise ValueError("too many uninformative patterns")
    return np.ascontiguousarray(np.stack(out, axis=1))


def asc_holder_patterns(patterns, freq, nstates):
    """Holder's +ASC for variant sites with missing data: append, after the
    observed patterns, nstates blocks of unobserved patterns with weight 0,
    block s holding for observed pattern p state s at every taxon where p has
    a state below nstates and STATE_UNKNOWN elsewhere (ASC_VARIANT_MISSING,
    alignment/alignment.cpp:4158-4180). Returns (patterns, freq, nobs)."""
    su = STATE_UNKNOWN.get(nstates, nstates)
    pat = np.asarray(patterns, np.uint8)
    nobs = pat.shape[1]
    known = pat < nstates
    blocks = [np.where(known, np.uint8(s), np.uint8(su)) for s in range(nstates)]
    return (np.ascontiguousarray(np.concatenate([pat] + blocks, axis=1)),
            np.concatenate([np.asarray(freq, np.float64), np.zeros(nstates * nobs)]), nobs)


def tip_vectors(nstates):
    """Standard-basis tip likelihood per alignment state, rows 0..STATE_UNKNOWN.

    Single states are unit vectors and STATE_UNKNOWN is all ones
    (ModelSubst::computeTipLikelihood, model/modelsubst.cpp:196-207). DNA
    ambiguity states 4..17 use the bitmask ``state-3`` (ModelDNA,
    model/modeldna.cpp:462-474); protein states 20..22 are B, Z and J
    (ModelProtein, model/modelprotein.cpp:1149-1165).
    """
    su = STATE_UNKNOWN.get(nstates, nstates)
    T = np.zeros((su + 1, nstates))
    for s in range(su + 1):
        if s < nstates:
            T[s, s] = 1.0
        elif nstates == 4 and s < 18:
            mask = s - 3
            for i in range(4):
                if mask & (1 << i):
                    T[s, i] = 1.0
        elif nstates == 20 and s < 23:
            pair = ((2, 3), (5, 6), (9, 10))[s - 20]
            T[s, pair[0]] = T[s, pair[1]] = 1.0
        else:
            T[s, :] = 1.0
    return T


@dataclass
class SubstModel:
    """A reversible model plus +G categories, in the engine's input form."""

    name: str
    nstates: int
    Q: np.ndarray
    pi: np.ndarray
    rates: np.ndarray
    props: np.ndarray
    eval: np.ndarray = field(init=False)
    evec: np.ndarray = field(init=False)
    inv_evec: np.ndarray = field(init=False)
    tip_lh: np.ndarray = field(init=False)

    def __post_init__(self):
        self.eval, self.evec, self.inv_evec = eigen_decompose(self.Q, self.pi)
        # eigen-space tip vectors: U^-1 . tipvec (ModelSubst::multiplyWithInvEigenvector)
        self.tip_lh = np.ascontiguousarray(tip_vectors(self.nstates) @ self.inv_evec.T)

    @property
    def ncat(self):
        return len(self.rates)

    @property
    def state_unknown(self):
        return STATE_UNKNOWN.get(self.nstates, self.nstates)

    def trans_matrix(self, t):
        """P(t) = U exp(Lambda t) U^-1 (standard basis)."""
        return (self.evec * np.exp(self.eval * t)[None, :]) @ self.inv_evec


def gtr_model(exch, pi, alpha, ncat=4):
    """GTR from 6 exchangeabilities (AC AG AT CG CT GT) and base frequencies."""
    R = np.zeros((4, 4))
    k = 0
    for i in range(4):
        for j in range(i + 1, 4):
            R[i, j] = R[j, i] = exch[k]
            k += 1
    pi = np.asarray(pi, dtype=np.float64)
    rates, props = gamma_rates_mean(alpha, ncat)
    return SubstModel("GTR+G%d" % ncat, 4, normalize_rate_matrix(R, pi), pi, rates, props)


def lg_exchangeabilities():
    """LG exchangeabilities (symmetric 20x20) and frequencies from ``data/lg.dat``."""
    vals = []
    with open(os.path.join(_DATA_DIR, "lg.dat")) as f:
        for line in f:
            if line.startswith("#"):
                continue
            vals.extend(float(t) for t in line.split())
    R = np.zeros((20, 20))
    k = 0
    for i in range(1, 20):
        for j in range(i):
            R[i, j] = R[j, i] = vals[k]
            k += 1
    freqs = np.array(vals[190:210])
    return R, freqs / freqs.sum()


def lg_model(pi, alpha, ncat=4):
    R, _ = lg_exchangeabilities()
    rates, props = gamma_rates_mean(alpha, ncat)
    pi = np.asarray(pi, dtype=np.float64)
    return SubstModel("LG+G%d" % ncat, 20, normalize_rate_matrix(R, pi), pi, rates, props)


def f3x4_frequencies(nt_pos_freqs):
    """F3x4 codon frequencies over the 61 sense codons (alignment/alignment.cpp:4924)."""
    f = np.asarray(nt_pos_freqs, dtype=np.float64).reshape(3, 4)
    pi = np.array([f[0, a] * f[1, b] * f[2, c] for (a, b, c) in sense_codons()])
    return pi / pi.sum()


def gy94_rate_matrix(kappa, omega):
    """GY94 exchangeabilities between the 61 sense codons.

    Non-zero only for codons that differ at one position; transitions carry
    kappa and non-synonymous changes carry omega, as in
    ``ModelCodon::computeCodonRateMatrix_1KAPPA`` (model/modelcodon.cpp:845-874).
    """
    cod = sense_codons()
    n = len(cod)
    R = np.zeros((n, n))
    for i, a in enumerate(cod):
        for j, b in enumerate(cod):
            if i == j:
                continue
            diff = [p for p in range(3) if a[p] != b[p]]
            if len(diff) != 1:
                continue
            p = diff[0]
            x, y = a[p], b[p]
            transition = {x, y} in ({0, 2}, {1, 3})
            synonymous = _codon_aa(*a) == _codon_aa(*b)
            r = 1.0
            if transition:
                r *= kappa
            if not synonymous:
                r *= omega
            R[i, j] = r
    return R


def gy94_model(kappa, omega, pi, alpha, ncat=4):
    R = gy94_rate_matrix(kappa, omega)
    rates, props = gamma_rates_mean(alpha, ncat)
    pi = np.asarray(pi, dtype=np.float64)
    return SubstModel("GY94+G%d" % ncat, 61, normalize_rate_matrix(R, pi), pi, rates, props)


@dataclass
class MixtureModel:
    """A mixture of reversible classes with +G rate categories, in the
    engine's input form (``Engine.set_mixture``): category c = m * ncat_rate
    + k is rate category k of class m (tree/phylokernelnew.h:908-918), its
    proportion the class weight times the rate proportion
    (tree/phylokernelnew.h:2327)."""

    name: str
    nstates: int
    classes: list
    weights: np.ndarray
    rate_rates: np.ndarray
    rate_props: np.ndarray

    @property
    def nmix(self):
        return len(self.classes)

    @property
    def ncat(self):
        return self.nmix * len(self.rate_rates)

    @property
    def state_unknown(self):
        return STATE_UNKNOWN.get(self.nstates, self.nstates)

    @property
    def cat_class(self):
        return np.repeat(np.arange(self.nmix), len(self.rate_rates))

    @property
    def rates(self):
        return np.tile(self.rate_rates, self.nmix)

    @property
    def props(self):
        return np.repeat(self.weights, len(self.rate_rates)) * np.tile(self.rate_props, self.nmix)

    @property
    def eval(self):
        return np.stack([c.eval for c in self.classes])

    @property
    def evec(self):
        return np.stack([c.evec for c in self.classes])

    @property
    def inv_evec(self):
        return np.stack([c.inv_evec for c in self.classes])

    @property
    def pi(self):
        return np.stack([c.pi for c in self.classes])

    @property
    def tip_lh(self):
        """[STATE_UNKNOWN+1][nmix][n]: class m's eigen-space tip vectors U_m^-1 tipvec."""
        return np.ascontiguousarray(np.stack([c.tip_lh for c in self.classes], axis=1))


def profile_mixture(exch, pis, weights, alpha, ncat_rate=4):
    """Profile mixture (the C10-C60 kind, ModelMixture): shared
    exchangeabilities, one state-frequency profile per class, class weights
    summing to 1, +G on top. Each class's Q is normalised to one substitution
    per unit time under its own profile."""
    n = len(pis[0])
    classes = [SubstModel("class%d" % m, n, normalize_rate_matrix(exch, p), np.asarray(p, np.float64),
                          np.ones(1), np.ones(1)) for m, p in enumerate(pis)]
    rr, rp = gamma_rates_mean(alpha, ncat_rate)
    w = np.asarray(weights, np.float64)
    return MixtureModel("MIX%d+G%d" % (len(pis), ncat_rate), n, classes, w / w.sum(), rr, rp)


def stationary_frequencies(Q):
    """pi with pi Q = 0 and sum(pi) = 1 (the left null vector of Q)."""
    n = Q.shape[0]
    A = np.vstack([Q.T, np.ones(n)])
    rhs = np.zeros(n + 1)
    rhs[-1] = 1.0
    return np.linalg.lstsq(A, rhs, rcond=None)[0]


@dataclass
class NonrevModel:
    """A non-reversible model plus +G categories, in the engine's input form.

    Q is a general rate matrix (rows sum to zero), scaled so that one unit of
    branch length is one expected substitution at stationarity, sum_i pi_i
    (-q_ii) = 1 (the normalisation of ModelMarkov for non-reversible models);
    pi is its stationary distribution. P(t) = Re(V diag(exp(lambda t)) V^-1)
    from the complex eigen system (ModelMarkov::computeTransMatrixNonrev,
    model/modelmarkov.cpp:480-490). Tip vectors stay in the standard basis.
    """

    name: str
    nstates: int
    Q: np.ndarray
    rates: np.ndarray
    props: np.ndarray
    pi: np.ndarray = field(init=False)
    ceval: np.ndarray = field(init=False)
    cevec: np.ndarray = field(init=False)
    cinv_evec: np.ndarray = field(init=False)
    tip_vec: np.ndarray = field(init=False)

    def __post_init__(self):
        self.pi = stationary_frequencies(self.Q)
        self.Q = self.Q / float(-(self.pi * np.diag(self.Q)).sum())
        self.ceval, self.cevec = np.linalg.eig(self.Q)
        self.cinv_evec = np.linalg.inv(self.cevec)
        self.tip_vec = np.ascontiguousarray(tip_vectors(self.nstates))

    @property
    def ncat(self):
        return len(self.rates)

    @property
    def state_unknown(self):
        return STATE_UNKNOWN.get(self.nstates, self.nstates)

    def trans_matrix(self, t):
        """P(t) from the complex eigen system (real part)."""
        return ((self.cevec * np.exp(self.ceval * t)[None, :]) @ self.cinv_evec).real


def unrest_model(nstates, seed, alpha, ncat=4, spread=(0.2, 3.0)):
    """A random general (UNREST-style) rate matrix: every off-diagonal rate
    drawn independently from U(spread), so q_ij != q_ji and the stationary
    distribution is not uniform. Seeded."""
    rng = np.random.default_rng(seed)
    Q = rng.uniform(spread[0], spread[1], (nstates, nstates))
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(axis=1))
    rates, props = gamma_rates_mean(alpha, ncat)
    return NonrevModel("UNREST+G%d" % ncat, nstates, Q, rates, props)
