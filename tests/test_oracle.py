"""The CPU oracle against closed forms and an independent standard-basis pruning."""
import numpy as np
import pytest

from helpers import GOLDEN, jc_model, load_golden, rel
import stdbasis


@pytest.mark.parametrize("tag,alpha,ncat", [("g1", 1.0, 1), ("g4", 0.5, 4)])
@pytest.mark.parametrize("safe", [False, True])
def test_jc_pair_closed_form(oracle_mod, tag, alpha, ncat, safe):
    d = np.load(f"{GOLDEN}/kat_jc.npz")
    m = jc_model(ncat, alpha)
    np.testing.assert_allclose(m.rates, d[f"rates_{tag}"], rtol=1e-12)
    t = oracle_mod.OracleTree(m, d["patterns"], d["freq"], d["edges"], d["lengths"], safe=safe)
    assert rel(t.compute_likelihood(), float(d[f"lnl_{tag}"])) < 1e-12


def test_jc_ml_distance(oracle_mod):
    d = np.load(f"{GOLDEN}/kat_jc.npz")
    m = jc_model(1, 1.0)
    t = oracle_mod.OracleTree(m, d["patterns"], d["freq"], d["edges"], d["lengths"])
    t.optimize_all_branches(tolerance=1e-9)
    L = t.lengths()
    assert abs((L[0] + L[1]) - float(d["ml_distance_g1"])) < 1e-5


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
@pytest.mark.parametrize("safe", [False, True])
def test_golden_standard_basis(oracle_mod, name, safe):
    g = load_golden(name)
    t = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe)
    lnl, plh = t.compute_likelihood(want_pattern_lh=True)
    assert rel(lnl, g.lnl_std) < 1e-12
    np.testing.assert_allclose(plh, g.pattern_lnl_std, rtol=1e-11, atol=1e-11)


def test_stationarity_rows_sum_to_one():
    g = load_golden("prot12")
    m = g.model
    for t in (0.0, 0.01, 0.3, 5.0):
        P = (m.evec * np.exp(m.eval * t)[None, :]) @ m.inv_evec
        np.testing.assert_allclose(P.sum(axis=1), 1.0, atol=1e-12)


def test_zero_length_star_tree(oracle_mod):
    """All branches at length 0: every taxon shares one state, so
    lnL = sum_ptn freq * log(pi[state])."""
    m = jc_model(4, 0.5)
    pi = np.array([0.1, 0.2, 0.3, 0.4])
    from iqtree2_gb300 import models
    m = models.gtr_model(np.array([1.0, 2.0, 0.5, 1.5, 3.0, 1.0]), pi, 0.5)
    ntaxa = 5
    from iqtree2_gb300 import simulate
    edges, _ = simulate.yule_tree(ntaxa, 0.1, np.random.default_rng(3))
    pats = np.repeat(np.arange(4, dtype=np.uint8)[None, :], ntaxa, axis=0)
    freq = np.array([3.0, 5.0, 7.0, 11.0])
    t = oracle_mod.OracleTree(m, pats, freq, edges, np.zeros(len(edges)))
    assert rel(t.compute_likelihood(), float(np.sum(freq * np.log(pi)))) < 1e-12


def test_scaling_triggers_and_matches_standard_basis(oracle_mod):
    """A 150-taxon protein tree with long branches underflows 2^-256: scale
    counts must appear and the scaled lnL must still equal the standard-basis
    value."""
    from iqtree2_gb300 import simulate
    ds = simulate.protein_lg_dataset(150, 40, 11, mean_bl=0.5)
    for safe in (False, True):
        t = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, safe=safe)
        lnl = t.compute_likelihood()
        ref, _ = stdbasis.tree_lnl(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, ds.ntaxa)
        assert rel(lnl, ref) < 1e-11
    # the root-adjacent partial carries a non-zero scale count somewhere
    t = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
    adj = {}
    for (u, v) in ds.edges:
        adj.setdefault(int(u), []).append(int(v))
        adj.setdefault(int(v), []).append(int(u))
    x = adj[0][0]
    _, s = t.partial(0, x)
    assert s.max() >= 1


def test_exact_derivative_matches_finite_difference_and_reference_quirk(oracle_mod):
    """Codon +G4 (odd nstates, even block): the exact derivative sum equals the
    finite difference of lnL; the reference's dotProductTriple tail (the last
    block entry added twice) gives a different value, reproduced on request."""
    g = load_golden("codon8")
    n1, n2 = map(int, g.edges[0])
    node, dad = (n2, n1) if n2 >= g.ntaxa else (n1, n2)
    exact = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths)
    quirk = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths, ref_triple_tail=True)
    h, L = 1e-6, 0.02

    def lnl(t, x):
        t.derv(n1, n2, x)
        return t.lnl_branch(node, dad)

    fd = (lnl(exact, L + h) - lnl(exact, L - h)) / (2 * h)
    df, _ = exact.derv(n1, n2, L)
    assert abs(df - fd) < 1e-4 * abs(fd)
    dq, _ = quirk.derv(n1, n2, L)
    assert abs(dq - fd) > 1.0  # the reference's sum is off for this model
    # DNA (even nstates) is unaffected by the flag
    d = load_golden("dna16")
    a = oracle_mod.OracleTree(d.model, d.patterns, d.freq, d.edges, d.lengths).derv(*map(int, d.edges[0]), 0.05)
    b = oracle_mod.OracleTree(d.model, d.patterns, d.freq, d.edges, d.lengths,
                              ref_triple_tail=True).derv(*map(int, d.edges[0]), 0.05)
    assert a == b


def test_invariant_site_terms():
    """+I term per pattern (computePtnInvar): constant state s -> p*pi[s];
    all unknown -> p; a DNA ambiguity shared by every taxon -> p * sum of its
    states; a variable pattern -> 0."""
    from iqtree2_gb300 import models
    pi = np.array([0.1, 0.2, 0.3, 0.4])
    su = models.STATE_UNKNOWN[4]
    R = 5 + 3  # DNA code of the mask A|G (bits 0 and 2): state = mask + 3
    pats = np.array([[2, su, 0, 2, R],
                     [2, su, 1, su, 0],
                     [2, su, 0, 2, 2]], dtype=np.uint8)
    got = models.invariant_site_lh(pats, pi, 0.25, 4)
    np.testing.assert_allclose(got, [0.25 * 0.3, 0.25, 0.0, 0.25 * 0.3, 0.0])
    pats2 = np.array([[R], [R], [su]], dtype=np.uint8)
    np.testing.assert_allclose(models.invariant_site_lh(pats2, pi, 0.25, 4), [0.25 * (0.1 + 0.3)])


@pytest.mark.parametrize("kind", ["+I+G4", "+R4"])
def test_rate_variants_match_standard_basis(oracle_mod, kind):
    """Oracle under +I+G4 and +R4 against the independent numpy pruning."""
    import dataclasses
    from iqtree2_gb300 import models, simulate
    ds = simulate.dna_gtr_dataset(10, 300, 71)
    if kind == "+I+G4":
        r, p = models.gamma_invar_rates(0.7, 0.2, 4)
        inv = models.invariant_site_lh(ds.patterns, ds.model.pi, 0.2, 4)
        np.testing.assert_allclose(p.sum(), 0.8)
        np.testing.assert_allclose(p @ r, 1.0)  # variable sites carry the whole mean rate
    else:
        r, p = models.free_rates([0.1, 0.5, 1.5, 4.0], [1, 2, 2, 1])
        inv = None
        np.testing.assert_allclose(p @ r, 1.0)
    m = dataclasses.replace(ds.model, rates=r, props=p)
    o = oracle_mod.OracleTree(m, ds.patterns, ds.freq, ds.edges, ds.lengths, invar=inv)
    want, _ = stdbasis.tree_lnl(m, ds.patterns, ds.freq, ds.edges, ds.lengths, ds.ntaxa, invar=inv)
    assert rel(o.compute_likelihood(), want) < 1e-12


def test_asc_lewis_matches_standard_basis_and_finite_differences(oracle_mod):
    """+ASC (Lewis) in the oracle: the corrected lnL equals the independent
    numpy pruning's sum over observed patterns minus nsite*log(1 - sum of the
    constant patterns' likelihoods); the corrected derivative matches central
    finite differences of the corrected lnL."""
    from iqtree2_gb300 import models, simulate
    ds = simulate.dna_gtr_dataset(8, 400, 81)
    vp, vf = models.variable_patterns(ds.patterns, ds.freq, 4)
    pats, freq, nconst, nsite = models.asc_lewis_patterns(vp, vf, 4, ds.model.pi)
    assert nconst == 4 and nsite == vf.sum()
    o = oracle_mod.OracleTree(ds.model, pats, freq, ds.edges, ds.lengths, asc=(nconst, nsite))
    got, plh = o.compute_likelihood(want_pattern_lh=True)
    _, p_std = stdbasis.tree_lnl(ds.model, pats, freq, ds.edges, ds.lengths, ds.ntaxa)
    nobs = pats.shape[1] - nconst
    pc = np.exp(p_std[nobs:]).sum()
    want = float(p_std[:nobs] @ freq[:nobs]) - nsite * np.log(1.0 - pc)
    assert rel(got, want) < 1e-12
    np.testing.assert_allclose(plh[:nobs], p_std[:nobs] - np.log(1.0 - pc), rtol=1e-12, atol=1e-12)
    # derivative of the corrected lnL along one internal branch
    k = next(i for i, e in enumerate(ds.edges) if min(e) >= ds.ntaxa)
    n1, n2 = map(int, ds.edges[k])
    t0 = float(ds.lengths[k])
    df, ddf = oracle_mod.OracleTree(ds.model, pats, freq, ds.edges, ds.lengths, asc=(nconst, nsite)).derv(n1, n2, t0)

    def lnl(t):
        lens = ds.lengths.copy()
        lens[k] = t
        return oracle_mod.OracleTree(ds.model, pats, freq, ds.edges, lens, asc=(nconst, nsite)).compute_likelihood()
    h = 1e-5
    assert abs(df - (lnl(t0 + h) - lnl(t0 - h)) / (2 * h)) < 1e-5 * max(1.0, abs(df))
    assert abs(ddf - (lnl(t0 + h) - 2 * lnl(t0) + lnl(t0 - h)) / h ** 2) < 1e-3 * max(1.0, abs(ddf))


def test_mixture_reference_one_class_and_root_invariance():
    """The numpy mixture pruning the mixture GPU tests compare with: one class
    equals the plain-model pruning; the lnL does not depend on the root."""
    from iqtree2_gb300 import models, simulate
    ds = simulate.dna_gtr_dataset(9, 300, 77)
    m = ds.model
    R = np.ones((4, 4))
    one = models.profile_mixture(R, [m.pi], [1.0], 0.8, 4)
    plain = models.SubstModel("x", 4, one.classes[0].Q, m.pi, one.rates, one.props)
    a, _ = stdbasis.tree_lnl_mixture(one, ds.patterns, ds.freq, ds.edges, ds.lengths, ds.ntaxa)
    b, _ = stdbasis.tree_lnl(plain, ds.patterns, ds.freq, ds.edges, ds.lengths, ds.ntaxa)
    assert rel(a, b) < 1e-12
    rng = np.random.default_rng(3)
    mix = models.profile_mixture(R, [rng.dirichlet(np.ones(4) * 2) for _ in range(3)], [0.2, 0.5, 0.3], 0.5, 2)
    l1, _ = stdbasis.tree_lnl_mixture(mix, ds.patterns, ds.freq, ds.edges, ds.lengths, ds.ntaxa)
    l2, _ = stdbasis.tree_lnl_mixture(mix, ds.patterns, ds.freq, ds.edges, ds.lengths, ds.ntaxa, root=ds.ntaxa + 3)
    assert rel(l1, l2) < 1e-10
