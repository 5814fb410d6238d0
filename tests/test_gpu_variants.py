"""Rate-heterogeneity variants on every path against the FP64 oracle.

+I+G4: a per-pattern invariant-site term (``ptn_invar``, built as the
reference's computePtnInvar does) added to each pattern's likelihood, and in
the FP64 path no 2^-256 rescaling of a pattern that carries one. +R4
(FreeRate): unequal category weights and rates.

Tolerances, as for each path: FP64 lnL <= 1e-10 relative and scale counts
identical; FP32 mixed and split-TF32 lnL <= 1e-6 relative; first and second
derivatives relative 1e-9 (FP64) or 1e-4 / 1e-3 (mixed) with, on the mixed
paths, an absolute floor of 1e-5 per site: each pattern's FP32 ratio carries
~1e-6 of its own size, and those errors add over patterns even where the sum
itself cancels (near the optimum the derivative is a few units over
thousands of sites).
"""
import dataclasses

import numpy as np
import pytest

from helpers import rel
from iqtree2_gb300 import engine, models, simulate
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu

P_INVAR = 0.3


def _variant(ds, kind):
    m = ds.model
    if kind == "+I+G4":
        r, p = models.gamma_invar_rates(0.5, P_INVAR, 4)
        inv = models.invariant_site_lh(ds.patterns, m.pi, P_INVAR, m.nstates)
    else:  # +R4
        r, p = models.free_rates([0.05, 0.4, 1.2, 3.5], [0.2, 0.3, 0.35, 0.15])
        inv = None
    return dataclasses.replace(m, rates=r, props=p), inv


def _dataset(data):
    return (simulate.dna_gtr_dataset(24, 2000, 61) if data == "dna"
            else simulate.protein_lg_dataset(16, 800, 62))


@pytest.mark.parametrize("kind", ["+I+G4", "+R4"])
@pytest.mark.parametrize("data,precision", [("dna", engine.F64), ("dna", engine.F32), ("protein", engine.F64),
                                            ("protein", engine.F32), ("protein", engine.TF32X3)])
def test_variant_lnl_and_derivatives(oracle_mod, kind, data, precision):
    ds = _dataset(data)
    m, inv = _variant(ds, kind)
    if inv is not None:
        assert (inv > 0).sum() > 0  # constant patterns carry the +I term
    tol = 1e-10 if precision == engine.F64 else 1e-6
    t = engine.GpuTree(m, ds.patterns, ds.freq, ds.edges, ds.lengths, precision=precision, invar=inv)
    o = oracle_mod.OracleTree(m, ds.patterns, ds.freq, ds.edges, ds.lengths, invar=inv)
    lg, plh = t.compute_likelihood(want_pattern_lh=True)
    lo, plo = o.compute_likelihood(want_pattern_lh=True)
    assert rel(lg, lo) < tol, (lg, lo)
    np.testing.assert_allclose(plh, plo, atol=1e-8 if precision == engine.F64 else 1e-4)

    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    eng = engine.Engine(ds.nptn, m.nstates, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots, precision=precision,
                        max_ops=topo.nslots)
    eng.set_model(m)
    eng.set_patterns(ds.freq, inv)
    eng.set_tip_states(ds.patterns)
    internal = [tuple(map(int, e)) for e in ds.edges if min(e) >= ds.ntaxa]
    done = set()
    for (n1, n2) in [tuple(map(int, ds.edges[0]))] + internal[:2]:
        node, dad = (n2, n1) if n2 >= ds.ntaxa else (n1, n2)
        ops = topo.ops_for(dad, node, done) + topo.ops_for(node, dad, done)
        a, b = topo.ref(dad, node), topo.ref(node, dad)
        o = oracle_mod.OracleTree(m, ds.patterns, ds.freq, ds.edges, ds.lengths, invar=inv)  # derv moves the branch
        for i, length in enumerate((0.03, 0.4)):
            df, ddf = eng.likelihood_derv(ops if i == 0 else [], a, b, length, theta_computed=i > 0)
            odf, oddf = o.derv(n1, n2, length)
            if precision == engine.F64:
                assert abs(df - odf) <= 1e-9 * abs(odf) + 1e-9
                assert abs(ddf - oddf) <= 1e-9 * abs(oddf) + 1e-9
            else:
                floor = 1e-5 * float(ds.freq.sum())
                assert abs(df - odf) <= 1e-4 * abs(odf) + floor, (df, odf)
                assert abs(ddf - oddf) <= 1e-3 * abs(oddf) + floor, (ddf, oddf)


@pytest.mark.parametrize("safe", [False, True])
def test_invar_scaling_counts_identical(oracle_mod, safe):
    """300-taxon long-branch DNA under +I+G4: patterns underflow 2^-256, and a
    pattern with an invariant-site term is never rescaled (the reference's
    condition lh_max < 2^-256 && ptn_invar == 0)."""
    ds = simulate.dna_gtr_dataset(300, 300, 5, mean_bl=0.5)
    m, inv = _variant(ds, "+I+G4")
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    eng = engine.Engine(ds.nptn, m.nstates, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots, safe=safe,
                        max_ops=topo.nslots)
    eng.set_model(m)
    eng.set_patterns(ds.freq, inv)
    eng.set_tip_states(ds.patterns)
    nb = topo.adj[0][0][0]
    ops = topo.branch_ops(nb, 0)
    lg = eng.compute_likelihood(ops, topo.ref(0, nb), topo.ref(nb, 0), topo.edge_len(0, nb))
    orc = oracle_mod.OracleTree(m, ds.patterns, ds.freq, ds.edges, ds.lengths, safe=safe, invar=inv)
    _, s_or = orc.partial(0, nb)
    assert s_or.max() >= 1
    _, s_gpu = eng.partial(topo.ref(0, nb))
    np.testing.assert_array_equal(s_gpu, s_or)
    assert rel(lg, orc.lnl_branch(nb, 0)) < 1e-10


def test_invar_optimize_all_branches(oracle_mod):
    ds = _dataset("dna")
    m, inv = _variant(ds, "+I+G4")
    t = engine.GpuTree(m, ds.patterns, ds.freq, ds.edges, ds.lengths, invar=inv)
    o = oracle_mod.OracleTree(m, ds.patterns, ds.freq, ds.edges, ds.lengths, invar=inv)
    lg, lo = t.optimize_all_branches(), o.optimize_all_branches()
    assert rel(lg, lo) < 1e-10
    np.testing.assert_allclose(t.lengths(), o.lengths(), atol=1e-5)


@pytest.mark.parametrize("data,precision", [("dna", engine.F64), ("dna", engine.F32), ("protein", engine.F64),
                                            ("protein", engine.TF32X3)])
def test_asc_lewis(oracle_mod, data, precision):
    """+ASC (Lewis) on variable-site data: the unobserved constant patterns
    appended with weight 0; lnL, the observed patterns' lnL, derivatives
    (FP64 1e-9, mixed with the floor above) and optimised branch lengths
    against the oracle's restatement."""
    ds = _dataset(data)
    n = ds.model.nstates
    vp, vf = models.variable_patterns(ds.patterns, ds.freq, n)
    pats, freq, nconst, nsite = models.asc_lewis_patterns(vp, vf, n, ds.model.pi)
    assert nconst > 0
    m = ds.model
    tol = 1e-10 if precision == engine.F64 else 1e-6
    t = engine.GpuTree(m, pats, freq, ds.edges, ds.lengths, precision=precision, asc=(nconst, nsite))
    o = oracle_mod.OracleTree(m, pats, freq, ds.edges, ds.lengths, asc=(nconst, nsite))
    lg, plh = t.compute_likelihood(want_pattern_lh=True)
    lo, plo = o.compute_likelihood(want_pattern_lh=True)
    plain = oracle_mod.OracleTree(m, pats, freq, ds.edges, ds.lengths).compute_likelihood()
    assert abs(lo - plain) > 1.0  # the correction is not negligible here
    assert rel(lg, lo) < tol, (lg, lo)
    nobs = pats.shape[1] - nconst
    np.testing.assert_allclose(plh[:nobs], plo[:nobs], atol=1e-8 if precision == engine.F64 else 1e-4)

    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    eng = engine.Engine(pats.shape[1], n, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots, precision=precision,
                        max_ops=topo.nslots)
    eng.set_model(m)
    eng.set_patterns(freq)
    eng.set_tip_states(pats)
    eng.set_asc(nconst, nsite)
    internal = [tuple(map(int, e)) for e in ds.edges if min(e) >= ds.ntaxa]
    done = set()
    for (n1, n2) in internal[:2]:
        ops = topo.ops_for(n1, n2, done) + topo.ops_for(n2, n1, done)
        a, b = topo.ref(n1, n2), topo.ref(n2, n1)
        oo = oracle_mod.OracleTree(m, pats, freq, ds.edges, ds.lengths, asc=(nconst, nsite))
        for i, length in enumerate((0.03, 0.4)):
            df, ddf = eng.likelihood_derv(ops if i == 0 else [], a, b, length, theta_computed=i > 0)
            odf, oddf = oo.derv(n1, n2, length)
            if precision == engine.F64:
                assert abs(df - odf) <= 1e-9 * abs(odf) + 1e-9, (df, odf)
                assert abs(ddf - oddf) <= 1e-9 * abs(oddf) + 1e-9, (ddf, oddf)
            else:
                floor = 1e-5 * float(freq.sum())
                assert abs(df - odf) <= 1e-4 * abs(odf) + floor, (df, odf)
                assert abs(ddf - oddf) <= 1e-3 * abs(oddf) + floor, (ddf, oddf)
            assert rel(eng.lnl_from_buffer(length), oo.lnl_branch(n2, n1)) < tol
    if precision == engine.F64 and data == "dna":
        lg2, lo2 = t.optimize_all_branches(), o.optimize_all_branches()
        assert rel(lg2, lo2) < 1e-10
        np.testing.assert_allclose(t.lengths(), o.lengths(), atol=1e-5)


def test_asc_refused_by_batched_paths():
    ds = _dataset("dna")
    vp, vf = models.variable_patterns(ds.patterns, ds.freq, 4)
    pats, freq, nconst, nsite = models.asc_lewis_patterns(vp, vf, 4, ds.model.pi)
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    eng = engine.Engine(pats.shape[1], 4, ds.model.ncat, ds.ntaxa, ds.model.state_unknown, topo.nslots,
                        precision=engine.F32, max_ops=topo.nslots)
    eng.set_model(ds.model)
    eng.set_patterns(freq)
    eng.set_tip_states(pats)
    eng.set_asc(nconst, nsite)
    with pytest.raises(engine.EngineError):
        engine.Group([eng])
    with pytest.raises(engine.EngineError):
        eng.set_asc(eng.nptn, nsite)  # no observed pattern left


def _mixture(data, nclass, ncat_rate, seed):
    rng = np.random.default_rng(seed)
    if data == "dna":
        ds = simulate.dna_gtr_dataset(20, 1500, 63)
        R = rng.uniform(0.5, 3.0, size=(4, 4))
        R = (R + R.T) / 2
        n = 4
    else:
        ds = simulate.protein_lg_dataset(16, 800, 64)
        R, _ = models.lg_exchangeabilities()
        n = 20
    pis = [rng.dirichlet(np.full(n, 3.0)) for _ in range(nclass)]
    w = rng.uniform(0.5, 1.5, size=nclass)
    return ds, models.profile_mixture(R, pis, w, 0.6, ncat_rate)


@pytest.mark.parametrize("data,precision,nclass,ncat_rate,safe", [
    ("dna", engine.F32, 2, 2, False), ("dna", engine.F32, 3, 2, False), ("protein", engine.F32, 3, 2, False),
    ("protein", engine.TF32X3, 3, 2, False), ("protein", engine.TF32X3, 4, 1, False),
    ("dna", engine.F64, 3, 2, False), ("protein", engine.F64, 3, 2, False), ("protein", engine.F64, 4, 1, True)])
def test_mixture_lnl_and_derivatives(data, precision, nclass, ncat_rate, safe):
    """Profile mixtures on every path (4-state kernels for 2 x 2
    categories, the generic CUDA-core and tensor-core kernels otherwise, one
    fused mix-rate case; FP64 with each category in its class's eigen basis,
    NORM and SAFE): lnL and pattern lnL against the independent numpy mixture
    pruning (1e-10 relative for FP64, 1e-6 mixed), the derivatives against
    its central differences, the lnL from the theta buffer against it."""
    import stdbasis
    ds, mix = _mixture(data, nclass, ncat_rate, 70 + nclass)
    want, pwant = stdbasis.tree_lnl_mixture(mix, ds.patterns, ds.freq, ds.edges, ds.lengths, ds.ntaxa)
    f64 = precision == engine.F64
    tol = 1e-10 if f64 else 1e-6
    t = engine.GpuTree(mix, ds.patterns, ds.freq, ds.edges, ds.lengths, precision=precision, safe=safe)
    lg, plh = t.compute_likelihood(want_pattern_lh=True)
    assert rel(lg, want) < tol, (lg, want)
    np.testing.assert_allclose(plh, pwant, atol=1e-8 if f64 else 1e-4)

    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    eng = engine.Engine(ds.nptn, mix.nstates, mix.ncat, ds.ntaxa, mix.state_unknown, topo.nslots, precision=precision,
                        max_ops=topo.nslots, safe=safe)
    eng.set_model(mix)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    k = next(i for i, e in enumerate(ds.edges) if min(e) >= ds.ntaxa)
    n1, n2 = map(int, ds.edges[k])
    ops = topo.ops_for(n1, n2, set()) + topo.ops_for(n2, n1, set())
    a, b = topo.ref(n1, n2), topo.ref(n2, n1)

    def lnl_at(x):
        lens = ds.lengths.copy()
        lens[k] = x
        return stdbasis.tree_lnl_mixture(mix, ds.patterns, ds.freq, ds.edges, lens, ds.ntaxa)[0]
    h = 1e-5
    for i, x in enumerate((0.05, 0.3)):
        df, ddf = eng.likelihood_derv(ops if i == 0 else [], a, b, x, theta_computed=i > 0)
        l0, lp, lm = lnl_at(x), lnl_at(x + h), lnl_at(x - h)
        fd1, fd2 = (lp - lm) / (2 * h), (lp - 2 * l0 + lm) / h ** 2
        floor = 1e-5 * float(ds.freq.sum())
        assert abs(df - fd1) <= 1e-4 * abs(fd1) + floor, (df, fd1)
        assert abs(ddf - fd2) <= 1e-2 * abs(fd2) + floor, (ddf, fd2)
        assert rel(eng.lnl_from_buffer(x), l0) < tol


@pytest.mark.parametrize("precision", [engine.F64, engine.TF32X3])
def test_tip_states_out_of_range_rejected(precision):
    """A tip state above STATE_UNKNOWN is an argument error (the range check
    runs on the uploaded copy); the engine then refuses to compute until valid
    states are set, and valid states give the same lnL as before."""
    ds = simulate.protein_lg_dataset(12, 600, 63)
    t = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, precision=precision)
    l0 = t.compute_likelihood()
    bad = ds.patterns.copy()
    bad[5, bad.shape[1] - 1] = ds.model.state_unknown + 1
    with pytest.raises(engine.EngineError, match="STATE_UNKNOWN"):
        t.engine.set_tip_states(bad)
    with pytest.raises(engine.EngineError):
        t.compute_likelihood()
    t.engine.set_tip_states(ds.patterns)
    assert rel(t.compute_likelihood(), l0) < 1e-12
