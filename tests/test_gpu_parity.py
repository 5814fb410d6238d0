"""FP64 GPU path against the CPU oracle and the golden fixtures.

Tolerances: lnL relative error <= 1e-10 (the drop-in contract is 1e-8);
partials relative to each pattern's largest entry <= 1e-10 (eigen-space
values carry cancellation: 61-state codon partials differ from the oracle's
summation order by ~2e-12); scale counts
identical; derivatives relative <= 1e-9; optimised branch lengths within the
Newton-Raphson tolerance (1e-6, the reference's min_branch_length) times 10.
"""
import numpy as np
import pytest

from helpers import load_golden, rel
from iqtree2_gb300 import engine, simulate
import stdbasis
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu

LNL_RTOL = 1e-10
PARTIAL_RTOL = 1e-10


def _gpu_tree(g, safe):
    # kernel-level parity: NORM and SAFE exactly as asked (the reference's
    # automatic SAFE rule is tested on its own below)
    return engine.GpuTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe,
                          flags=engine.FLAG_SAFE_AS_GIVEN)


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
@pytest.mark.parametrize("safe", [False, True])
def test_golden_lnl(oracle_mod, name, safe):
    g = load_golden(name)
    t = _gpu_tree(g, safe)
    lnl, plh = t.compute_likelihood(want_pattern_lh=True)
    assert rel(lnl, g.lnl_std) < LNL_RTOL
    np.testing.assert_allclose(plh, g.pattern_lnl_std, rtol=1e-10, atol=1e-10)
    o = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe)
    assert rel(lnl, o.compute_likelihood()) < LNL_RTOL


def _partials_match(eng, orc, topo, safe):
    """Every directed partial: values (scaled per pattern) and scale counts."""
    for (u, v), s in topo.slot.items():
        gp, gs = eng.partial(s)
        op, os_ = orc.partial(u, v)
        np.testing.assert_array_equal(gs, os_)
        scale = np.maximum(np.abs(op).max(axis=1, keepdims=True), 1e-300)
        assert np.max(np.abs(gp - op) / scale) < PARTIAL_RTOL, (u, v)


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
@pytest.mark.parametrize("safe", [False, True])
def test_kernel_level_partials(oracle_mod, name, safe):
    g = load_golden(name)
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    eng = engine.Engine(g.patterns.shape[1], g.model.nstates, g.model.ncat, g.ntaxa, g.model.state_unknown,
                        topo.nslots, safe=safe, max_ops=topo.nslots,
                        flags=engine.FLAG_SAFE_AS_GIVEN)
    eng.set_model(g.model)
    eng.set_patterns(g.freq)
    eng.set_tip_states(g.patterns)
    done, ops = set(), []
    for (u, v) in sorted(topo.slot):
        ops += topo.ops_for(u, v, done)
    eng.compute_partials(ops)
    orc = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe)
    _partials_match(eng, orc, topo, safe)
    # branch lnL at an internal-internal branch and at a tip branch, through the kernel pointer
    for (u, v) in [e for e in map(tuple, g.edges) if min(e) >= g.ntaxa][:1] + [tuple(g.edges[0])]:
        u, v = int(u), int(v)
        node, dad = (v, u) if v >= g.ntaxa else (u, v)
        lg = eng.branch_lnl(topo.ref(dad, node), topo.ref(node, dad), topo.edge_len(node, dad))
        lo = orc.lnl_branch(node, dad)
        assert rel(lg, lo) < LNL_RTOL


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
@pytest.mark.parametrize("safe", [False, True])
def test_derivatives_and_from_buffer(oracle_mod, name, safe):
    g = load_golden(name)
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    eng = engine.Engine(g.patterns.shape[1], g.model.nstates, g.model.ncat, g.ntaxa, g.model.state_unknown,
                        topo.nslots, safe=safe, max_ops=topo.nslots,
                        flags=engine.FLAG_SAFE_AS_GIVEN)
    eng.set_model(g.model)
    eng.set_patterns(g.freq)
    eng.set_tip_states(g.patterns)
    internal = [tuple(map(int, e)) for e in g.edges if min(e) >= g.ntaxa]
    branches = [tuple(map(int, g.edges[0]))] + internal[:2]
    done = set()
    for (n1, n2) in branches:
        # a fresh oracle per branch: its derivative hook moves that branch's length
        orc = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe)
        node, dad = n2, n1
        if node < g.ntaxa:
            node, dad = n1, n2
        ops = topo.ops_for(dad, node, done) + topo.ops_for(node, dad, done)
        a, b = topo.ref(dad, node), topo.ref(node, dad)
        first = True
        for length in (0.02, 0.1, 0.7):
            df, ddf = eng.likelihood_derv(ops if first else [], a, b, length, theta_computed=not first)
            first = False
            odf, oddf = orc.derv(n1, n2, length)
            assert abs(df - odf) <= 1e-9 * max(1.0, abs(odf))
            assert abs(ddf - oddf) <= 1e-9 * max(1.0, abs(oddf))
            lb = eng.lnl_from_buffer(length)
            assert rel(lb, orc.lnl_branch(node, dad)) < LNL_RTOL


@pytest.mark.parametrize("name", ["dna16", "prot12"])
@pytest.mark.parametrize("safe", [False, True])
def test_optimize_all_branches(oracle_mod, name, safe):
    g = load_golden(name)
    t = _gpu_tree(g, safe)
    o = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe)
    lg = t.optimize_all_branches()
    lo = o.optimize_all_branches()
    assert rel(lg, lo) < 1e-9
    np.testing.assert_allclose(t.lengths(), o.lengths(), atol=1e-5)
    # the tree lnL after optimisation, recomputed from scratch, agrees too
    assert rel(t.compute_likelihood(), o.compute_likelihood()) < 1e-9


@pytest.mark.parametrize("safe", [False, True])
def test_scaling_counts_identical(oracle_mod, safe):
    """Long-branch 150-taxon protein and 300-taxon DNA trees underflow 2^-256."""
    for ds in (simulate.protein_lg_dataset(150, 300, 11, mean_bl=0.5),
               simulate.dna_gtr_dataset(300, 200, 5, mean_bl=0.5)):
        topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
        eng = engine.Engine(ds.nptn, ds.model.nstates, ds.model.ncat, ds.ntaxa, ds.model.state_unknown,
                            topo.nslots, safe=safe, max_ops=topo.nslots,
                        flags=engine.FLAG_SAFE_AS_GIVEN)
        eng.set_model(ds.model)
        eng.set_patterns(ds.freq)
        eng.set_tip_states(ds.patterns)
        root_nb = topo.adj[0][0][0]
        ops = topo.branch_ops(root_nb, 0)
        lg = eng.compute_likelihood(ops, topo.ref(0, root_nb), topo.ref(root_nb, 0), topo.edge_len(0, root_nb))
        orc = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, safe=safe)
        _, s_or = orc.partial(0, root_nb)
        assert s_or.max() >= 1  # the case really scales
        _, s_gpu = eng.partial(topo.ref(0, root_nb))
        np.testing.assert_array_equal(s_gpu, s_or)
        assert rel(lg, orc.lnl_branch(root_nb, 0)) < LNL_RTOL


def test_ambiguous_and_unknown_states(oracle_mod):
    rng = np.random.default_rng(5)
    for ds in (simulate.dna_gtr_dataset(12, 400, 21), simulate.protein_lg_dataset(10, 200, 22)):
        pats = ds.patterns.copy()
        su = ds.model.state_unknown
        mask = rng.random(pats.shape) < 0.15
        pats[mask] = rng.integers(ds.model.nstates, su + 1, size=mask.sum())
        for safe in (False, True):
            t = engine.GpuTree(ds.model, pats, ds.freq, ds.edges, ds.lengths, safe=safe)
            o = oracle_mod.OracleTree(ds.model, pats, ds.freq, ds.edges, ds.lengths, safe=safe)
            lg = t.compute_likelihood()
            assert rel(lg, o.compute_likelihood()) < LNL_RTOL
            ref, _ = stdbasis.tree_lnl(ds.model, pats, ds.freq, ds.edges, ds.lengths, ds.ntaxa)
            assert rel(lg, ref) < 1e-10


@pytest.mark.parametrize("nptn", [1, 127, 128, 129, 1000])
def test_ragged_pattern_counts(oracle_mod, nptn):
    ds = simulate.dna_gtr_dataset(9, 3000, 31)
    pats, freq = ds.patterns[:, :nptn], ds.freq[:nptn]
    t = engine.GpuTree(ds.model, pats, freq, ds.edges, ds.lengths)
    o = oracle_mod.OracleTree(ds.model, pats, freq, ds.edges, ds.lengths)
    assert rel(t.compute_likelihood(), o.compute_likelihood()) < LNL_RTOL


def test_single_category_and_three_taxa(oracle_mod):
    from helpers import jc_model, GOLDEN
    d = np.load(f"{GOLDEN}/kat_jc.npz")
    m = jc_model(1, 1.0)
    t = engine.GpuTree(m, d["patterns"], d["freq"], d["edges"], d["lengths"])
    assert rel(t.compute_likelihood(), float(d["lnl_g1"])) < 1e-12
    t.optimize_all_branches(tolerance=1e-9)
    L = t.lengths()
    assert abs((L[0] + L[1]) - float(d["ml_distance_g1"])) < 1e-5


def test_config_protein_full_size(oracle_mod):
    """Protein LG+G4, 100 taxa x 50,000 sites: the FP64 GPU lnL against the oracle."""
    ds = simulate.protein_lg_dataset(100, 50000, 2)
    t = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
    o = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
    lg, plg = t.compute_likelihood(want_pattern_lh=True)
    lo, plo = o.compute_likelihood(want_pattern_lh=True)
    assert rel(lg, lo) < LNL_RTOL
    np.testing.assert_allclose(plg, plo, rtol=1e-11, atol=1e-9)


def test_engine_errors_are_reported():
    g = load_golden("dna16")
    eng = engine.Engine(g.patterns.shape[1], 4, 4, g.ntaxa, 18, 4, max_ops=4)
    with pytest.raises(engine.EngineError) as ei:
        eng.branch_lnl(0, -1, 0.1)  # nothing uploaded yet
    assert ei.value.code == 6
    eng.set_model(g.model)
    eng.set_patterns(g.freq)
    eng.set_tip_states(g.patterns)
    with pytest.raises(engine.EngineError) as ei:
        eng.compute_partials([(0, 9, -1, 0.1, 0.1)])  # slot 9 out of range
    assert ei.value.code == 1
    with pytest.raises(engine.EngineError) as ei:
        eng.lnl_from_buffer(0.1)  # no theta yet
    assert ei.value.code == 6


def test_reference_triple_tail_flag(oracle_mod):
    """IQGPU_FLAG_REF_TRIPLE_TAIL reproduces the reference's codon derivative sum."""
    g = load_golden("codon8")
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    n1, n2 = map(int, g.edges[0])
    node, dad = (n2, n1) if n2 >= g.ntaxa else (n1, n2)
    for flag, quirk in ((0, False), (engine.FLAG_REF_TRIPLE_TAIL, True)):
        eng = engine.Engine(g.patterns.shape[1], 61, g.model.ncat, g.ntaxa, 61, topo.nslots,
                            max_ops=topo.nslots, flags=flag)
        eng.set_model(g.model)
        eng.set_patterns(g.freq)
        eng.set_tip_states(g.patterns)
        ops = topo.branch_ops(node, dad)
        df, ddf = eng.likelihood_derv(ops, topo.ref(dad, node), topo.ref(node, dad), 0.02)
        orc = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths, ref_triple_tail=quirk)
        odf, oddf = orc.derv(n1, n2, 0.02)
        assert abs(df - odf) <= 1e-9 * max(1.0, abs(odf))
        assert abs(ddf - oddf) <= 1e-9 * max(1.0, abs(oddf))


def test_reference_safe_rule():
    """The engine picks SAFE as PhyloTree::setLikelihoodKernel does
    (tree/phylotreesse.cpp:95-96): always for state counts other than 4 and
    20 (codon), from 2000 taxa on, and when asked; NORM otherwise. The flag
    IQGPU_FLAG_SAFE_AS_GIVEN keeps the caller's choice."""
    g = load_golden("codon8")
    t = engine.GpuTree(g.model, g.patterns, g.freq, g.edges, g.lengths)
    assert t.engine.safe
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    _, s = t.engine.partial(0)
    assert s.shape == (g.patterns.shape[1], g.model.ncat)  # one count per pattern x category
    e = engine.Engine(g.patterns.shape[1], 61, 4, g.ntaxa, 61, topo.nslots, flags=engine.FLAG_SAFE_AS_GIVEN)
    assert not e.safe
    for n, ntaxa, want in ((4, 16, False), (20, 16, False), (20, 16, True), (4, 2000, True), (20, 2500, True),
                           (2, 16, True)):
        asked = want and ntaxa < 2000 and n in (4, 20)
        e = engine.Engine(64, n, 4, ntaxa, n if n > 4 else 18, 4, safe=asked, max_ops=4)
        assert e.safe == want, (n, ntaxa)
