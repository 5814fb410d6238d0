"""Multifurcating nodes on the FP64 drop-in (tree/phylokernelnew.h:1407-1631).

Trees with contracted internal edges (nodes of degree 4, 5, 6): every
partial within 1e-10 of each pattern's largest entry and scale counts
identical to the oracle (itself bit-exact with the reference's compiled
multifurcating kernel), NORM and SAFE, including a 150-taxon case whose
partials underflow 2^-256; branch lnL 1e-10 relative, derivatives 1e-9,
the tree drivers (iqgpu_tree_create_n) within the Newton-Raphson tolerance;
the mixed-precision paths (FP32 and split TF32 engines, whose multifurcating
records run on the fused CUDA-core kernel) within their tolerances.
"""
import numpy as np
import pytest

from helpers import load_golden, rel
from iqtree2_gb300 import engine, simulate, topology
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu


def _collapsed(g, pick):
    internal = [k for k, (u, v) in enumerate(g.edges) if min(int(u), int(v)) >= g.ntaxa]
    return topology.collapse_edges(g.edges, g.lengths, g.ntaxa, pick(internal))[:2]


def _engine(g, topo, safe, nptn=None):
    eng = engine.Engine(g.patterns.shape[1], g.model.nstates, g.model.ncat, g.ntaxa, g.model.state_unknown,
                        topo.nslots, safe=safe, max_ops=2 * topo.nslots + 8, flags=engine.FLAG_SAFE_AS_GIVEN)
    eng.set_model(g.model)
    eng.set_patterns(g.freq)
    eng.set_tip_states(g.patterns)
    return eng


def _check(oracle_mod, g, edges, lengths, safe):
    topo = Topology(edges, lengths, g.ntaxa)
    eng = _engine(g, topo, safe)
    eng.compute_partials(topo.all_partials_ops())
    orc = oracle_mod.OracleTree(g.model, g.patterns, g.freq, edges, lengths, safe=safe)
    for (u, v), slot in topo.slot.items():
        gp, gs = eng.partial(slot)
        op, os_ = orc.partial(u, v)
        np.testing.assert_array_equal(gs, os_)
        scale = np.maximum(np.abs(op).max(axis=1, keepdims=True), 1e-300)
        assert np.max(np.abs(gp - op) / scale) < 1e-10, (u, v)
    for (u, v) in edges[:6]:
        u, v = int(u), int(v)
        node, dad = (v, u) if v >= g.ntaxa else (u, v)
        lg = eng.branch_lnl(topo.ref(dad, node), topo.ref(node, dad), topo.edge_len(node, dad))
        assert rel(lg, orc.lnl_branch(node, dad)) < 1e-10
    internal = [(int(u), int(v)) for (u, v) in edges if min(int(u), int(v)) >= g.ntaxa][:2]
    for (n1, n2) in internal:
        orc2 = oracle_mod.OracleTree(g.model, g.patterns, g.freq, edges, lengths, safe=safe)
        ops = topo.branch_ops(n2, n1)
        df, ddf = eng.likelihood_derv(ops, topo.ref(n1, n2), topo.ref(n2, n1), 0.07)
        odf, oddf = orc2.derv(n1, n2, 0.07)
        assert abs(df - odf) <= 1e-9 * max(1.0, abs(odf)) and abs(ddf - oddf) <= 1e-9 * max(1.0, abs(oddf))


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
@pytest.mark.parametrize("safe", [False, True])
def test_multifurcating_partials_match_oracle(oracle_mod, name, safe):
    g = load_golden(name)
    edges, lengths = _collapsed(g, lambda internal: internal[:3])
    assert np.bincount(np.asarray(edges).ravel()).max() >= 4
    _check(oracle_mod, g, edges, lengths, safe)


@pytest.mark.parametrize("safe", [False, True])
def test_multifurcating_underflow_scale_counts(oracle_mod, safe):
    ds = simulate.protein_lg_dataset(150, 40, 11, mean_bl=0.5)
    from types import SimpleNamespace
    g = SimpleNamespace(model=ds.model, patterns=ds.patterns, freq=ds.freq, edges=ds.edges, lengths=ds.lengths,
                        ntaxa=ds.ntaxa)
    edges, lengths = _collapsed(g, lambda internal: internal[::6])
    orc = oracle_mod.OracleTree(g.model, g.patterns, g.freq, edges, lengths, safe=safe)
    leaf_edge = next(e for e in edges if 0 in (int(e[0]), int(e[1])))
    _, s = orc.partial(0, int(leaf_edge[0]) + int(leaf_edge[1]))
    assert s.sum() > 0
    _check(oracle_mod, g, edges, lengths, safe)


@pytest.mark.parametrize("name", ["dna16", "prot12"])
def test_multifurcating_tree_drivers(oracle_mod, name):
    g = load_golden(name)
    edges, lengths = _collapsed(g, lambda internal: internal[1:4])
    t = engine.GpuTree(g.model, g.patterns, g.freq, edges, lengths)
    o = oracle_mod.OracleTree(g.model, g.patterns, g.freq, edges, lengths)
    assert rel(t.compute_likelihood(), o.compute_likelihood()) < 1e-10
    lg, lo = t.optimize_all_branches(), o.optimize_all_branches()
    assert rel(lg, lo) < 1e-9
    np.testing.assert_allclose(t.lengths(), o.lengths(), atol=1e-5)


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
@pytest.mark.parametrize("precision", [engine.F32, engine.TF32X3])
def test_mixed_multifurcating_match_oracle(oracle_mod, name, precision):
    """The mixed paths on multifurcating nodes: every partial (standard basis,
    exponents applied) within 1e-5 of each pattern's largest entry, branch lnL
    within 1e-6, derivatives within the mixed tolerances of the tensor-core
    tests, the tree drivers within 1e-6 after branch optimisation."""
    g = load_golden(name)
    edges, lengths = _collapsed(g, lambda internal: internal[:3])
    assert np.bincount(np.asarray(edges).ravel()).max() >= 4
    topo = Topology(edges, lengths, g.ntaxa)
    eng = engine.Engine(g.patterns.shape[1], g.model.nstates, g.model.ncat, g.ntaxa, g.model.state_unknown,
                        topo.nslots, precision=precision, max_ops=2 * topo.nslots + 8)
    eng.set_model(g.model)
    eng.set_patterns(g.freq)
    eng.set_tip_states(g.patterns)
    eng.compute_partials(topo.all_partials_ops())
    orc = oracle_mod.OracleTree(g.model, g.patterns, g.freq, edges, lengths)
    n, C = g.model.nstates, g.model.ncat
    for (u, v), slot in topo.slot.items():
        gp, _ = eng.partial(slot)
        op, _ = orc.partial(u, v)
        std = np.einsum("xi,pci->pcx", g.model.evec, op.reshape(-1, C, n)).reshape(op.shape)
        gn = gp / np.abs(gp).max(axis=1, keepdims=True)
        on = std / np.abs(std).max(axis=1, keepdims=True)
        assert np.max(np.abs(gn - on)) < 1e-5, (u, v)
    for (u, v) in edges[:6]:
        u, v = int(u), int(v)
        node, dad = (v, u) if v >= g.ntaxa else (u, v)
        lg = eng.branch_lnl(topo.ref(dad, node), topo.ref(node, dad), topo.edge_len(node, dad))
        assert rel(lg, orc.lnl_branch(node, dad)) < 1e-6, (u, v)
    internal = [(int(u), int(v)) for (u, v) in edges if min(int(u), int(v)) >= g.ntaxa][:2]
    for (n1, n2) in internal:
        orc2 = oracle_mod.OracleTree(g.model, g.patterns, g.freq, edges, lengths)
        ops = topo.branch_ops(n2, n1)
        df, ddf = eng.likelihood_derv(ops, topo.ref(n1, n2), topo.ref(n2, n1), 0.07)
        odf, oddf = orc2.derv(n1, n2, 0.07)
        assert abs(df - odf) <= 1e-4 * abs(odf) + 1e-3 and abs(ddf - oddf) <= 1e-3 * abs(oddf) + 1e-3
    t = engine.GpuTree(g.model, g.patterns, g.freq, edges, lengths, precision=precision)
    o = oracle_mod.OracleTree(g.model, g.patterns, g.freq, edges, lengths)
    assert rel(t.compute_likelihood(), o.compute_likelihood()) < 1e-6
    lg, lo = t.optimize_all_branches(), o.optimize_all_branches()
    assert rel(lg, lo) < 1e-6
    np.testing.assert_allclose(t.lengths(), o.lengths(), atol=1e-4)


def test_mixed_multifurcating_underflow():
    """150 taxa, long branches: partials that underflow FP32 many times over
    carry the per-pattern exponents through multifurcating nodes (lnL within
    1e-6 of the FP64 drop-in)."""
    ds = simulate.protein_lg_dataset(150, 400, 11, mean_bl=0.5)
    from types import SimpleNamespace
    g = SimpleNamespace(model=ds.model, patterns=ds.patterns, freq=ds.freq, edges=ds.edges, lengths=ds.lengths,
                        ntaxa=ds.ntaxa)
    edges, lengths = _collapsed(g, lambda internal: internal[::6])
    want = engine.GpuTree(g.model, g.patterns, g.freq, edges, lengths, safe=True).compute_likelihood()
    for precision in (engine.F32, engine.TF32X3):
        got = engine.GpuTree(g.model, g.patterns, g.freq, edges, lengths, precision=precision).compute_likelihood()
        assert rel(got, want) < 1e-6, (precision, got, want)
