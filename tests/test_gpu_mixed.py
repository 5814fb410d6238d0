"""Mixed-precision path (FP32 standard-basis partials, per-pattern power-of-two
exponents, FP64 exp/log/sums) against the FP64 oracle.

Tolerances (stated per quantity): lnL |dlnL| <= 1e-6 |lnL|; pattern lnL
absolute <= 1e-4; partials relative to each pattern's largest entry <= 1e-5;
first derivative relative <= 1e-4, second derivative relative <= 1e-3 (+1e-3
absolute floor); optimised branch lengths within 1e-4.
"""
import numpy as np
import pytest

from helpers import load_golden, rel
from iqtree2_gb300 import engine, simulate
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu

LNL_RTOL = 1e-6


def _engine(g, topo):
    eng = engine.Engine(g.patterns.shape[1], g.model.nstates, g.model.ncat, g.ntaxa, g.model.state_unknown,
                        topo.nslots, precision=engine.F32, max_ops=topo.nslots)
    eng.set_model(g.model)
    eng.set_patterns(g.freq)
    eng.set_tip_states(g.patterns)
    return eng


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
def test_golden_lnl_mixed(oracle_mod, name):
    g = load_golden(name)
    t = engine.GpuTree(g.model, g.patterns, g.freq, g.edges, g.lengths, precision=engine.F32)
    lnl, plh = t.compute_likelihood(want_pattern_lh=True)
    assert rel(lnl, g.lnl_std) < LNL_RTOL
    np.testing.assert_allclose(plh, g.pattern_lnl_std, atol=1e-4)


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
def test_mixed_partials_match_oracle(oracle_mod, name):
    g = load_golden(name)
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    eng = _engine(g, topo)
    done, ops = set(), []
    for (u, v) in sorted(topo.slot):
        ops += topo.ops_for(u, v, done)
    eng.compute_partials(ops)
    orc = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths)
    n, C = g.model.nstates, g.model.ncat
    U = g.model.evec
    for (u, v), s in list(topo.slot.items())[:12]:
        gp, _ = eng.partial(s)
        op, _ = orc.partial(u, v)
        # oracle eigen-space -> standard basis per category: L = U . Le
        std = np.einsum("xi,pci->pcx", U, op.reshape(-1, C, n)).reshape(op.shape)
        gn = gp / np.abs(gp).max(axis=1, keepdims=True)
        on = std / np.abs(std).max(axis=1, keepdims=True)
        assert np.max(np.abs(gn - on)) < 1e-5, (u, v)


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
def test_mixed_derivatives(oracle_mod, name):
    g = load_golden(name)
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    eng = _engine(g, topo)
    internal = [tuple(map(int, e)) for e in g.edges if min(e) >= g.ntaxa]
    done = set()
    for (n1, n2) in [tuple(map(int, g.edges[0]))] + internal[:2]:
        node, dad = n2, n1
        if node < g.ntaxa:
            node, dad = n1, n2
        ops = topo.ops_for(dad, node, done) + topo.ops_for(node, dad, done)
        a, b = topo.ref(dad, node), topo.ref(node, dad)
        orc = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths)
        first = True
        for length in (0.02, 0.1, 0.7):
            df, ddf = eng.likelihood_derv(ops if first else [], a, b, length, theta_computed=not first)
            first = False
            odf, oddf = orc.derv(n1, n2, length)
            assert abs(df - odf) <= 1e-4 * abs(odf) + 1e-3
            # second derivative: FP32 eigen-space theta (61-state transform) costs ~1e-4
            assert abs(ddf - oddf) <= 1e-3 * abs(oddf) + 1e-3
            assert rel(eng.lnl_from_buffer(length), orc.lnl_branch(node, dad)) < LNL_RTOL


@pytest.mark.parametrize("name", ["dna16", "prot12"])
def test_mixed_optimize_all_branches(oracle_mod, name):
    g = load_golden(name)
    t = engine.GpuTree(g.model, g.patterns, g.freq, g.edges, g.lengths, precision=engine.F32)
    o = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths)
    lg, lo = t.optimize_all_branches(), o.optimize_all_branches()
    assert rel(lg, lo) < LNL_RTOL
    np.testing.assert_allclose(t.lengths(), o.lengths(), atol=1e-4)


def test_mixed_deep_tree_exponents(oracle_mod):
    """Long-branch 300-taxon DNA: FP32 would underflow without the exponents."""
    ds = simulate.dna_gtr_dataset(300, 200, 5, mean_bl=0.5)
    t = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, precision=engine.F32)
    o = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
    assert rel(t.compute_likelihood(), o.compute_likelihood()) < LNL_RTOL


def test_mixed_ambiguous_states(oracle_mod):
    rng = np.random.default_rng(9)
    for ds in (simulate.dna_gtr_dataset(12, 400, 21), simulate.protein_lg_dataset(10, 200, 22)):
        pats = ds.patterns.copy()
        mask = rng.random(pats.shape) < 0.15
        pats[mask] = rng.integers(ds.model.nstates, ds.model.state_unknown + 1, size=mask.sum())
        t = engine.GpuTree(ds.model, pats, ds.freq, ds.edges, ds.lengths, precision=engine.F32)
        o = oracle_mod.OracleTree(ds.model, pats, ds.freq, ds.edges, ds.lengths)
        assert rel(t.compute_likelihood(), o.compute_likelihood()) < LNL_RTOL


@pytest.mark.parametrize("kind", ["protein", "codon"])
def test_mixed_full_size_configs(oracle_mod, kind):
    """Protein 100x50,000 and codon 40x10,000: mixed lnL within 1e-6 of the FP64 oracle."""
    ds = (simulate.protein_lg_dataset(100, 50000, 2) if kind == "protein"
          else simulate.codon_gy94_dataset(40, 10000, 3))
    t = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, precision=engine.F32)
    o = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
    lg, lo = t.compute_likelihood(), o.compute_likelihood()
    err = rel(lg, lo)
    print(f"{kind}: mixed lnL {lg:.6f} oracle {lo:.6f} rel err {err:.2e}")
    assert err < LNL_RTOL


@pytest.mark.parametrize("kind,ncat,schedule", [("codon", 3, 1), ("protein", 7, 0), ("protein", 7, 1),
                                                ("protein", 8, 0), ("codon", 1, 0)])
def test_mixed_category_counts_and_shared_memory(oracle_mod, kind, ncat, schedule):
    """Category counts whose P(t) staging sits just under the 48 KB default of
    dynamic shared memory while the kernel's static arrays push it over
    (codon x 3 categories on the level kernel, protein x 7 on the fused one):
    the launchers raise the limit whenever they stage, and the lnL matches the
    oracle."""
    import dataclasses
    from iqtree2_gb300 import autotune, models
    ds = (simulate.codon_gy94_dataset(12, 300, 91) if kind == "codon" else simulate.protein_lg_dataset(16, 600, 92))
    rates, props = models.gamma_rates_mean(0.6, ncat)
    m = dataclasses.replace(ds.model, rates=np.asarray(rates, np.float64), props=np.asarray(props, np.float64))
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    eng = engine.Engine(ds.nptn, m.nstates, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots, precision=engine.F32,
                        max_ops=topo.nslots)
    eng.set_model(m)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    autotune.apply(eng, (32, schedule, 0, 0))
    leaf, nb = 0, topo.adj[0][0][0]
    lg = eng.compute_likelihood(topo.branch_ops(nb, leaf), topo.ref(leaf, nb), topo.ref(nb, leaf),
                                topo.edge_len(leaf, nb))
    lo = oracle_mod.OracleTree(m, ds.patterns, ds.freq, ds.edges, ds.lengths).lnl_branch(nb, leaf)
    assert rel(lg, lo) < LNL_RTOL, (lg, lo)
