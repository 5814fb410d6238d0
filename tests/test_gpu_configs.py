"""The benchmark configurations checked against the oracle at full size.

* DNA GTR+G4, 200 taxa x 100,000 sites (the batched workload's alignment):
  mixed FP32 lnL within 1e-6 and FP64 within 1e-8 of the oracle (relative).
* Codon GY94+G4, 40 taxa x 10,000 codons through the FP64 drop-in in SAFE,
  as the reference chooses for 61 states (tree/phylotreesse.cpp:95-96): lnL
  within 1e-10, the scale counts of every partial of the traversal identical
  to the oracle's, partial values within 1e-6 of each pattern's maximum:
  deep 61-state eigen-space partials cancel, so summation order shows at
  1e-7 -- IQ-TREE's own SIMD+FMA kernels differ from its one-lane kernels by
  1.7e-7 on the same partial (partial 56->42 of this tree).
* 64 NNI candidates on a 120-taxon tree in one batch: each candidate's lnL
  within 1e-6 and optimised central branch within 1e-4 of the oracle's
  optimizeOneBranch on the swapped tree (tree/phylotree.cpp:4069-4320).
"""
import numpy as np
import pytest

from helpers import rel
from iqtree2_gb300 import engine, simulate
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu


def test_dna_200x100k_mixed_and_fp64(oracle_mod):
    ds = simulate.dna_gtr_dataset(200, 100000, 7)
    o = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
    lo = o.compute_likelihood()
    del o
    tm = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, precision=engine.F32)
    lm = tm.compute_likelihood()
    tm.close()
    assert rel(lm, lo) < 1e-6, (lm, lo)
    t64 = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
    l64 = t64.compute_likelihood()
    assert rel(l64, lo) < 1e-8, (l64, lo)


def test_codon_40x10k_fp64_safe_scale_counts(oracle_mod):
    ds = simulate.codon_gy94_dataset(40, 10000, 3)
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    m = ds.model
    eng = engine.Engine(ds.nptn, 61, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots, max_ops=topo.nslots)
    assert eng.safe  # chosen by the engine, as setLikelihoodKernel does for 61 states
    eng.set_model(m)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    u0, v0 = next((int(u), int(v)) for (u, v) in ds.edges if 0 in (int(u), int(v)))
    nb = u0 + v0
    ops = topo.branch_ops(nb, 0)
    lg = eng.compute_likelihood(ops, topo.ref(0, nb), topo.ref(nb, 0), topo.edge_len(0, nb))
    o = oracle_mod.OracleTree(m, ds.patterns, ds.freq, ds.edges, ds.lengths, safe=True)
    assert rel(lg, o.lnl_branch(nb, 0)) < 1e-10
    slot_of = {s: uv for uv, s in topo.slot.items()}
    scaled = 0
    for k, op in enumerate(ops):
        u, v = slot_of[op[0]]
        gp, gs = eng.partial(op[0])
        op_, os_ = o.partial(u, v)
        np.testing.assert_array_equal(gs, os_)
        scaled += int(gs.sum())
        if k % 9 == 0:
            scale = np.maximum(np.abs(op_).max(axis=1, keepdims=True), 1e-300)
            assert np.max(np.abs(gp - op_) / scale) < 1e-6, (u, v)
    print(f"codon 40x10k SAFE: {len(ops)} partials, {scaled} scale events, all identical")


def _swapped(edges, u, v, x, y):
    e = np.array(edges, copy=True)
    for k, (p, q) in enumerate(e):
        if {int(p), int(q)} == {u, x}:
            e[k] = (v, x)
        elif {int(p), int(q)} == {v, y}:
            e[k] = (u, y)
    return e


def test_nni_batch_64_candidates_120_taxa(oracle_mod):
    ds = simulate.dna_gtr_dataset(120, 4000, 45)
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    cands = topo.nni_candidates(64)
    assert len(cands) == 64
    nslots = topo.nslots + 2 * len(cands)
    eng = engine.Engine(ds.nptn, 4, 4, ds.ntaxa, 18, nslots, precision=engine.F32,
                        max_ops=max(nslots, 2 * len(cands)))
    eng.set_model(ds.model)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    eng.compute_partials(topo.all_partials_ops())
    lnl, blen = eng.nni_batch(topo.nni_batch_entries(cands, topo.nslots), max_nr_step=10, min_bl=1e-6,
                              max_bl=10.0)
    for k, c in enumerate(cands):
        u, v = c["u"], c["v"]
        edges = _swapped(ds.edges, u, v, c["n2"][0], c["n1"][1])
        o = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, edges, ds.lengths)
        assert o.optimize_one_branch(u, v, 10) == 0
        ol = o.compute_likelihood()
        ob = o.lengths()[[i for i, (p, q) in enumerate(edges) if {int(p), int(q)} == {u, v}][0]]
        assert rel(lnl[k], ol) < 1e-6, (k, lnl[k], ol)
        assert abs(blen[k] - ob) < 1e-4, (k, blen[k], ob)
