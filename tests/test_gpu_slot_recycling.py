"""Partials that do not fit: slot recycling (the reference's LM_MEM_SAVE,
tree/memslot.h:44-74, tree/phylotree.cpp:967-1027).

An engine with fewer partial slots than the tree has directed internal
partials recycles them least-recently-used first and recomputes partials
when needed again. Every op computes the same values in any slot, so the
likelihood, the optimised branch lengths and the optimised likelihood are
bit-identical to the run with a slot for every partial; only the number of
pattern-node updates grows. The serving loop admits a job whose partials do
not fit in half its arena with such an engine instead of refusing it.
"""
import numpy as np
import pytest

from helpers import load_golden
from iqtree2_gb300 import engine, serving, simulate, topology

pytestmark = pytest.mark.gpu


def _min_slots(ntaxa):
    lg = 1
    while (1 << lg) < ntaxa:
        lg += 1
    return 2 * lg + 4


@pytest.mark.parametrize("precision", [engine.F64, engine.F32])
def test_recycled_slots_give_identical_results(precision):
    ds = simulate.dna_gtr_dataset(96, 3000, 61)
    full = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, precision=precision)
    few = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, precision=precision,
                         slots=_min_slots(96))
    assert few.compute_likelihood() == full.compute_likelihood()
    lf, lr = full.optimize_all_branches(), few.optimize_all_branches()
    assert lf == lr
    np.testing.assert_array_equal(full.lengths(), few.lengths())
    assert few.num_updates() > full.num_updates()  # partials were recomputed


def test_recycled_slots_multifurcating_fp64(oracle_mod):
    g = load_golden("prot12")
    ds = simulate.protein_lg_dataset(70, 800, 63)
    internal = [k for k, (u, v) in enumerate(ds.edges) if min(int(u), int(v)) >= ds.ntaxa]
    e2, l2, _ = topology.collapse_edges(ds.edges, ds.lengths, ds.ntaxa, internal[::5])
    full = engine.GpuTree(ds.model, ds.patterns, ds.freq, e2, l2)
    few = engine.GpuTree(ds.model, ds.patterns, ds.freq, e2, l2, slots=_min_slots(70))
    assert few.compute_likelihood() == full.compute_likelihood()
    assert few.optimize_all_branches(iterations=2) == full.optimize_all_branches(iterations=2)
    del g


def test_too_few_slots_refused():
    ds = simulate.dna_gtr_dataset(40, 500, 62)
    with pytest.raises(engine.EngineError) as ei:
        engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, slots=_min_slots(40) - 1)
    assert ei.value.code == 1


def test_server_admits_oversized_job_with_recycled_slots():
    ds = simulate.dna_gtr_dataset(200, 20000, 64)
    need_full = engine.Engine.memory_required(nptn=ds.nptn, nstates=4, ncat=4, ntaxa=200, state_unknown=18,
                                              nslots=3 * 198, precision=engine.F32, max_ops=400)
    budget = need_full // 3  # the full engine would take 1.5x the budget's half
    s_big = serving.Server(max_active=2, memory_budget=8 << 30)
    want = s_big.wait(s_big.submit(ds, opt_iterations=1), nedge=len(ds.edges))
    s_big.close()
    s = serving.Server(max_active=2, memory_budget=budget)
    got = s.wait(s.submit(ds, opt_iterations=1), nedge=len(ds.edges))
    st = s.stats()
    s.close()
    assert want["status"] == 0 and got["status"] == 0, got["error"]
    assert st["refused"] == 0
    assert got["slots"] < 3 * 198 and got["bytes"] <= budget // 2 + (1 << 20)
    assert got["lnl_initial"] == want["lnl_initial"] and got["lnl"] == want["lnl"]
    np.testing.assert_array_equal(got["lengths"], want["lengths"])
