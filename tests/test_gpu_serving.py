"""Serving loop: continuous batching, admission by memory, and results that
do not depend on what else runs.

Tolerances: a job's lnL and optimised branch lengths are bit-identical alone
and in the mix (every reduction is deterministic); the initial lnL matches the
FP64 oracle within 1e-6 (mixed) / 1e-10 (FP64) relative.
"""
import numpy as np
import pytest

from helpers import rel
from iqtree2_gb300 import engine, serving, simulate

pytestmark = pytest.mark.gpu


def _jobs():
    return [simulate.dna_gtr_dataset(12, 800, 101), simulate.protein_lg_dataset(10, 300, 102),
            simulate.dna_gtr_dataset(30, 2000, 103), simulate.protein_lg_dataset(16, 600, 104),
            simulate.dna_gtr_dataset(8, 500, 105), simulate.dna_gtr_dataset(20, 1500, 106)]


@pytest.mark.parametrize("precision", [engine.F32, engine.F64])
def test_same_result_alone_and_in_the_mix(oracle_mod, precision):
    """Continuous batching: a long job starts, the others arrive while it runs
    and are admitted beside it (their intervals overlap its own); every result
    is bit-identical to the same job run alone."""
    import time
    long_job = simulate.dna_gtr_dataset(120, 30000, 107)
    jobs = [long_job] + _jobs()
    alone = []
    s1 = serving.Server(max_active=1, memory_budget=16 << 30)
    for ds in jobs:
        jid = s1.submit(ds, precision=precision, opt_iterations=2)
        alone.append(s1.wait(jid, nedge=len(ds.edges)))
    s1.close()
    s2 = serving.Server(max_active=6, memory_budget=16 << 30)
    ids = [s2.submit(long_job, precision=precision, opt_iterations=2)]
    time.sleep(0.05)  # the long job is admitted and running when the others arrive
    ids += [s2.submit(ds, precision=precision, opt_iterations=2) for ds in jobs[1:]]
    mixed = [s2.wait(j, nedge=len(ds.edges)) for j, ds in zip(ids, jobs)]
    st = s2.stats()
    s2.close()
    assert st["completed"] == len(jobs) and st["refused"] == 0
    first = mixed[0]
    arrived_while_running = [r for r in mixed[1:] if first["t_start"] < r["t_submit"] < first["t_end"]]
    overlapping = [r for r in arrived_while_running if r["t_start"] < first["t_end"]]
    assert arrived_while_running, "no job arrived while the long one ran"
    assert overlapping, "no job was admitted while the long one ran"
    assert st["peak_active"] >= 2
    tol = 1e-6 if precision == engine.F32 else 1e-10
    for a, b, ds in zip(alone, mixed, jobs):
        assert a["status"] == 0 and b["status"] == 0, (a["error"], b["error"])
        assert a["lnl"] == b["lnl"] and a["lnl_initial"] == b["lnl_initial"]
        np.testing.assert_array_equal(a["lengths"], b["lengths"])
        if ds is not long_job:
            o = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
            assert rel(a["lnl_initial"], o.compute_likelihood()) < tol
        assert b["lnl"] >= b["lnl_initial"] - 1e-6 * abs(b["lnl_initial"])


def test_admission_by_memory_and_refusal():
    small = [simulate.dna_gtr_dataset(40, 8000, 200 + k) for k in range(5)]
    big = simulate.protein_lg_dataset(300, 20000, 209)  # does not fit even with recycled slots
    need_small = max(engine.Engine.memory_required(nptn=ds.nptn, nstates=4, ncat=4, ntaxa=40, state_unknown=18,
                                                   nslots=114, precision=engine.F32, max_ops=80) for ds in small)
    budget = int(need_small * 2.5)  # room for two small jobs at a time
    s = serving.Server(max_active=8, memory_budget=budget)
    ids = [s.submit(ds) for ds in small[:2]] + [s.submit(big)] + [s.submit(ds) for ds in small[2:]]
    res = [s.wait(j) for j in ids]
    st = s.stats()
    s.close()
    assert res[2]["status"] == 2 and "admission refused" in res[2]["error"]
    assert all(r["status"] == 0 for k, r in enumerate(res) if k != 2)
    assert st["refused"] == 1 and st["completed"] == 5
    assert st["peak_bytes"] <= budget
    assert st["peak_active"] == 2  # the two small jobs ran together; the budget holds no third
