"""Failure paths, made on the host or by a bounded wait that runs out.

* A wait on another CTA's progress (the producer flags of the 4-state
  dataflow kernel and of the tensor-core dataflow schedules) that gives up:
  with the per-engine limit set to one poll the launch stops, the call
  returns IQGPU_ERR_TIMEOUT, and the same engine then computes the right
  likelihood. No GPU fault is involved: every wait is bounded and a CTA that
  gives up drains what it has in flight and returns.
* IQGPU_ERR_NONFINITE, the reference's outError "Numerical underflow
  (lh-derivative) ... -safe" (tree/phylokernelnew.h:2577-2578): a pattern
  whose likelihood is exactly zero (a tip vector of zeros) makes the NORM
  derivative non-finite; the SAFE kernel sets df = ddf = 0 instead, as the
  reference does (:2629-2632).
* IQGPU_ERR_NEWTON, the reference's nrerror in minimizeNewton
  (utils/optimization.cpp:496): no Newton step allowed.
"""
import numpy as np
import pytest

from helpers import load_golden, rel
from iqtree2_gb300 import engine, simulate
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu

TIMEOUT = 5
NONFINITE = 4
NEWTON = 8


def test_dataflow_wait_gives_up_and_engine_stays_usable():
    ds = simulate.dna_gtr_dataset(200, 20000, 7)
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    m = ds.model
    eng = engine.Engine(ds.nptn, 4, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots, precision=engine.F32,
                        max_ops=topo.nslots)
    eng.set_model(m)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    engine.lib().iqgpu_set_tile(eng.h, 1)
    engine.lib().iqgpu_set_schedule(eng.h, 2)  # dataflow: items wait on their producers' flags
    u0, v0 = next((int(u), int(v)) for (u, v) in ds.edges if 0 in (int(u), int(v)))
    nb = u0 + v0
    ops = topo.branch_ops(nb, 0)
    args = (topo.ref(0, nb), topo.ref(nb, 0), topo.edge_len(0, nb))
    want = eng.compute_likelihood(ops, *args)
    for _ in range(2):
        engine._check(engine.lib().iqgpu_set_wait_limit(eng.h, 1))
        with pytest.raises(engine.EngineError) as ei:
            eng.compute_likelihood(ops, *args)
        assert ei.value.code == TIMEOUT
        assert "gave up" in str(ei.value)
        engine._check(engine.lib().iqgpu_set_wait_limit(eng.h, 0))
        assert eng.compute_likelihood(ops, *args) == want  # deterministic reductions: bit for bit


@pytest.mark.parametrize("schedule", [6, 7])
def test_tensor_core_dataflow_wait_gives_up_and_engine_stays_usable(schedule):
    """The tensor-core dataflow schedules (6: category-split items, 7: whole
    items) with a one-poll limit on their producer-flag waits: the workers of
    an item whose producers are not done stop at the item boundary, the issuer
    drains its copies and MMAs and frees its tensor memory, the launch reports
    IQGPU_ERR_TIMEOUT, and the same engine then computes the lnL bit for bit."""
    from iqtree2_gb300 import autotune
    ds = simulate.codon_gy94_dataset(40, 3000, 36)
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    m = ds.model
    eng = engine.Engine(ds.nptn, m.nstates, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots,
                        precision=engine.TF32X3, max_ops=topo.nslots)
    eng.set_model(m)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    autotune.apply(eng, (0, schedule, 2, 1))
    u0, v0 = next((int(u), int(v)) for (u, v) in ds.edges if 0 in (int(u), int(v)))
    nb = u0 + v0
    ops = topo.branch_ops(nb, 0)
    args = (topo.ref(0, nb), topo.ref(nb, 0), topo.edge_len(0, nb))
    want = eng.compute_likelihood(ops, *args)
    for _ in range(2):
        engine._check(engine.lib().iqgpu_set_wait_limit(eng.h, 1))
        with pytest.raises(engine.EngineError) as ei:
            eng.compute_likelihood(ops, *args)
        assert ei.value.code == TIMEOUT
        engine._check(engine.lib().iqgpu_set_wait_limit(eng.h, 0))
        assert eng.compute_likelihood(ops, *args) == want


def _zero_tip_model(g):
    from types import SimpleNamespace
    tip = np.array(g.model.tip_lh, copy=True)
    tip[0, :] = 0.0  # state A contributes nothing: patterns with an A have likelihood 0
    return SimpleNamespace(**{**g.model.__dict__, "tip_lh": tip})


@pytest.mark.parametrize("safe", [False, True])
def test_nonfinite_derivative_norm_error_safe_zero(safe):
    g = load_golden("dna16")
    m = _zero_tip_model(g)
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    eng = engine.Engine(g.patterns.shape[1], 4, m.ncat, g.ntaxa, m.state_unknown, topo.nslots, safe=safe,
                        max_ops=topo.nslots, flags=engine.FLAG_SAFE_AS_GIVEN)
    eng.set_model(m)
    eng.set_patterns(g.freq)
    eng.set_tip_states(g.patterns)
    n1, n2 = (int(x) for x in g.edges[0])
    node, dad = (n2, n1) if n2 >= g.ntaxa else (n1, n2)
    ops = topo.branch_ops(node, dad)
    if safe:
        df, ddf = eng.likelihood_derv(ops, topo.ref(dad, node), topo.ref(node, dad), 0.1)
        assert df == 0.0 and ddf == 0.0
    else:
        with pytest.raises(engine.EngineError) as ei:
            eng.likelihood_derv(ops, topo.ref(dad, node), topo.ref(node, dad), 0.1)
        assert ei.value.code == NONFINITE
        assert "-safe" in str(ei.value) or "SAFE" in str(ei.value)


def test_newton_without_steps_reports_nrerror():
    g = load_golden("dna16")
    t = engine.GpuTree(g.model, g.patterns, g.freq, g.edges, g.lengths * 3.0)
    n1, n2 = (int(x) for x in g.edges[0])
    with pytest.raises(engine.EngineError) as ei:
        t.optimize_one_branch(n1, n2, max_nr_step=0)
    assert ei.value.code == NEWTON
    # the tree stays usable
    t.optimize_one_branch(n1, n2, max_nr_step=100)
    assert np.isfinite(t.compute_likelihood())
