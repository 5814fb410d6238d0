"""minimizeNewton on the device (iqgpu_newton_branch) against the same loop
on the host (utils/optimization.cpp:422-499, one iqgpu_likelihood_derv per
step) and the tree driver's two modes against each other and the oracle.

The device kernel sums the same per-pattern derivative terms as
iqgpu_likelihood_derv in another order, so the two loops agree to rounding:
the same iteration count on nearly every branch, and the optimum within the
tolerance xacc both stop at."""
import numpy as np
import pytest

from helpers import load_golden, load_ref_golden, rel
from iqtree2_gb300 import engine, models, simulate
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu
NONFINITE, NEWTON, ARG = 4, 8, 1


def newton_host(eng, ops, a, b, x1, xguess, x2, xacc, max_steps):
    """minimizeNewton over computeFuncDerv (f = -df, df = -ddf), derivatives
    from iqgpu_likelihood_derv: (optx, iterations)."""
    first = [True]

    def fd(x):
        df, ddf = eng.likelihood_derv(ops if first[0] else [], a, b, x, theta_computed=not first[0])
        first[0] = False
        return -df, -ddf
    rts = min(max(xguess, x1), x2)
    f, df = fd(rts)
    assert np.isfinite(f) and np.isfinite(df)
    if df >= 0.0 and abs(f) < xacc:
        return rts, 0
    xl, xh = (rts, x2) if f < 0.0 else (x1, rts)
    for j in range(1, max_steps + 1):
        rts_old = rts
        if df <= 0.0 or ((rts - xh) * df - f) * ((rts - xl) * df - f) >= 0.0:
            dx = 0.5 * (xh - xl)
            rts = xl + dx
            if xl == rts:
                return rts, j
        else:
            dx = f / df
            temp = rts
            rts -= dx
            if temp == rts:
                return rts, j
        if abs(dx) < xacc or j == max_steps:
            return rts_old, j
        f, df = fd(rts)
        assert np.isfinite(f) and np.isfinite(df)
        if df > 0.0 and abs(f) < xacc:
            return rts, j
        if f < 0.0:
            xl = rts
        elif f > 0.0:
            xh = rts
    raise AssertionError("iteration limit")


def _engine(model, patterns, freq, topo, ntaxa, safe=False, precision=engine.F64):
    eng = engine.Engine(patterns.shape[1], model.nstates, model.ncat, ntaxa, model.state_unknown, topo.nslots,
                        safe=safe, precision=precision, max_ops=2 * topo.nslots, flags=engine.FLAG_SAFE_AS_GIVEN)
    eng.set_model(model)
    eng.set_patterns(freq)
    eng.set_tip_states(patterns)
    return eng


def _branches(edges, ntaxa, k=6):
    out = []
    for u, v in edges[:k]:
        u, v = int(u), int(v)
        out.append((v, u) if v >= ntaxa else (u, v))  # (node, dad): node internal where one is
    return out


@pytest.mark.parametrize("name,safe", [("dna16", False), ("prot12", False), ("codon8", True), ("dna16", True)])
def test_kernel_level_matches_host_loop(name, safe):
    g = load_golden(name)
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    eng = _engine(g.model, g.patterns, g.freq, topo, g.ntaxa, safe)
    same_steps = 0
    for node, dad in _branches(g.edges, g.ntaxa):
        ops = topo.ops_for(dad, node, set()) + topo.ops_for(node, dad, set())
        a, b = topo.ref(dad, node), topo.ref(node, dad)
        x0 = topo.edge_len(node, dad)
        xh, jh = newton_host(eng, ops, a, b, 1e-6, x0, 10.0, 1e-6, 100)
        xd, jd, d2l, last = eng.newton_branch([], a, b, 1e-6, x0, 10.0, 1e-6, 100, theta_computed=True, full=True)
        same_steps += jh == jd
        assert abs(xd - xh) <= 1e-6 * max(1.0, xh), (node, dad, xd, xh)
        # d2l is computeFuncDerv's second value (-ddf) at the last evaluated length
        _, ddf = eng.likelihood_derv([], a, b, last, theta_computed=True)
        assert abs(d2l + ddf) <= 1e-9 * max(1.0, abs(ddf)), (d2l, ddf)
        assert 1e-6 <= last <= 10.0 and (jd > 0 or last == min(max(x0, 1e-6), 10.0))
        # the theta buffer stays valid: the lnL at the optimum from it
        assert rel(eng.lnl_from_buffer(xd), eng.compute_likelihood(ops, a, b, xd)) < 1e-12
        # and with theta_computed = 0 the traversal runs first, same answer
        xd2, _ = eng.newton_branch(ops, a, b, 1e-6, x0, 10.0, 1e-6, 100)
        assert xd2 == xd
    assert same_steps >= len(_branches(g.edges, g.ntaxa)) - 1


@pytest.mark.parametrize("name,safe", [("example", False), ("prot_M126_27_269", False), ("underflow150", True)])
def test_tree_driver_device_and_host_newton_agree(oracle_mod, name, safe):
    g = load_ref_golden(name)
    runs = []
    for dev in (True, False):
        t = engine.GpuTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe,
                           flags=engine.FLAG_SAFE_AS_GIVEN)
        t.set_device_newton(dev)
        lnl = t.optimize_all_branches()
        runs.append((lnl, t.lengths(), t.compute_likelihood()))
    (ld, Ld, cd), (lh, Lh, ch) = runs
    assert rel(ld, lh) < 1e-10
    np.testing.assert_allclose(Ld, Lh, atol=1e-5)
    assert rel(cd, ch) < 1e-10
    o = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe)
    assert rel(ld, o.optimize_all_branches()) < 1e-9


def test_mixture_tree_device_newton():
    """Profile mixture (eigen system per class): device and host loops agree."""
    rng = np.random.default_rng(5)
    ds = simulate.dna_gtr_dataset(20, 1500, 63)
    R = rng.uniform(0.5, 3.0, size=(4, 4))
    R = (R + R.T) / 2
    mix = models.profile_mixture(R, [rng.dirichlet(np.full(4, 3.0)) for _ in range(3)],
                                 rng.uniform(0.5, 1.5, size=3), 0.6, 2)
    res = []
    for dev in (True, False):
        t = engine.GpuTree(mix, ds.patterns, ds.freq, ds.edges, ds.lengths)
        t.set_device_newton(dev)
        res.append((t.optimize_all_branches(), t.lengths()))
    assert rel(res[0][0], res[1][0]) < 1e-10
    np.testing.assert_allclose(res[0][1], res[1][1], atol=1e-5)


@pytest.mark.parametrize("safe", [False, True])
def test_nonfinite_derivative(safe):
    """All-zero tip likelihoods: NORM reports the reference's underflow error,
    SAFE zeroes the derivative and minimizeNewton returns its start."""
    from types import SimpleNamespace
    g = load_golden("dna16")
    m = SimpleNamespace(**{**g.model.__dict__, "tip_lh": np.zeros_like(g.model.tip_lh)})
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    eng = _engine(m, g.patterns, g.freq, topo, g.ntaxa, safe)
    node, dad = _branches(g.edges, g.ntaxa, 1)[0]
    ops = topo.branch_ops(node, dad)
    a, b = topo.ref(dad, node), topo.ref(node, dad)
    if safe:
        assert eng.newton_branch(ops, a, b, 1e-6, 0.1, 10.0, 1e-6, 100) == (0.1, 0)
    else:
        with pytest.raises(engine.EngineError) as ei:
            eng.newton_branch(ops, a, b, 1e-6, 0.1, 10.0, 1e-6, 100)
        assert ei.value.code == NONFINITE


def test_iteration_limit_and_refusals():
    g = load_golden("dna16")
    topo = Topology(g.edges, g.lengths * 3.0, g.ntaxa)
    eng = _engine(g.model, g.patterns, g.freq, topo, g.ntaxa)
    node, dad = _branches(g.edges, g.ntaxa, 1)[0]
    ops = topo.branch_ops(node, dad)
    a, b = topo.ref(dad, node), topo.ref(node, dad)
    with pytest.raises(engine.EngineError) as ei:
        eng.newton_branch(ops, a, b, 1e-6, 0.3, 10.0, 1e-6, 0)
    assert ei.value.code == NEWTON and "Maximum number of iterations" in str(ei.value)
    x, _ = eng.newton_branch([], a, b, 1e-6, 0.3, 10.0, 1e-6, 100, theta_computed=True)
    assert 1e-6 <= x <= 10.0
    # theta_computed for another branch is a state error
    n2, d2 = _branches(g.edges, g.ntaxa, 2)[1]
    with pytest.raises(engine.EngineError):
        eng.newton_branch([], topo.ref(d2, n2), topo.ref(n2, d2), 1e-6, 0.3, 10.0, 1e-6, 100, theta_computed=True)
    assert eng.newton_supported()
    # mixed-precision engines keep the host loop: refused before any work
    em = _engine(g.model, g.patterns, g.freq, topo, g.ntaxa, precision=engine.F32)
    assert not em.newton_supported()
    with pytest.raises(engine.EngineError) as ei:
        em.newton_branch(ops, a, b, 1e-6, 0.3, 10.0, 1e-6, 100)
    assert ei.value.code == ARG


def _optimise(g_or_ds, mode, safe=False, bounds=None, slots=None, max_nr_step=100):
    t = engine.GpuTree(g_or_ds.model, g_or_ds.patterns, g_or_ds.freq, g_or_ds.edges, g_or_ds.lengths, safe=safe,
                       flags=engine.FLAG_SAFE_AS_GIVEN, slots=slots)
    t.set_device_newton(mode)
    if bounds:
        t.set_bounds(*bounds)
    lnl = t.optimize_all_branches(max_nr_step=max_nr_step)
    out = (lnl, t.lengths(), t.compute_likelihood(), t.num_updates())
    t.close()
    return out


@pytest.mark.parametrize("name,safe", [("example", False), ("prot_M126_27_269", False), ("underflow150", True)])
def test_device_pass_matches_branch_by_branch(oracle_mod, name, safe):
    """optimizeAllBranches with each pass on the device (one host wait per
    pass, lengths kept in device memory between the branches' solves) runs the
    same kernels on the same inputs as the branch-by-branch device driver: the
    same lnL, lengths and tree lnL afterwards, bit for bit, and the oracle's
    lnL within 1e-9."""
    g = load_ref_golden(name)
    (lp, Lp, cp, up), (lb, Lb, cb, ub) = _optimise(g, 1, safe), _optimise(g, 2, safe)
    assert lp == lb and cp == cb
    np.testing.assert_array_equal(Lp, Lb)
    assert up >= ub  # a branch that kept its length may leave partials the pass recomputes
    o = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe)
    assert rel(lp, o.optimize_all_branches()) < 1e-9


def test_device_pass_short_alignment():
    """DNA GTR+G4 16 taxa x 1,000 sites, the CPU-runnable configuration: the
    pass and the branch-by-branch driver agree bit for bit."""
    ds = simulate.dna_gtr_dataset(16, 1000, 1, mean_bl=0.1, alpha=0.5)
    (lp, Lp, cp, _), (lb, Lb, cb, _) = _optimise(ds, 1), _optimise(ds, 2)
    assert lp == lb and cp == cb
    np.testing.assert_array_equal(Lp, Lb)


def test_device_pass_taken_again_at_the_bound():
    """With max_bl low enough that optima land above 0.95 max_bl (where the
    reference compares the lnL at the bound with the one at the old length),
    or with no Newton step allowed (the solve fails), the pass goes back to
    its start and runs branch by branch: the same results, or the same error,
    as that driver."""
    g = load_ref_golden("example")
    assert g.lengths.max() > 0.02
    for kw in (dict(bounds=(1e-6, 0.02)), dict(max_nr_step=0)):
        try:
            ref = _optimise(g, 2, **kw)
        except engine.EngineError as err:
            with pytest.raises(engine.EngineError) as ei:
                _optimise(g, 1, **kw)
            assert ei.value.code == err.code
            continue
        lp, Lp, cp, _ = _optimise(g, 1, **kw)
        assert lp == ref[0] and cp == ref[2]
        np.testing.assert_array_equal(Lp, ref[1])


def test_device_pass_not_taken_without_a_slot_per_partial():
    """Fewer slots than directed internal partials (slots recycled, the
    reference's LM_MEM_SAVE): the branch-by-branch driver runs, results as
    with a slot per partial."""
    g = load_ref_golden("example")
    full = _optimise(g, 1)
    few = _optimise(g, 1, slots=max(6, 3 * (g.ntaxa - 2) // 2))
    assert rel(few[0], full[0]) < 1e-12
    np.testing.assert_allclose(few[1], full[1], atol=1e-12)
