"""Tensor-core path (tcgen05, split TF32 in three passes) for 20- and 61-state
models against the FP64 oracle and against the FP32 CUDA-core kernels.

Tolerances, as for the FP32 path: lnL |dlnL| <= 1e-6 |lnL|; pattern lnL
absolute <= 1e-4; partials relative to each pattern's largest entry <= 1e-5;
first derivative relative <= 1e-4, second <= 1e-3 (+1e-3 absolute floor);
optimised branch lengths within 1e-4. The two schedules of the tensor-core
kernel run the same per-op arithmetic and agree bit for bit.
"""
import numpy as np
import pytest

from helpers import load_golden, rel
from iqtree2_gb300 import autotune, engine, simulate
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu

LNL_RTOL = 1e-6


def _engine(g, topo, precision=engine.TF32X3):
    eng = engine.Engine(g.patterns.shape[1], g.model.nstates, g.model.ncat, g.patterns.shape[0], g.model.state_unknown,
                        topo.nslots, precision=precision, max_ops=topo.nslots)
    eng.set_model(g.model)
    eng.set_patterns(g.freq)
    eng.set_tip_states(g.patterns)
    return eng


@pytest.mark.parametrize("name", ["prot12", "codon8"])
def test_tc_golden_lnl(oracle_mod, name):
    g = load_golden(name)
    t = engine.GpuTree(g.model, g.patterns, g.freq, g.edges, g.lengths, precision=engine.TF32X3)
    lnl, plh = t.compute_likelihood(want_pattern_lh=True)
    assert rel(lnl, g.lnl_std) < LNL_RTOL
    np.testing.assert_allclose(plh, g.pattern_lnl_std, atol=1e-4)


@pytest.mark.parametrize("name", ["prot12", "codon8"])
def test_tc_partials_match_oracle(oracle_mod, name):
    g = load_golden(name)
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    eng = _engine(g, topo)
    assert eng.tensor_cores
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
        std = np.einsum("xi,pci->pcx", U, op.reshape(-1, C, n)).reshape(op.shape)
        gn = gp / np.abs(gp).max(axis=1, keepdims=True)
        on = std / np.abs(std).max(axis=1, keepdims=True)
        assert np.max(np.abs(gn - on)) < 1e-5, (u, v)


@pytest.mark.parametrize("name", ["prot12", "codon8"])
def test_tc_derivatives(oracle_mod, name):
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
            assert abs(ddf - oddf) <= 1e-3 * abs(oddf) + 1e-3
            assert rel(eng.lnl_from_buffer(length), orc.lnl_branch(node, dad)) < LNL_RTOL


def test_tc_optimize_all_branches(oracle_mod):
    g = load_golden("prot12")
    t = engine.GpuTree(g.model, g.patterns, g.freq, g.edges, g.lengths, precision=engine.TF32X3)
    o = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths)
    lg, lo = t.optimize_all_branches(), o.optimize_all_branches()
    assert rel(lg, lo) < LNL_RTOL
    np.testing.assert_allclose(t.lengths(), o.lengths(), atol=1e-4)


@pytest.mark.parametrize("kind", ["protein", "codon"])
def test_tc_schedules_agree_and_match_cuda_cores(oracle_mod, kind):
    """Ragged pattern count (not a multiple of 128), tip-tip, tip-internal and
    internal-internal ops. Codon (no CUDA-core tail: every level of every
    schedule on the tensor cores, the warp-specialised kernel with
    category-split items): all schedules and ring depths bit-identical.
    Protein: schedules differ in which narrow levels go to the CUDA-core tail
    (FP32) rather than the split-TF32 tensor cores (the dataflow schedule puts
    every level on the tensor cores; split TF32 is ~1.5e-7 from FP64 at
    worst), so they agree within 3e-7. The CUDA-core FP32 kernel within the
    mixed tolerance."""
    ds = (simulate.protein_lg_dataset(40, 1500, 31) if kind == "protein"
          else simulate.codon_gy94_dataset(16, 700, 32))
    topo = Topology(ds.edges, ds.lengths, ds.patterns.shape[0])
    leaf, nb = 0, topo.adj[0][0][0]
    ops = engine.Engine.ops_array(topo.branch_ops(nb, leaf))
    a, b, length = topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb)
    want = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths).lnl_branch(nb, leaf)
    tc = _engine(ds, topo)
    got = {}
    for cand in autotune.candidates(tc):
        autotune.apply(tc, cand)
        got[cand] = tc.compute_likelihood(ops, a, b, length)
        assert rel(got[cand], want) < LNL_RTOL, cand
    vals = set(got.values())
    if kind == "codon":
        assert len(vals) == 1, got  # same per-op arithmetic in every schedule and ring depth
    else:
        assert max(vals) - min(vals) <= 3e-7 * abs(min(vals)), got
    cc = _engine(ds, topo, engine.F32)
    assert rel(cc.compute_likelihood(ops, a, b, length), vals.pop()) < LNL_RTOL


def _levels(ops):
    """Height of each op's output in the traversal (0: both children tips)."""
    h, out = {}, []
    for (dad, c0, c1, _, _) in ops:
        lv = max([h[c] + 1 for c in (c0, c1) if c >= 0], default=0)
        h[dad] = lv
        out.append(lv)
    return out


def test_tc_level_kernels_protein(oracle_mod):
    """Protein 100 taxa x 20,000 sites: wide enough that the level schedules
    launch the tensor-core level kernels (single-issuer, warp-specialised and
    A-in-tensor-memory), with tip-internal and internal-internal items mixed
    in one launch and a ragged last tile. Every candidate within 1e-6 of the
    FP64 oracle and within 3e-7 of the others (schedules may differ in which
    narrow levels go to the CUDA-core tail); the partials of levels 1-3, which
    every schedule computes on the tensor cores (operand A in shared or in
    tensor memory), bit-identical; the A-in-tensor-memory kernel
    deterministic; schedule 5 runs the narrow levels as category-split items
    (bit-identical partials on the levels every schedule puts on the tensor
    cores); schedules 8 and 9 run the deep-ring kernel (one CTA per SM, eight
    worker warps splitting each row's states between two warps), bit-identical
    on those levels and deterministic; schedule 9 runs the one-op levels in
    one launch of it per pattern tile (each CTA waiting only on its own
    earlier items), on a tree and on a small alignment where every op goes
    there."""
    ds = simulate.protein_lg_dataset(100, 20000, 35)
    topo = Topology(ds.edges, ds.lengths, ds.patterns.shape[0])
    leaf, nb = 0, topo.adj[0][0][0]
    ops_l = topo.branch_ops(nb, leaf)
    ops = engine.Engine.ops_array(ops_l)
    a, b, length = topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb)
    want = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths).lnl_branch(nb, leaf)
    lv = _levels(ops_l)
    check = [op[0] for op, l in zip(ops_l, lv) if 1 <= l <= 3]
    assert len(check) >= 20
    eng = _engine(ds, topo)
    got, launches, parts = {}, {}, {}
    for cand in [(0, 0, 2, 1), (0, 1, 2, 1), (0, 3, 2, 1), (0, 4, 0, 0), (0, 5, 2, 1), (0, 6, 2, 1), (0, 7, 2, 1),
                 (0, 8, 0, 0), (0, 9, 0, 0)]:
        autotune.apply(eng, cand)
        l0 = eng.launches()
        got[cand] = eng.compute_likelihood(ops, a, b, length)
        launches[cand] = eng.launches() - l0
        parts[cand] = [eng.partial(sl)[0].copy() for sl in check]
        assert rel(got[cand], want) < LNL_RTOL, (cand, got[cand], want)
    print("lnL", got, "rel err", {k: rel(v, want) for k, v in got.items()}, "launches per evaluation", launches)
    assert launches[(0, 4, 0, 0)] > launches[(0, 0, 2, 1)]  # one launch per wide level on top of the tail
    ref = parts[(0, 1, 2, 1)]
    for cand, pl in parts.items():
        for x, y in zip(pl, ref):
            np.testing.assert_array_equal(x, y, err_msg=str(cand))
    base = got[(0, 1, 2, 1)]
    assert all(rel(v, base) < 3e-7 for v in got.values()), got
    for cand in [(0, 4, 0, 0), (0, 8, 0, 0), (0, 9, 0, 0)]:
        autotune.apply(eng, cand)
        again = [eng.compute_likelihood(ops, a, b, length) for _ in range(3)]
        assert again == [got[cand]] * 3, cand
    assert launches[(0, 9, 0, 0)] == launches[(0, 8, 0, 0)] + 1  # one per-tile launch beside the CUDA-core epilogue


@pytest.mark.parametrize("kind", ["codon", "protein"])
def test_tc_dataflow_schedule(oracle_mod, kind):
    """Schedules 6 and 7 (one persistent launch of (tile, op, category) items,
    or of whole (tile, op) items, each waiting for the items writing its
    children): partials, exponents and lnL bit-identical to the level schedule
    of category-split items (same per-item arithmetic) where both put every op
    on the tensor cores, deterministic over repeated runs, and the lnL within 1e-6 of
    the FP64 oracle; also on a partial traversal (the ops below one internal
    branch after a length change, so some children come from earlier
    traversals). Protein 100 x 20,000: more (op, tile) pairs than one launch's
    counters hold, so the ops run in several windows."""
    ds = (simulate.codon_gy94_dataset(40, 3000, 36) if kind == "codon"
          else simulate.protein_lg_dataset(100, 20000, 35))
    topo = Topology(ds.edges, ds.lengths, ds.patterns.shape[0])
    leaf, nb = 0, topo.adj[0][0][0]
    ops_l = topo.branch_ops(nb, leaf)
    ops = engine.Engine.ops_array(ops_l)
    a, b, length = topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb)
    want = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths).lnl_branch(nb, leaf)
    eng = _engine(ds, topo)
    res = {}
    for cand in [(0, 5, 2, 1), (0, 6, 2, 1), (0, 6, 3, 1), (0, 7, 2, 1)] + ([(0, 6, 2, 4)] if kind == "codon" else []):
        autotune.apply(eng, cand)
        l0 = eng.launches()
        lnl = [eng.compute_likelihood(ops, a, b, length) for _ in range(3)]
        nl = (eng.launches() - l0) // 3
        assert lnl == [lnl[0]] * 3, (cand, lnl)
        res[cand] = (lnl[0], nl, [(eng.partial(op[0])[0], eng.exponent(op[0])) for op in ops_l[::7]])
        assert rel(lnl[0], want) < LNL_RTOL, (cand, lnl[0], want)
    print({c: (v[0], v[1]) for c, v in res.items()}, "oracle", want)
    ref = res[(0, 5, 2, 1)]
    if kind == "codon":  # every op on the tensor cores in every schedule: same per-item arithmetic
        for cand in [(0, 6, 2, 1), (0, 6, 3, 1), (0, 7, 2, 1), (0, 6, 2, 4)]:
            assert res[cand][0] == ref[0], cand
            for (p1, e1), (p2, e2) in zip(res[cand][2], ref[2]):
                np.testing.assert_array_equal(p1, p2)
                np.testing.assert_array_equal(e1, e2)
        assert res[(0, 6, 2, 1)][1] < ref[1]  # fewer launches than one per level
    else:  # schedule 5 puts the narrowest levels on other kernels: agreement to rounding
        assert abs(res[(0, 6, 2, 1)][0] - ref[0]) <= 3e-7 * abs(ref[0])
        assert res[(0, 7, 2, 1)][0] == res[(0, 6, 2, 1)][0]  # both dataflow forms: every op on the tensor cores
    # the tree driver on schedule 6: after a length change only the stale
    # partials are recomputed (children from earlier traversals, tip-tip ops
    # inside the dataflow launch), then branch-length optimisation
    t = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, precision=engine.TF32X3)
    autotune.apply(t.engine, (0, 6, 2, 1) if kind == "codon" else (0, 7, 2, 1))
    o = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
    assert rel(t.compute_likelihood(), o.compute_likelihood()) < LNL_RTOL
    lens = ds.lengths.copy()
    internal = [i for i, (u, v) in enumerate(ds.edges) if min(u, v) >= ds.ntaxa]
    for i in internal[::3]:
        lens[i] *= 1.7
    t.set_lengths(lens)
    o.set_lengths(lens)
    lg, lo = t.compute_likelihood(), o.compute_likelihood()
    assert rel(lg, lo) < LNL_RTOL, (lg, lo)
    if kind == "codon":
        n1, n2 = (int(x) for x in ds.edges[internal[0]])
        t.optimize_one_branch(n1, n2)
        o.optimize_one_branch(n1, n2)
        np.testing.assert_allclose(t.lengths(), o.lengths(), atol=1e-4)
        assert rel(t.compute_likelihood(), o.compute_likelihood()) < LNL_RTOL


def test_tc_deep_tree_exponents(oracle_mod):
    """200-taxon protein tree with long branches: the per-pattern exponents are
    exercised on the tensor-core path."""
    ds = simulate.protein_lg_dataset(200, 300, 33, mean_bl=0.3)
    t = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, precision=engine.TF32X3)
    o = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
    assert rel(t.compute_likelihood(), o.compute_likelihood()) < LNL_RTOL


def test_tc_ambiguous_states(oracle_mod):
    rng = np.random.default_rng(19)
    ds = simulate.protein_lg_dataset(14, 500, 34)
    pats = ds.patterns.copy()
    mask = rng.random(pats.shape) < 0.15
    pats[mask] = rng.integers(ds.model.nstates, ds.model.state_unknown + 1, size=mask.sum())
    t = engine.GpuTree(ds.model, pats, ds.freq, ds.edges, ds.lengths, precision=engine.TF32X3)
    o = oracle_mod.OracleTree(ds.model, pats, ds.freq, ds.edges, ds.lengths)
    assert rel(t.compute_likelihood(), o.compute_likelihood()) < LNL_RTOL


@pytest.mark.parametrize("kind", ["protein", "codon"])
def test_tc_full_size_configs(oracle_mod, kind):
    """Protein 100x50,000 and codon 40x10,000 on the tensor cores: lnL within
    1e-6 of the FP64 oracle."""
    ds = (simulate.protein_lg_dataset(100, 50000, 2) if kind == "protein"
          else simulate.codon_gy94_dataset(40, 10000, 3))
    t = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, precision=engine.TF32X3)
    o = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
    lg, lo = t.compute_likelihood(), o.compute_likelihood()
    err = rel(lg, lo)
    print(f"{kind}: split-TF32 lnL {lg:.6f} oracle {lo:.6f} rel err {err:.2e}")
    assert err < LNL_RTOL


# BF16 operands (one pass, FP32 accumulate): not a drop-in; the error is
# measured and bounded loosely (stated here): lnL within 1e-3 relative of the
# FP64 oracle, partials within 2e-2 of each pattern's largest entry.
BF16_LNL_RTOL = 1e-3


@pytest.mark.parametrize("name", ["prot12", "codon8"])
def test_bf16_golden_lnl_and_partials(oracle_mod, name):
    g = load_golden(name)
    t = engine.GpuTree(g.model, g.patterns, g.freq, g.edges, g.lengths, precision=engine.BF16)
    lnl = t.compute_likelihood()
    err = rel(lnl, g.lnl_std)
    print(f"{name}: bf16 lnL rel err {err:.2e}")
    assert err < BF16_LNL_RTOL
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    eng = _engine(g, topo, engine.BF16)
    assert eng.tensor_cores
    done, ops = set(), []
    for (u, v) in sorted(topo.slot):
        ops += topo.ops_for(u, v, done)
    eng.compute_partials(ops)
    orc = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths)
    n, C = g.model.nstates, g.model.ncat
    for (u, v), s in list(topo.slot.items())[:8]:
        gp, _ = eng.partial(s)
        op, _ = orc.partial(u, v)
        std = np.einsum("xi,pci->pcx", g.model.evec, op.reshape(-1, C, n)).reshape(op.shape)
        gn = gp / np.abs(gp).max(axis=1, keepdims=True)
        on = std / np.abs(std).max(axis=1, keepdims=True)
        assert np.max(np.abs(gn - on)) < 2e-2, (u, v)


@pytest.mark.parametrize("kind", ["protein", "codon"])
def test_bf16_schedules_agree(oracle_mod, kind):
    ds = (simulate.protein_lg_dataset(30, 900, 41) if kind == "protein"
          else simulate.codon_gy94_dataset(12, 500, 42))
    topo = Topology(ds.edges, ds.lengths, ds.patterns.shape[0])
    leaf, nb = 0, topo.adj[0][0][0]
    ops = engine.Engine.ops_array(topo.branch_ops(nb, leaf))
    a, b, length = topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb)
    want = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths).lnl_branch(nb, leaf)
    eng = _engine(ds, topo, engine.BF16)
    got = {}
    for cand in autotune.candidates(eng):
        autotune.apply(eng, cand)
        got[cand] = eng.compute_likelihood(ops, a, b, length)
    # codon: every schedule runs every op on the tensor cores, bit-identical.
    # protein: the dataflow schedules (6, 7) also run the narrow tail there (BF16
    # operands) where the others use FP32 CUDA cores: identical within each group
    groups = ([got] if kind == "codon" else
              [{c: v for c, v in got.items() if c[1] in (6, 7)}, {c: v for c, v in got.items() if c[1] not in (6, 7)}])
    for grp in groups:
        assert len(set(grp.values())) == 1, grp
    for v in set(got.values()):
        err = rel(v, want)
        print(f"{kind}: bf16 lnL rel err {err:.2e}")
        assert err < BF16_LNL_RTOL


@pytest.mark.parametrize("kind,ncat", [("protein", 1), ("protein", 3), ("protein", 8), ("codon", 1), ("codon", 3)])
def test_tc_category_counts_every_schedule(oracle_mod, kind, ncat):
    """Odd and single category counts on every tensor-core candidate (the
    accumulators alternate by category parity; category-split items with one
    category; the dataflow schedules): lnL within 1e-6 of the FP64 oracle,
    and every codon candidate bit-identical (every op on the tensor cores)."""
    import dataclasses
    from iqtree2_gb300 import models
    ds = (simulate.protein_lg_dataset(30, 900, 93) if kind == "protein" else simulate.codon_gy94_dataset(14, 400, 94))
    rates, props = models.gamma_rates_mean(0.6, ncat)
    m = dataclasses.replace(ds.model, rates=np.asarray(rates, np.float64), props=np.asarray(props, np.float64))
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    eng = engine.Engine(ds.nptn, m.nstates, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots,
                        precision=engine.TF32X3, max_ops=topo.nslots)
    eng.set_model(m)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    leaf, nb = 0, topo.adj[0][0][0]
    ops = engine.Engine.ops_array(topo.branch_ops(nb, leaf))
    a, b, length = topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb)
    want = oracle_mod.OracleTree(m, ds.patterns, ds.freq, ds.edges, ds.lengths).lnl_branch(nb, leaf)
    got = {}
    for cand in autotune.candidates(eng):
        autotune.apply(eng, cand)
        got[cand] = eng.compute_likelihood(ops, a, b, length)
        assert rel(got[cand], want) < LNL_RTOL, (cand, got[cand], want)
    if kind == "codon":
        assert len(set(got.values())) == 1, got


@pytest.mark.parametrize("ncat", [1, 3, 6])
def test_ring_kernel_category_counts(oracle_mod, ncat):
    """The deep-ring kernel (schedules 8 and 9) with 1, 3 and 6 categories on
    an alignment wide enough for its level launches (100 taxa x 20,000 sites):
    partials of levels 1-3 bit-identical to the level-synchronous kernel (same
    three MMA passes, same products and rescale), lnL within 1e-6 of the FP64
    oracle."""
    import dataclasses
    from iqtree2_gb300 import models
    ds = simulate.protein_lg_dataset(100, 20000, 95)
    rates, props = models.gamma_rates_mean(0.6, ncat)
    m = dataclasses.replace(ds.model, rates=np.asarray(rates, np.float64), props=np.asarray(props, np.float64))
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    eng = engine.Engine(ds.nptn, m.nstates, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots,
                        precision=engine.TF32X3, max_ops=topo.nslots)
    eng.set_model(m)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    leaf, nb = 0, topo.adj[0][0][0]
    ops_l = topo.branch_ops(nb, leaf)
    ops = engine.Engine.ops_array(ops_l)
    a, b, length = topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb)
    want = oracle_mod.OracleTree(m, ds.patterns, ds.freq, ds.edges, ds.lengths).lnl_branch(nb, leaf)
    lv = _levels(ops_l)
    check = [op[0] for op, l in zip(ops_l, lv) if 1 <= l <= 3]
    assert len(check) >= 20
    parts = {}
    for cand in [(0, 1, 2, 1), (0, 8, 0, 0), (0, 9, 0, 0)]:
        autotune.apply(eng, cand)
        lnl = eng.compute_likelihood(ops, a, b, length)
        assert rel(lnl, want) < LNL_RTOL, (cand, lnl, want)
        parts[cand] = [eng.partial(sl)[0].copy() for sl in check]
    for cand in [(0, 8, 0, 0), (0, 9, 0, 0)]:
        for x, y in zip(parts[cand], parts[(0, 1, 2, 1)]):
            np.testing.assert_array_equal(x, y, err_msg=str(cand))


def test_ring_per_tile_several_tiles_per_cta(oracle_mod):
    """Schedule 9's per-tile launch with more pattern tiles than SMs (about
    200 tiles: some CTAs take two through the one-op levels, each waiting on
    its own earlier items for the chained child): lnL within 3e-7 of schedule 8
    (the same levels on the CUDA-core tail) and within 1e-6 of the FP64
    oracle; then the tree driver on schedule 9 after a branch-length change,
    so the per-tile launch also meets children written by earlier
    traversals."""
    ds = simulate.protein_lg_dataset(100, 30000, 96)
    topo = Topology(ds.edges, ds.lengths, ds.patterns.shape[0])
    assert ds.nptn > 128 * 152  # more tiles than CTAs
    leaf, nb = 0, topo.adj[0][0][0]
    ops = engine.Engine.ops_array(topo.branch_ops(nb, leaf))
    a, b, length = topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb)
    want = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths).lnl_branch(nb, leaf)
    eng = _engine(ds, topo)
    got = {}
    for cand in [(0, 8, 0, 0), (0, 9, 0, 0)]:
        autotune.apply(eng, cand)
        got[cand] = [eng.compute_likelihood(ops, a, b, length) for _ in range(2)]
        assert got[cand][0] == got[cand][1], cand  # deterministic
        assert rel(got[cand][0], want) < LNL_RTOL, (cand, got[cand][0], want)
    assert rel(got[(0, 9, 0, 0)][0], got[(0, 8, 0, 0)][0]) < 3e-7
    t = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, precision=engine.TF32X3)
    autotune.apply(t.engine, (0, 9, 0, 0))
    o = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
    assert rel(t.compute_likelihood(), o.compute_likelihood()) < LNL_RTOL
    lens = ds.lengths.copy()
    internal = [i for i, (u, v) in enumerate(ds.edges) if min(u, v) >= ds.ntaxa]
    for i in internal[::5]:
        lens[i] *= 1.3
    t.set_lengths(lens)
    o.set_lengths(lens)
    assert rel(t.compute_likelihood(), o.compute_likelihood()) < LNL_RTOL
