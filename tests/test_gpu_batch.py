"""Batched evaluation: NNI candidates in one graph-captured launch sequence and
UFBoot RELL scores, against the FP64 oracle and numpy.

Tolerances: NNI candidate lnL relative <= 1e-6 and optimised central branch
within 1e-4 of the oracle's optimizeOneBranch (mixed-precision path); RELL
scores relative <= 1e-6 of an FP64 numpy product.
"""
import numpy as np
import pytest

from helpers import rel
from iqtree2_gb300 import engine, simulate
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu


def nni_candidates(topo, nmax):
    return topo.nni_candidates(nmax)


def swapped_edges(ds, u, v, x, y):
    """Edge list after moving subtree x from u to v and subtree y from v to u."""
    edges = ds.edges.copy()
    for k, (p, q) in enumerate(edges):
        if {int(p), int(q)} == {u, x}:
            edges[k] = (v, x)
        elif {int(p), int(q)} == {v, y}:
            edges[k] = (u, y)
    return edges


def test_nni_batch_matches_oracle(oracle_mod):
    ds = simulate.dna_gtr_dataset(24, 3000, 41)
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    cands = nni_candidates(topo, 16)
    ncand = len(cands)
    nslots = topo.nslots + 2 * ncand
    eng = engine.Engine(ds.nptn, 4, 4, ds.ntaxa, 18, nslots, precision=engine.F32, max_ops=max(nslots, 2 * ncand))
    eng.set_model(ds.model)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    eng.compute_partials(topo.all_partials_ops())
    arr = topo.nni_batch_entries(cands, topo.nslots)
    lnl, blen = eng.nni_batch(arr, max_nr_step=10, min_bl=1e-6, max_bl=10.0)
    for k, c in enumerate(cands):
        u, v = c["u"], c["v"]
        x = c["n2"][0]  # moved from u to v
        y = c["n1"][1]  # moved from v to u
        edges = swapped_edges(ds, u, v, x, y)
        o = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, edges, ds.lengths)
        assert o.optimize_one_branch(u, v, 10) == 0
        ol = o.compute_likelihood()
        ob = o.lengths()[[i for i, (p, q) in enumerate(edges) if {int(p), int(q)} == {u, v}][0]]
        assert rel(lnl[k], ol) < 1e-6, (k, lnl[k], ol)
        assert abs(blen[k] - ob) < 1e-4, (k, blen[k], ob)


def test_rell_matches_numpy():
    ds = simulate.dna_gtr_dataset(10, 5000, 43)
    rng = np.random.default_rng(3)
    w = simulate.bootstrap_weights(ds.freq, 200, rng)
    eng = engine.Engine(ds.nptn, 4, 4, ds.ntaxa, 18, 24, precision=engine.F32, max_ops=24)
    eng.set_model(ds.model)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    plh = -rng.uniform(2.0, 30.0, size=(70, ds.nptn))
    eng.set_boot_weights(w)
    got = eng.rell(plh)
    want = plh @ w.astype(np.float64).T
    assert got.shape == (70, 200)
    assert np.max(np.abs(got - want) / np.abs(want)) < 1e-6


def test_rell_current_tree_on_device(oracle_mod):
    """RELL of the last evaluated tree from its device-resident pattern lnL
    equals the host-input path on the same vector; 1,000 replicates."""
    ds = simulate.dna_gtr_dataset(16, 20000, 44)
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    eng = engine.Engine(ds.nptn, 4, 4, ds.ntaxa, 18, topo.nslots, precision=engine.F32, max_ops=topo.nslots)
    eng.set_model(ds.model)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    leaf, nb = 0, topo.adj[0][0][0]
    eng.compute_likelihood(topo.branch_ops(nb, leaf), topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb))
    w = simulate.bootstrap_weights(ds.freq, 1000, np.random.default_rng(8))
    eng.set_boot_weights(w)
    cur = eng.rell_current()
    plh = eng.pattern_lh()
    host = eng.rell(plh[None, :])[0]
    want = w.astype(np.float64) @ plh
    assert cur.shape == (1000,)
    np.testing.assert_array_equal(cur, host)
    assert np.max(np.abs(cur - want) / np.abs(want)) < 1e-6


@pytest.mark.parametrize("precision", [engine.F32, engine.F64])
def test_partition_group_one_graph(oracle_mod, precision):
    """12 uneven DNA partitions with separate GTR+G4 on one tree, evaluated by
    one graph launch: each partition's lnL equals the same engine evaluated
    alone (bit for bit: same kernels) and the oracle's (1e-6 relative mixed,
    1e-10 FP64); new branch lengths through set_lengths as well."""
    from iqtree2_gb300 import simulate
    sizes = [2000, 3000, 5000, 800, 12000, 7000, 2500, 1500, 9000, 4000, 6000, 30000]
    parts = simulate.partitioned_dna_datasets(24, sizes, 61)
    ds0 = parts[0]
    topo = Topology(ds0.edges, ds0.lengths, ds0.ntaxa)
    leaf, nb = 0, topo.adj[0][0][0]
    ops = topo.branch_ops(nb, leaf)
    a, b, length = topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb)
    engs = []
    for ds in parts:
        e = engine.Engine(ds.nptn, 4, ds.model.ncat, ds.ntaxa, ds.model.state_unknown, topo.nslots,
                          precision=precision, max_ops=topo.nslots)
        e.set_model(ds.model)
        e.set_patterns(ds.freq)
        e.set_tip_states(ds.patterns)
        engs.append(e)
    alone = [e.compute_likelihood(ops, a, b, length) for e in engs]
    grp = engine.Group(engs)
    grp.prepare([ops] * len(engs), [a] * len(engs), [b] * len(engs), [length] * len(engs))
    tot, per = grp.lnl()
    tot2, per2 = grp.lnl()  # replay
    assert list(per) == alone and list(per2) == alone
    assert tot == pytest.approx(sum(alone), rel=1e-14)
    tol = 1e-6 if precision == engine.F32 else 1e-10
    for ds, v in zip(parts, per):
        want = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths).lnl_branch(nb, leaf)
        assert rel(v, want) < tol
    # all branch lengths scaled by 1.3: same traversals, new lengths
    ops2 = [(d, c0, c1, 1.3 * l0, 1.3 * l1) for (d, c0, c1, l0, l1) in ops]
    grp.set_lengths([ops2] * len(engs), [1.3 * length] * len(engs))
    _, per3 = grp.lnl()
    for e, v in zip(engs, per3):
        assert v == e.compute_likelihood(ops2, a, b, 1.3 * length)
    grp.close()
