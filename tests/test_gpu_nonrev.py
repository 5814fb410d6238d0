"""Non-reversible models on the mixed-precision path against an FP64 numpy
pruning that exponentiates the rate matrix directly (scipy expm, no eigen
system): UNREST-style random rate matrices with complex eigenvalues.

Unrooted convention (tree/phylokernelnonrev.h:1117-1130): the evaluated
branch (dad, node) is weighted by the stationary frequencies on the dad
side, so the lnL depends on the branch and its orientation; every op's
children lie away from that branch and no matrix is transposed.

Rooted convention: a root leaf R hangs from the root node r. Branches carry
no frequencies; partials computed against the edge direction use P(t)^T and
the root leaf's rows are P(t)^T times the root frequencies (= the stationary
frequencies); tree/phylokernelnew.h:932-963. Every branch then gives the
same lnL, the rooted tree's.

Tolerances: mixed path lnL 1e-6 relative, first and second derivatives
1e-4 / 1e-3 relative with an absolute floor of 1e-5 per site; FP64 path
(standard-basis partials, U^-1 = I in the traversal, NORM and SAFE scaling)
lnL 1e-10 relative, derivatives 1e-8 relative with a floor of 1e-9 per site.
"""
import numpy as np
import pytest

import stdbasis
from helpers import rel
from iqtree2_gb300 import engine, models, simulate
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu


def _data(kind):
    if kind == "dna":
        return simulate.dna_gtr_dataset(14, 1500, 71), models.unrest_model(4, 73, 0.6)
    return simulate.protein_lg_dataset(12, 600, 73), models.unrest_model(20, 74, 0.8)


def _engine(ds, m, topo, precision, safe=False):
    return engine.Engine(ds.patterns.shape[1], m.nstates, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots,
                         precision=precision, safe=safe)


def _tol(precision):
    return 1e-10 if precision == engine.F64 else 1e-6


def _internal_branches(topo, ds):
    return [(int(u), int(v)) for (u, v) in ds.edges if u >= ds.ntaxa and v >= ds.ntaxa]


CASES = [("dna", engine.F32, False), ("protein", engine.F32, False), ("protein", engine.TF32X3, False),
         ("dna", engine.F64, False), ("protein", engine.F64, True)]


@pytest.mark.parametrize("kind,precision,safe", CASES)
def test_nonrev_unrooted_lnl(kind, precision, safe):
    ds, m = _data(kind)
    assert np.abs(m.ceval.imag).max() > 1e-3  # complex eigenvalues: the complex path is exercised
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    e = _engine(ds, m, topo, precision, safe)
    try:
        e.set_model(m)
        e.set_patterns(ds.freq)
        e.set_tip_states(ds.patterns)
        branches = _internal_branches(topo, ds)[:3] + [(int(ds.edges[0][1]), int(ds.edges[0][0]))]
        values = []
        for (u, v) in branches:
            for (dad, node) in ((u, v), (v, u)):
                if dad < ds.ntaxa:
                    continue
                ops = e.ops_array(topo.branch_ops(node, dad))
                lg = e.compute_likelihood(ops, topo.ref(node, dad), topo.ref(dad, node), topo.edge_len(dad, node))
                lo = stdbasis.branch_lnl_nonrev(m, ds.patterns, ds.freq, ds.edges, ds.lengths, ds.ntaxa, dad, node)
                assert rel(lg, lo) < _tol(precision), (dad, node, lg, lo)
                values.append(lo)
        assert max(values) - min(values) > 1e-6 * abs(values[0])  # not root-invariant: the convention matters
    finally:
        e.close()


def _rooted_ops(topo, ds, parent, R, dad, node):
    """Post-order ops for partial dad->node with the rooted flags: a child that
    is the node's parent is reached against the edge direction (TRANSPOSE); the
    root leaf R also gets ROOTLEAF."""
    ops, done = [], set()

    def rec(d, n):
        if n < ds.ntaxa or (d, n) in done:
            return
        kids = [(c, k) for (c, k) in topo.adj[n] if c != d]
        for (c, _) in kids:
            rec(n, c)
        flags = 0
        for j, (c, _) in enumerate(kids):
            if parent.get(n) == c:
                flags |= engine.OP_TRANSPOSE0 << j
            if c == R:
                flags |= engine.OP_ROOTLEAF0 << j
        (c0, k0), (c1, k1) = kids
        ops.append((topo.slot[(d, n)], topo.ref(n, c0), topo.ref(n, c1), topo.lengths[k0], topo.lengths[k1], flags))
        done.add((d, n))

    rec(dad, node)
    return ops


@pytest.mark.parametrize("kind,precision,safe", CASES)
def test_nonrev_rooted_every_branch(kind, precision, safe):
    ds, m = _data(kind)
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    R = ds.ntaxa - 1                 # the root leaf
    r = topo.adj[R][0][0]            # the root
    parent = {r: R}
    stack = [r]
    while stack:                     # edge directions away from the root
        n = stack.pop()
        for (c, _) in topo.adj[n]:
            if c != parent.get(n) and c >= ds.ntaxa:
                parent[c] = n
                stack.append(c)
            elif c != parent.get(n):
                parent[c] = n
    pat = ds.patterns.copy()
    pat[R, :] = m.state_unknown      # the root leaf carries no data
    # the rooted tree's lnL: frequencies at the root, no data at R
    l_root = stdbasis.branch_lnl_nonrev(m, pat, ds.freq, ds.edges, ds.lengths, ds.ntaxa, r, R)
    e = _engine(ds, m, topo, precision, safe)
    try:
        e.set_model_nonrev(m, rooted=True)
        e.set_patterns(ds.freq)
        e.set_tip_states(ds.patterns)
        checked = 0
        for (u, v) in _internal_branches(topo, ds)[:4]:
            dad, node = (u, v) if parent.get(v) == u else (v, u)  # dad is the upper end
            ops = e.ops_array(_rooted_ops(topo, ds, parent, R, node, dad) +
                              _rooted_ops(topo, ds, parent, R, dad, node))
            lg = e.compute_likelihood(ops, topo.ref(node, dad), topo.ref(dad, node), topo.edge_len(dad, node))
            assert rel(lg, l_root) < _tol(precision), (dad, node, lg, l_root)
            checked += 1
        assert checked >= 3
    finally:
        e.close()


@pytest.mark.parametrize("kind,precision,safe", CASES)
def test_nonrev_derivatives_and_from_buffer(kind, precision, safe):
    ds, m = _data(kind)
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    e = _engine(ds, m, topo, precision, safe)
    f64 = precision == engine.F64
    r1, r2, floor = (1e-8, 1e-8, 1e-9) if f64 else (1e-4, 1e-3, 1e-5)
    try:
        e.set_model(m)
        e.set_patterns(ds.freq)
        e.set_tip_states(ds.patterns)
        nsite = float(ds.freq.sum())
        for (dad, node) in _internal_branches(topo, ds)[:2] + [(int(ds.edges[0][1]), int(ds.edges[0][0]))]:
            if dad < ds.ntaxa:
                dad, node = node, dad
            ops = e.ops_array(topo.branch_ops(node, dad))
            a, b = topo.ref(node, dad), topo.ref(dad, node)
            for t in (topo.edge_len(dad, node), 0.02, 0.4):
                df, ddf = e.likelihood_derv(ops, a, b, t)
                lo, d1, d2 = stdbasis.branch_lnl_nonrev(m, ds.patterns, ds.freq, ds.edges, ds.lengths, ds.ntaxa,
                                                        dad, node, blen=t, derivatives=True)
                assert abs(df - d1) < r1 * abs(d1) + floor * nsite, (t, df, d1)
                assert abs(ddf - d2) < r2 * abs(d2) + floor * nsite, (t, ddf, d2)
                lb = e.lnl_from_buffer(t)
                assert rel(lb, lo) < _tol(precision), (t, lb, lo)
    finally:
        e.close()


def test_nonrev_refusals():
    ds, m = _data("dna")
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    e = _engine(ds, m, topo, engine.F32)
    try:
        e.set_model(m)
        with pytest.raises(engine.EngineError, match="ASC"):
            e.set_asc(2, 100.0)
        # flags need a non-reversible model
        e.set_model(ds.model)
        e.set_patterns(ds.freq)
        e.set_tip_states(ds.patterns)
        u, v = _internal_branches(topo, ds)[0]
        ops = topo.branch_ops(v, u)
        ops[0] = ops[0] + (engine.OP_TRANSPOSE0,)
        with pytest.raises(engine.EngineError, match="flags"):
            e.compute_likelihood(e.ops_array(ops), topo.ref(v, u), topo.ref(u, v), topo.edge_len(u, v))
    finally:
        e.close()
