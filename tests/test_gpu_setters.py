"""Setters copy the caller's arrays before they return.

iqgpu_set_patterns / set_model / set_state_freq / set_tip_partials queue
their copies in stream order, so the data goes through engine-owned staging
first, or, from a page-locked buffer of 16 KB or more, is copied from where it
is and the setter waits for that copy: a caller may overwrite or free its
buffer as soon as the setter returns, pinned memory included (IQ-TREE
reweights ptn_freq in place for every bootstrap replicate). The test keeps
the stream busy with a traversal, passes pinned buffers, overwrites them at
once and checks the likelihood against the undisturbed value.
"""
import numpy as np
import pytest

from helpers import rel
from iqtree2_gb300 import engine, simulate
from iqtree2_gb300.engine import _check, _dp, lib
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu


def _pinned(a):
    torch = pytest.importorskip("torch")
    t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    return t, t.numpy()


def test_pinned_inputs_can_be_overwritten_after_the_setter_returns():
    ds = simulate.protein_lg_dataset(60, 8000, 21)
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    m = ds.model
    eng = engine.Engine(ds.nptn, m.nstates, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots, max_ops=topo.nslots)
    eng.set_model(m)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    leaf = 0
    u0, v0 = next((int(u), int(v)) for (u, v) in ds.edges if leaf in (int(u), int(v)))
    nb = u0 + v0 - leaf
    ops = topo.branch_ops(nb, leaf)
    a, b, length = topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb)
    want = eng.compute_likelihood(ops, a, b, length)

    keep_f, freq = _pinned(ds.freq.astype(np.float64))
    keep_e, ev = _pinned(m.eval.astype(np.float64))
    for _ in range(3):
        eng.compute_partials(topo.all_partials_ops())  # the stream is busy when the copies are queued
        eng.set_patterns(freq)
        freq[:] = 0.0                                   # overwritten before the copy could have run
        arrs = [np.ascontiguousarray(x, np.float64) for x in (m.evec, m.inv_evec, m.rates, m.props)]
        _check(lib().iqgpu_set_model(eng.h, _dp(ev), *[_dp(x) for x in arrs]))
        ev[:] = np.nan
        got = eng.compute_likelihood(ops, a, b, length)
        assert rel(got, want) < 1e-12, (got, want)
        freq[:] = ds.freq
        ev[:] = m.eval
