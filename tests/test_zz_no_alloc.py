"""The allocation-free derivative entry point (iqgpu_derv_noalloc).

It serves callers that may not allocate device memory where they need a
branch-length derivative; it keeps its reduction scratch in a static device
array and takes all buffers from the caller. Here the caller's buffers are
torch tensors (the test allocates; the entry point does not), filled with the
theta buffer of one branch, and the entry point's {df, ddf} must equal what
the engine's own iqgpu_likelihood_derv returns for that branch, within the
derivative tolerance of the other GPU tests (1e-9 relative), on two calls in a
row at different branch lengths.
"""
import ctypes as ct

import numpy as np
import pytest

from helpers import load_golden
from iqtree2_gb300 import engine
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu

LOG_SCALING_THRESHOLD = -177.4456782233459932741


def test_noalloc_derivative_matches_engine(oracle_mod):
    torch = pytest.importorskip("torch")
    g = load_golden("prot12")
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    n1, n2 = next(tuple(map(int, e)) for e in g.edges if min(e) >= g.ntaxa)
    node, dad = n2, n1
    m = g.model
    nptn = g.patterns.shape[1]

    # existing entry point: the engine builds theta itself
    eng = engine.Engine(nptn, m.nstates, m.ncat, g.ntaxa, m.state_unknown, topo.nslots, max_ops=topo.nslots)
    eng.set_model(m)
    eng.set_patterns(g.freq)
    eng.set_tip_states(g.patterns)
    ops = topo.branch_ops(node, dad)
    a, b = topo.ref(dad, node), topo.ref(node, dad)
    lengths = (0.03, 0.4)
    want = [eng.likelihood_derv(ops, a, b, lengths[0]),
            eng.likelihood_derv([], a, b, lengths[1], theta_computed=True)]
    want_lnl = [eng.lnl_from_buffer(length) for length in lengths]  # lnL at each length, same theta

    # the caller's own buffers: theta = node o dad in eigen space, NORM scale offset
    orc = oracle_mod.OracleTree(m, g.patterns, g.freq, g.edges, g.lengths)
    pa, sa = orc.partial(dad, node)
    pb, sb = orc.partial(node, dad)
    theta = np.ascontiguousarray((pa * pb).T)  # [B][nptn]
    bscale = (sa[:, 0].astype(np.float64) + sb[:, 0]) * LOG_SCALING_THRESHOLD
    dev = torch.device("cuda:0")
    t_theta = torch.from_numpy(theta).to(dev)
    t_bscale = torch.from_numpy(bscale).to(dev)
    t_freq = torch.from_numpy(np.ascontiguousarray(g.freq)).to(dev)
    t_invar = torch.zeros(nptn, dtype=torch.float64, device=dev)
    t_out = torch.zeros(3, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    ev, rv, pv = (np.ascontiguousarray(x, np.float64) for x in (m.eval, m.rates, m.props))
    dp = ct.POINTER(ct.c_double)
    for k, length in enumerate(lengths):
        t_out.zero_()
        rc = engine.lib().iqgpu_derv_noalloc(
            ct.c_void_p(t_theta.data_ptr()), ct.c_void_p(t_bscale.data_ptr()), ct.c_void_p(t_freq.data_ptr()),
            ct.c_void_p(t_invar.data_ptr()), nptn, nptn, m.nstates, m.ncat, ev.ctypes.data_as(dp),
            rv.ctypes.data_as(dp), pv.ctypes.data_as(dp), length, ct.c_void_p(t_out.data_ptr()),
            ct.c_void_p(stream.cuda_stream))
        assert rc == 0, engine.lib().iqgpu_last_error()
        df, ddf, lnl = t_out.cpu().numpy()
        wdf, wddf = want[k]
        assert abs(df - wdf) <= 1e-9 * max(1.0, abs(wdf))
        assert abs(ddf - wddf) <= 1e-9 * max(1.0, abs(wddf))
        assert abs(lnl - want_lnl[k]) <= 1e-9 * abs(want_lnl[k])


def test_noalloc_rejects_oversized_input():
    dp = ct.POINTER(ct.c_double)
    one = np.ones(64)
    dummy = ct.c_void_p(16)  # never dereferenced: the size check comes first
    rc = engine.lib().iqgpu_derv_noalloc(dummy, dummy, dummy, dummy, 524289, 524289, 4, 4,
                                         one.ctypes.data_as(dp), one.ctypes.data_as(dp), one.ctypes.data_as(dp),
                                         0.1, dummy, None)
    assert rc == 1
    assert b"524288" in engine.lib().iqgpu_last_error()
