"""Python side of the serving loop (``iqgpu_server_*`` in the C ABI).

``Server`` submits likelihood + branch-optimisation jobs to the engine's
continuous-batching scheduler, which admits them into one HBM arena as memory
and worker slots free up and runs admitted jobs concurrently on their own
CUDA streams. ``poisson_stream`` drives a seeded Poisson arrival process and
reports per-job latency (completion minus arrival).
"""
from __future__ import annotations

import ctypes as ct
import threading
import time

import numpy as np

from . import engine

_DP = ct.POINTER(ct.c_double)


class Job(ct.Structure):
    _fields_ = [("ntaxa", ct.c_int32), ("nptn", ct.c_int32), ("nstates", ct.c_int32), ("ncat", ct.c_int32),
                ("state_unknown", ct.c_int32), ("opt_iterations", ct.c_int32),
                ("eval", ct.c_void_p), ("evec", ct.c_void_p), ("inv_evec", ct.c_void_p), ("rates", ct.c_void_p),
                ("props", ct.c_void_p), ("state_freq", ct.c_void_p), ("tip_lh", ct.c_void_p),
                ("ptn_freq", ct.c_void_p), ("tip_states", ct.c_void_p), ("edges", ct.c_void_p),
                ("lengths", ct.c_void_p), ("tolerance", ct.c_double)]


class JobResult(ct.Structure):
    _fields_ = [("id", ct.c_int64), ("status", ct.c_int32), ("slots", ct.c_int32), ("lnl_initial", ct.c_double),
                ("lnl", ct.c_double), ("t_submit", ct.c_double), ("t_start", ct.c_double), ("t_end", ct.c_double),
                ("bytes", ct.c_int64), ("error", ct.c_char * 128)]


class ServerConfig(ct.Structure):
    _fields_ = [("device", ct.c_int32), ("precision_unused", ct.c_int32), ("max_active", ct.c_int32),
                ("pad", ct.c_int32), ("memory_budget", ct.c_uint64)]


class ServerStats(ct.Structure):
    _fields_ = [("submitted", ct.c_int64), ("admitted", ct.c_int64), ("refused", ct.c_int64),
                ("completed", ct.c_int64), ("peak_active", ct.c_int64), ("peak_bytes", ct.c_uint64),
                ("arena_bytes", ct.c_uint64)]


def _bind():
    L = engine.lib()
    vp = ct.c_void_p
    for name, args in {
        "iqgpu_server_create": [ct.POINTER(ServerConfig), ct.POINTER(vp)],
        "iqgpu_server_submit": [vp, ct.POINTER(Job), ct.c_int32, ct.POINTER(ct.c_int64)],
        "iqgpu_server_wait": [vp, ct.c_int64, ct.POINTER(JobResult), _DP],
        "iqgpu_server_get_stats": [vp, ct.POINTER(ServerStats)],
        "iqgpu_server_destroy": [vp],
    }.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ct.c_int
    return L


class Server:
    def __init__(self, max_active=16, memory_budget=0, device=0):
        self.L = _bind()
        cfg = ServerConfig(device, 0, int(max_active), 0, int(memory_budget))
        h = ct.c_void_p()
        engine._check(self.L.iqgpu_server_create(ct.byref(cfg), ct.byref(h)))
        self.h = h
        self._keep = {}

    def submit(self, ds, precision=engine.F32, opt_iterations=1, tolerance=1e-3):
        """Queue one job for dataset ``ds`` (a simulate.Dataset); returns the job id."""
        m = ds.model
        arrays = [np.ascontiguousarray(x, np.float64) for x in
                  (m.eval, m.evec, m.inv_evec, m.rates, m.props, m.pi, m.tip_lh, ds.freq, ds.lengths)]
        states = np.ascontiguousarray(ds.patterns, np.uint8)
        edges = np.ascontiguousarray(ds.edges, np.int32)
        j = Job(ds.ntaxa, ds.nptn, m.nstates, m.ncat, m.state_unknown, int(opt_iterations),
                *[a.ctypes.data for a in arrays[:8]], states.ctypes.data, edges.ctypes.data, arrays[8].ctypes.data,
                float(tolerance))
        jid = ct.c_int64()
        engine._check(self.L.iqgpu_server_submit(self.h, ct.byref(j), int(precision), ct.byref(jid)))
        return jid.value

    def wait(self, jid, nedge=None):
        r = JobResult()
        lengths = np.zeros(nedge) if nedge else None
        engine._check(self.L.iqgpu_server_wait(self.h, jid, ct.byref(r),
                                               lengths.ctypes.data_as(_DP) if lengths is not None else None))
        out = {k: getattr(r, k) for k in ("id", "status", "slots", "lnl_initial", "lnl", "t_submit", "t_start",
                                           "t_end", "bytes")}
        out["error"] = r.error.decode()
        if lengths is not None:
            out["lengths"] = lengths
        return out

    def stats(self):
        s = ServerStats()
        engine._check(self.L.iqgpu_server_get_stats(self.h, ct.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.L.iqgpu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_stream(server, jobs, rate, seed, precision=engine.F32, opt_iterations=1):
    """Submit ``jobs`` (datasets) at seeded Poisson arrival times (mean ``rate``/s);
    return per-job dicts with latency = completion - arrival (seconds)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(jobs))
    arrivals = np.cumsum(gaps)
    ids, t_arr = [], []
    t0 = time.perf_counter()
    for ds, ta in zip(jobs, arrivals):
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        t_arr.append(time.perf_counter())
        ids.append(server.submit(ds, precision=precision, opt_iterations=opt_iterations))
    results = []
    for jid, ds in zip(ids, jobs):
        r = server.wait(jid)
        # the server stamps submission (= arrival) and completion on its own clock
        r["latency"] = r["t_end"] - r["t_submit"]
        r["queue_wait"] = r["t_start"] - r["t_submit"]
        r["ntaxa"], r["nptn"], r["nstates"] = ds.ntaxa, ds.nptn, ds.model.nstates
        results.append(r)
    return results, time.perf_counter() - t0
