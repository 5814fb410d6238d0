"""Python binding of the GB300 likelihood engine (``libiqgpu.so``, C ABI).

There is no CPU fallback: if the in-tree library cannot be loaded, or the
device is not a GB300 (sm_103), every call raises.

``Engine`` mirrors the reference's kernel function pointers
(tree/phylotreesse.cpp:91-236) and ``GpuTree`` the PhyloTree drivers around
them (computeLikelihood, optimizeOneBranch, optimizeAllBranches).
"""
from __future__ import annotations

import ctypes as ct
import os

import numpy as np

from . import build as _build

F64, F32, TF32X3, BF16 = 0, 1, 2, 3

_lib = None


class EngineError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"iqgpu error {code}: {msg}")
        self.code = code


class Config(ct.Structure):
    _fields_ = [("nptn", ct.c_int32), ("nstates", ct.c_int32), ("ncat", ct.c_int32), ("ntaxa", ct.c_int32),
                ("state_unknown", ct.c_int32), ("nslots", ct.c_int32), ("safe", ct.c_int32),
                ("precision", ct.c_int32), ("device", ct.c_int32), ("max_ops", ct.c_int32),
                ("flags", ct.c_int32)]


FLAG_REF_TRIPLE_TAIL = 1
# take cfg.safe as given instead of the reference's SAFE rule (SAFE for
# nstates not in {4, 20} and for 2000 taxa or more, tree/phylotreesse.cpp:95-96)
FLAG_SAFE_AS_GIVEN = 2


class Op(ct.Structure):
    _fields_ = [("dad_slot", ct.c_int32), ("child", ct.c_int32 * 2), ("flags", ct.c_int32),
                ("len", ct.c_double * 2)]


# iqgpu_op flags (non-reversible models): transpose P for a child reached
# against the edge direction; a tip child that is the root leaf
OP_TRANSPOSE0, OP_TRANSPOSE1, OP_ROOTLEAF0, OP_ROOTLEAF1 = 1, 2, 4, 8
# multifurcating nodes: records of one node after the first carry on its
# child list (OP_MORE on every record but the last; NO_CHILD pads an odd count)
OP_MORE = 16
NO_CHILD = -(2 ** 31)
OP_DTYPE = np.dtype([("dad_slot", np.int32), ("child", np.int32, (2,)), ("flags", np.int32),
                     ("len", np.float64, (2,))])
assert OP_DTYPE.itemsize == ct.sizeof(Op) == 32
NNI_DTYPE = np.dtype([("sub", np.int32, (4,)), ("scratch", np.int32, (2,)), ("len", np.float64, (4,)),
                      ("central", np.float64)])
assert NNI_DTYPE.itemsize == 64

_DP = ct.POINTER(ct.c_double)
_U8P = ct.POINTER(ct.c_uint8)
_I32P = ct.POINTER(ct.c_int32)


def library_path():
    return _build.LIB


def lib():
    """Load the in-tree engine library (built on demand if nvcc is present)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        _build.build()
    L = ct.CDLL(path)
    vp = ct.c_void_p
    sig = {
        "iqgpu_last_error": ([], ct.c_char_p),
        "iqgpu_memory_required": ([ct.POINTER(Config), ct.POINTER(ct.c_size_t)], ct.c_int),
        "iqgpu_create": ([ct.POINTER(Config), ct.POINTER(vp)], ct.c_int),
        "iqgpu_destroy": ([vp], ct.c_int),
        "iqgpu_get_config": ([vp, ct.POINTER(Config)], ct.c_int),
        "iqgpu_set_model": ([vp, _DP, _DP, _DP, _DP, _DP], ct.c_int),
        "iqgpu_set_tip_partials": ([vp, _DP], ct.c_int),
        "iqgpu_set_state_freq": ([vp, _DP], ct.c_int),
        "iqgpu_set_patterns": ([vp, _DP, _DP], ct.c_int),
        "iqgpu_set_tip_states": ([vp, _U8P], ct.c_int),
        "iqgpu_compute_partials": ([vp, vp, ct.c_int32], ct.c_int),
        "iqgpu_branch_lnl": ([vp, ct.c_int32, ct.c_int32, ct.c_double, _DP], ct.c_int),
        "iqgpu_compute_likelihood": ([vp, vp, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_double, _DP], ct.c_int),
        "iqgpu_likelihood_derv": ([vp, vp, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_double, ct.c_int32, _DP, _DP],
                                  ct.c_int),
        "iqgpu_lnl_from_buffer": ([vp, ct.c_double, _DP], ct.c_int),
        "iqgpu_newton_supported": ([vp, _I32P], ct.c_int),
        "iqgpu_newton_branch": ([vp, vp, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_double, ct.c_double,
                                 ct.c_double, ct.c_double, ct.c_int32, _DP, _DP, _DP, _I32P], ct.c_int),
        "iqgpu_get_pattern_lh": ([vp, _DP], ct.c_int),
        "iqgpu_get_partial": ([vp, ct.c_int32, _DP, _U8P], ct.c_int),
        "iqgpu_get_exponent": ([vp, ct.c_int32, _I32P], ct.c_int),
        "iqgpu_sync": ([vp], ct.c_int),
        "iqgpu_set_stream": ([vp, vp], ct.c_int),
        "iqgpu_set_timing": ([vp, ct.c_int32], ct.c_int),
        "iqgpu_get_timing": ([vp, _DP, ct.POINTER(ct.c_int64)], ct.c_int),
        "iqgpu_set_tile": ([vp, ct.c_int32], ct.c_int),
        "iqgpu_set_schedule": ([vp, ct.c_int32], ct.c_int),
        "iqgpu_set_asc": ([vp, ct.c_int32, ct.c_double], ct.c_int),
        "iqgpu_set_mixture": ([vp, ct.c_int32] + [ct.c_void_p] * 7, ct.c_int),
        "iqgpu_set_model_nonrev": ([vp] + [ct.c_void_p] * 10, ct.c_int),
        "iqgpu_set_asc_holder": ([vp, ct.c_int32], ct.c_int),
        "iqgpu_set_stages": ([vp, ct.c_int32], ct.c_int),
        "iqgpu_set_wait_limit": ([vp, ct.c_uint32], ct.c_int),
        "iqgpu_group_create": ([ct.c_void_p, ct.c_int32, ct.POINTER(ct.c_void_p)], ct.c_int),
        "iqgpu_group_prepare": ([vp, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p], ct.c_int),
        "iqgpu_group_set_lengths": ([vp, ct.c_void_p, ct.c_void_p], ct.c_int),
        "iqgpu_group_lnl": ([vp, ct.c_void_p, ct.c_void_p], ct.c_int),
        "iqgpu_group_destroy": ([vp], ct.c_int),
        "iqgpu_set_kpieces": ([vp, ct.c_int32], ct.c_int),
        "iqgpu_get_launches": ([vp, ct.POINTER(ct.c_int64)], ct.c_int),
        "iqgpu_rell_current": ([vp, ct.c_void_p], ct.c_int),
        "iqgpu_derv_noalloc": ([vp, vp, vp, vp, ct.c_int32, ct.c_int64, ct.c_int32, ct.c_int32, _DP, _DP, _DP,
                                ct.c_double, vp, vp], ct.c_int),
        "iqgpu_nni_batch": ([vp, vp, ct.c_int32, ct.c_int32, ct.c_double, ct.c_double, _DP, _DP], ct.c_int),
        "iqgpu_set_boot_weights": ([vp, ct.POINTER(ct.c_float), ct.c_int32], ct.c_int),
        "iqgpu_rell": ([vp, _DP, ct.c_int32, _DP], ct.c_int),
        "iqgpu_tree_create": ([vp, _I32P, _DP, ct.POINTER(vp)], ct.c_int),
        "iqgpu_tree_create_n": ([vp, ct.c_int32, _I32P, _DP, ct.POINTER(vp)], ct.c_int),
        "iqgpu_tree_destroy": ([vp], ct.c_int),
        "iqgpu_tree_compute_likelihood": ([vp, _DP, _DP], ct.c_int),
        "iqgpu_tree_optimize_one_branch": ([vp, ct.c_int32, ct.c_int32, ct.c_int32], ct.c_int),
        "iqgpu_tree_optimize_all_branches": ([vp, ct.c_int32, ct.c_double, ct.c_int32, _DP], ct.c_int),
        "iqgpu_tree_get_lengths": ([vp, _DP], ct.c_int),
        "iqgpu_tree_set_lengths": ([vp, _DP], ct.c_int),
        "iqgpu_tree_set_bounds": ([vp, ct.c_double, ct.c_double], ct.c_int),
        "iqgpu_tree_num_updates": ([vp, ct.POINTER(ct.c_int64)], ct.c_int),
        "iqgpu_tree_set_device_newton": ([vp, ct.c_int32], ct.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def exported_symbols():
    """Names the header declares (checked by the CPU tests)."""
    hdr = os.path.join(_build.ROOT, "include", "iqgpu.h")
    import re
    names = re.findall(r"^\s*(?:int|const char \*)\s*\*?\s*(iqgpu_\w+)\s*\(", open(hdr).read(), re.M)
    return sorted(set(names))


def _check(rc):
    if rc != 0:
        raise EngineError(rc, lib().iqgpu_last_error().decode())


def _dp(a):
    return a.ctypes.data_as(_DP)


class Engine:
    """One engine = one HBM workspace and one CUDA stream (a PhyloTree's buffers)."""

    def __init__(self, nptn, nstates, ncat, ntaxa, state_unknown, nslots, safe=False, precision=F64,
                 device=0, max_ops=None, flags=0):
        self.cfg = Config(int(nptn), int(nstates), int(ncat), int(ntaxa), int(state_unknown), int(nslots),
                          int(bool(safe)), int(precision), int(device),
                          int(max_ops if max_ops is not None else max(2 * ntaxa, 8)), int(flags))
        h = ct.c_void_p()
        _check(lib().iqgpu_create(ct.byref(self.cfg), ct.byref(h)))
        self.h = h
        self.nptn, self.nstates, self.ncat, self.ntaxa = int(nptn), int(nstates), int(ncat), int(ntaxa)
        eff = Config()
        _check(lib().iqgpu_get_config(self.h, ct.byref(eff)))
        self.safe = bool(eff.safe)  # after the reference's SAFE rule
        self.precision = int(precision)

    @property
    def tensor_cores(self):
        """True when the pattern-node update runs on the tensor cores (split TF32 or BF16, 16..64 states)."""
        return self.precision in (TF32X3, BF16) and 16 <= self.nstates <= 64

    @staticmethod
    def memory_required(**kw):
        c = Config(kw["nptn"], kw["nstates"], kw["ncat"], kw["ntaxa"], kw["state_unknown"], kw["nslots"],
                   int(kw.get("safe", 0)), int(kw.get("precision", F64)), 0,
                   kw.get("max_ops", max(2 * kw["ntaxa"], 8)), int(kw.get("flags", 0)))
        out = ct.c_size_t()
        _check(lib().iqgpu_memory_required(ct.byref(c), ct.byref(out)))
        return out.value

    def close(self):
        if getattr(self, "h", None):
            lib().iqgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def block(self):
        return self.nstates * self.ncat

    def set_model(self, model):
        if getattr(model, "nmix", 1) > 1:
            return self.set_mixture(model)
        if hasattr(model, "ceval"):
            return self.set_model_nonrev(model)
        a = [np.ascontiguousarray(x, np.float64) for x in (model.eval, model.evec, model.inv_evec,
                                                            model.rates, model.props)]
        _check(lib().iqgpu_set_model(self.h, *[_dp(x) for x in a]))
        _check(lib().iqgpu_set_state_freq(self.h, _dp(np.ascontiguousarray(model.pi, np.float64))))
        _check(lib().iqgpu_set_tip_partials(self.h, _dp(np.ascontiguousarray(model.tip_lh, np.float64))))

    def set_mixture(self, mix):
        """A ``models.MixtureModel``: per-class eigen systems, profiles and tip
        vectors, per-category rates and proportions (mixed-precision engines)."""
        arrs = [np.ascontiguousarray(x, np.float64) for x in (mix.eval, mix.evec, mix.inv_evec, mix.rates,
                                                               mix.props, mix.tip_lh, mix.pi)]
        _check(lib().iqgpu_set_mixture(self.h, int(mix.nmix), *[_dp(x) for x in arrs]))

    def set_model_nonrev(self, model, rooted=False):
        """A ``models.NonrevModel``. Unrooted (default): the evaluated branch
        is weighted by the stationary frequencies. Rooted: branches carry no
        frequencies; the root leaf (op flag ``ROOTLEAF``) carries them."""
        c = lambda x: np.ascontiguousarray(x, np.float64)
        arrs = [c(model.ceval.real), c(model.ceval.imag), c(model.cevec.real), c(model.cevec.imag),
                c(model.cinv_evec.real), c(model.cinv_evec.imag), c(model.rates), c(model.props),
                c(model.tip_vec), c(model.pi)]
        _check(lib().iqgpu_set_model_nonrev(self.h, *[_dp(x) for x in arrs]))
        w = np.ones(model.nstates) if rooted else model.pi
        _check(lib().iqgpu_set_state_freq(self.h, _dp(c(w))))

    def set_patterns(self, freq, invar=None):
        f = np.ascontiguousarray(freq, np.float64)
        iv = None if invar is None else _dp(np.ascontiguousarray(invar, np.float64))
        _check(lib().iqgpu_set_patterns(self.h, _dp(f), iv))

    def set_asc(self, nconst, nsite):
        """+ASC (Lewis): the last ``nconst`` patterns are the unobserved constant
        patterns (``models.asc_lewis_patterns``); lnL and derivatives are
        corrected with ``nsite`` sites. 0 switches it off."""
        _check(lib().iqgpu_set_asc(self.h, int(nconst), float(nsite)))

    def set_asc_holder(self, nobs):
        """+ASC (Holder, missing data): the first ``nobs`` patterns are observed,
        the rest their unobserved patterns (``models.asc_holder_patterns``)."""
        _check(lib().iqgpu_set_asc_holder(self.h, int(nobs)))

    def set_tip_states(self, patterns):
        s = np.ascontiguousarray(patterns, np.uint8)
        _check(lib().iqgpu_set_tip_states(self.h, s.ctypes.data_as(_U8P)))

    @staticmethod
    def ops_array(ops):
        """(dad, child0, child1, len0, len1[, flags]) tuples; flags are the
        OP_* bits of non-reversible models."""
        arr = np.zeros(len(ops), OP_DTYPE)
        for k, op in enumerate(ops):
            dad, c0, c1, l0, l1 = op[:5]
            arr[k] = (dad, (c0, c1), op[5] if len(op) > 5 else 0, (l0, l1))
        return arr

    def compute_partials(self, ops):
        arr = ops if isinstance(ops, np.ndarray) else self.ops_array(ops)
        _check(lib().iqgpu_compute_partials(self.h, arr.ctypes.data, len(arr)))

    def branch_lnl(self, a, b, length):
        out = ct.c_double()
        _check(lib().iqgpu_branch_lnl(self.h, a, b, length, ct.byref(out)))
        return out.value

    def compute_likelihood(self, ops, a, b, length):
        arr = ops if isinstance(ops, np.ndarray) else self.ops_array(ops)
        out = ct.c_double()
        _check(lib().iqgpu_compute_likelihood(self.h, arr.ctypes.data, len(arr), a, b, length, ct.byref(out)))
        return out.value

    def likelihood_derv(self, ops, a, b, length, theta_computed=False):
        arr = ops if isinstance(ops, np.ndarray) else self.ops_array(ops)
        df, ddf = ct.c_double(), ct.c_double()
        _check(lib().iqgpu_likelihood_derv(self.h, arr.ctypes.data, len(arr), a, b, length,
                                           int(theta_computed), ct.byref(df), ct.byref(ddf)))
        return df.value, ddf.value

    def newton_supported(self):
        out = ct.c_int32()
        _check(lib().iqgpu_newton_supported(self.h, ct.byref(out)))
        return bool(out.value)

    def newton_branch(self, ops, a, b, x1, xguess, x2, xacc, max_nr_step=100, theta_computed=False, full=False):
        """minimizeNewton of one branch on the device: (optx, iterations);
        with full=True also its d2l output and the last evaluated length."""
        arr = ops if isinstance(ops, np.ndarray) else self.ops_array(ops)
        out, d2l, last, steps = ct.c_double(), ct.c_double(), ct.c_double(), ct.c_int32()
        _check(lib().iqgpu_newton_branch(self.h, arr.ctypes.data, len(arr), a, b, int(theta_computed), x1, xguess,
                                         x2, xacc, max_nr_step, ct.byref(out), ct.byref(d2l), ct.byref(last),
                                         ct.byref(steps)))
        if full:
            return out.value, steps.value, d2l.value, last.value
        return out.value, steps.value

    def lnl_from_buffer(self, length):
        out = ct.c_double()
        _check(lib().iqgpu_lnl_from_buffer(self.h, length, ct.byref(out)))
        return out.value

    def pattern_lh(self):
        out = np.zeros(self.nptn)
        _check(lib().iqgpu_get_pattern_lh(self.h, _dp(out)))
        return out

    def partial(self, slot):
        p = np.zeros((self.nptn, self.block))
        s = np.zeros((self.nptn, self.ncat if self.safe else 1), np.uint8)
        _check(lib().iqgpu_get_partial(self.h, slot, _dp(p), s.ctypes.data_as(_U8P)))
        return p, s

    def exponent(self, slot):
        e = np.zeros(self.nptn, np.int32)
        _check(lib().iqgpu_get_exponent(self.h, slot, e.ctypes.data_as(_I32P)))
        return e

    def sync(self):
        _check(lib().iqgpu_sync(self.h))

    def set_stream(self, cuda_stream_handle):
        """Run on a caller stream (an int cudaStream_t, e.g. torch.cuda.Stream().cuda_stream)."""
        _check(lib().iqgpu_set_stream(self.h, ct.c_void_p(cuda_stream_handle or None)))

    def set_timing(self, enable=True):
        _check(lib().iqgpu_set_timing(self.h, int(enable)))

    def timing(self):
        ms, n = ct.c_double(), ct.c_int64()
        _check(lib().iqgpu_get_timing(self.h, ct.byref(ms), ct.byref(n)))
        return ms.value, n.value

    def set_tile(self, patterns_per_cta):
        _check(lib().iqgpu_set_tile(self.h, int(patterns_per_cta)))

    def set_schedule(self, schedule):
        """0 = fused, 1 = level-synchronous, 2 = dataflow (4-state kernel),
        3 = level-synchronous on the warp-specialised tensor-core kernel,
        4 = level-synchronous with operand A in tensor memory (20 states),
        5 = as 3 with category-split narrow levels, 6 / 7 = dataflow on the
        tensor cores (category-split / whole items), 8 / 9 = level-synchronous
        on the deep-ring kernel (20 states; 9 with the one-op levels in one
        launch per pattern tile)."""
        _check(lib().iqgpu_set_schedule(self.h, int(schedule)))

    def launches(self):
        """Kernel launches this engine has issued so far."""
        n = ct.c_int64()
        _check(lib().iqgpu_get_launches(self.h, ct.byref(n)))
        return n.value

    def set_stages(self, stages):
        """Ring depth of the tensor-core traversal (0 = default, 2, 3 or 4)."""
        _check(lib().iqgpu_set_stages(self.h, int(stages)))

    def set_kpieces(self, pieces):
        """K pieces per stage of the tensor-core traversal (0/1 whole K, 2 halves)."""
        _check(lib().iqgpu_set_kpieces(self.h, int(pieces)))

    def nni_batch(self, cands, max_nr_step=10, min_bl=1e-6, max_bl=10.0):
        """cands: iterable of ((sub0..sub3), (scratch0, scratch1), (len0..len3), central)."""
        cands = list(cands)
        arr = np.zeros(len(cands), NNI_DTYPE)
        for k, (sub, scr, lens, central) in enumerate(cands):
            arr[k] = (sub, scr, lens, central)
        lnl, blen = np.zeros(len(cands)), np.zeros(len(cands))
        _check(lib().iqgpu_nni_batch(self.h, arr.ctypes.data, len(cands), int(max_nr_step), float(min_bl),
                                     float(max_bl), _dp(lnl), _dp(blen)))
        return lnl, blen

    def set_boot_weights(self, weights):
        w = np.ascontiguousarray(weights, np.float32)
        _check(lib().iqgpu_set_boot_weights(self.h, w.ctypes.data_as(ct.POINTER(ct.c_float)), w.shape[0]))
        self._nreps = w.shape[0]

    def rell_current(self):
        """RELL scores of the last evaluated tree against every replicate (device-resident inputs)."""
        out = np.zeros(self._nreps)
        _check(lib().iqgpu_rell_current(self.h, _dp(out)))
        return out

    def rell(self, pattern_lh):
        plh = np.ascontiguousarray(pattern_lh, np.float64)
        out = np.zeros((plh.shape[0], self._nreps))
        _check(lib().iqgpu_rell(self.h, _dp(plh), plh.shape[0], _dp(out)))
        return out


class Group:
    """Partitions as one graph launch: engines (one per partition) evaluated together."""

    def __init__(self, engines):
        self.engines = list(engines)
        arr = (ct.c_void_p * len(self.engines))(*[e.h.value for e in self.engines])
        h = ct.c_void_p()
        _check(lib().iqgpu_group_create(ct.cast(arr, ct.c_void_p), len(self.engines), ct.byref(h)))
        self.h = h
        self._keep = None

    def _lists(self, ops_list):
        arrs = [o if isinstance(o, np.ndarray) else Engine.ops_array(o) for o in ops_list]
        ptrs = (ct.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        return arrs, ptrs

    def prepare(self, ops_list, a, b, lengths):
        arrs, ptrs = self._lists(ops_list)
        self._keep = arrs
        nops = np.array([len(x) for x in arrs], np.int32)
        aa, bb = np.asarray(a, np.int32), np.asarray(b, np.int32)
        ll = np.asarray(lengths, np.float64)
        _check(lib().iqgpu_group_prepare(self.h, ct.cast(ptrs, ct.c_void_p), nops.ctypes.data, aa.ctypes.data,
                                         bb.ctypes.data, ll.ctypes.data))

    def set_lengths(self, ops_list, lengths):
        arrs, ptrs = self._lists(ops_list)
        self._keep = arrs
        ll = np.asarray(lengths, np.float64)
        _check(lib().iqgpu_group_set_lengths(self.h, ct.cast(ptrs, ct.c_void_p), ll.ctypes.data))

    def lnl(self):
        per = np.zeros(len(self.engines))
        tot = ct.c_double()
        _check(lib().iqgpu_group_lnl(self.h, per.ctypes.data, ct.byref(tot)))
        return tot.value, per

    def close(self):
        if getattr(self, "h", None):
            lib().iqgpu_group_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuTree:
    """PhyloTree drivers on the GPU engine (one engine per tree)."""

    def __init__(self, model, patterns, freq, edges, lengths, safe=False, precision=F64, device=0, invar=None,
                 flags=0, asc=None, slots=None):
        """asc=(nconst, nsite): +ASC (Lewis) with the last nconst patterns as
        the unobserved constant patterns (``models.asc_lewis_patterns``).
        slots: partial slots of the engine (default one per directed internal
        partial, 3*(ntaxa-2)); fewer are recycled and partials recomputed as
        needed (the reference's LM_MEM_SAVE)."""
        ntaxa = patterns.shape[0]
        self.ntaxa = ntaxa
        self.nedge = len(edges)  # 2*ntaxa-3, fewer with multifurcating nodes
        self.engine = Engine(patterns.shape[1], model.nstates, model.ncat, ntaxa, model.state_unknown,
                             slots or 3 * (ntaxa - 2), safe=safe, precision=precision, device=device,
                             max_ops=2 * ntaxa, flags=flags)
        self.engine.set_model(model)
        self.engine.set_patterns(freq, invar)
        self.engine.set_tip_states(patterns)
        if asc:
            self.engine.set_asc(*asc)
        self.edges = np.ascontiguousarray(edges, np.int32)
        h = ct.c_void_p()
        _check(lib().iqgpu_tree_create_n(self.engine.h, self.nedge, self.edges.ctypes.data_as(_I32P),
                                         _dp(np.ascontiguousarray(lengths, np.float64)), ct.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().iqgpu_tree_destroy(self.h)
            self.h = None
        if getattr(self, "engine", None):
            self.engine.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def compute_likelihood(self, want_pattern_lh=False):
        out = ct.c_double()
        plh = np.zeros(self.engine.nptn) if want_pattern_lh else None
        _check(lib().iqgpu_tree_compute_likelihood(self.h, ct.byref(out), _dp(plh) if plh is not None else None))
        return (out.value, plh) if want_pattern_lh else out.value

    def optimize_one_branch(self, n1, n2, max_nr_step=100):
        _check(lib().iqgpu_tree_optimize_one_branch(self.h, n1, n2, max_nr_step))

    def optimize_all_branches(self, iterations=100, tolerance=1e-3, max_nr_step=100):
        out = ct.c_double()
        _check(lib().iqgpu_tree_optimize_all_branches(self.h, iterations, tolerance, max_nr_step, ct.byref(out)))
        return out.value

    def lengths(self):
        out = np.zeros(self.nedge)
        _check(lib().iqgpu_tree_get_lengths(self.h, _dp(out)))
        return out

    def set_lengths(self, lengths):
        _check(lib().iqgpu_tree_set_lengths(self.h, _dp(np.ascontiguousarray(lengths, np.float64))))

    def set_bounds(self, min_bl, max_bl):
        _check(lib().iqgpu_tree_set_bounds(self.h, min_bl, max_bl))

    def set_device_newton(self, on):
        """False: minimizeNewton on the host; True (1): on the device, whole
        optimizeAllBranches passes at once where served; 2: on the device,
        one branch at a time."""
        _check(lib().iqgpu_tree_set_device_newton(self.h, 2 if on == 2 else int(bool(on))))

    def num_updates(self):
        out = ct.c_int64()
        _check(lib().iqgpu_tree_num_updates(self.h, ct.byref(out)))
        return out.value
