"""ctypes binding of the CPU FP64 oracle (test infrastructure only).

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module; it is the checker, never the product path.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libphylo_oracle.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ct.CDLL(_LIB_PATH)
        dp, ip, u8p = ct.POINTER(ct.c_double), ct.POINTER(ct.c_int), ct.POINTER(ct.c_uint8)
        L.orc_compute_partials.argtypes = [ct.c_void_p, dp, u8p, ct.c_void_p, ct.c_int, ct.c_int]
        L.orc_branch_lnl.argtypes = [ct.c_void_p, dp, u8p, ct.c_int, ct.c_int, ct.c_double, dp, ct.c_int]
        L.orc_branch_lnl.restype = ct.c_double
        L.orc_compute_theta.argtypes = [ct.c_void_p, dp, u8p, ct.c_int, ct.c_int, dp, dp, ct.c_int]
        L.orc_derv.argtypes = [ct.c_void_p, dp, dp, ct.c_double, dp, dp, ct.c_int]
        L.orc_lnl_from_buffer.argtypes = [ct.c_void_p, dp, dp, ct.c_double, dp, ct.c_int]
        L.orc_lnl_from_buffer.restype = ct.c_double
        L.orc_tree_new.argtypes = [ct.c_void_p, ip, ct.c_int, dp, ct.c_int]
        L.orc_tree_new.restype = ct.c_void_p
        L.orc_tree_free.argtypes = [ct.c_void_p]
        L.orc_tree_compute_likelihood.argtypes = [ct.c_void_p, dp]
        L.orc_tree_compute_likelihood.restype = ct.c_double
        L.orc_tree_optimize_one_branch.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, ct.c_int]
        L.orc_tree_optimize_all_branches.argtypes = [ct.c_void_p, ct.c_int, ct.c_double, ct.c_int, ip]
        L.orc_tree_optimize_all_branches.restype = ct.c_double
        L.orc_tree_get_lengths.argtypes = [ct.c_void_p, dp]
        L.orc_tree_set_lengths.argtypes = [ct.c_void_p, dp]
        L.orc_tree_set_bounds.argtypes = [ct.c_void_p, ct.c_double, ct.c_double]
        L.orc_tree_num_updates.argtypes = [ct.c_void_p]
        L.orc_tree_num_updates.restype = ct.c_longlong
        L.orc_tree_get_partial.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, dp, u8p]
        L.orc_tree_derv.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, ct.c_double, dp, dp]
        L.orc_tree_lnl_branch.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, dp]
        L.orc_tree_lnl_branch.restype = ct.c_double
        _lib = L
    return _lib


class _Model(ct.Structure):
    _fields_ = [("nptn", ct.c_int), ("nstates", ct.c_int), ("ncat", ct.c_int), ("ntaxa", ct.c_int),
                ("state_unknown", ct.c_int), ("safe", ct.c_int),
                ("eval", ct.c_void_p), ("evec", ct.c_void_p), ("inv_evec", ct.c_void_p),
                ("rates", ct.c_void_p), ("props", ct.c_void_p), ("tip_lh", ct.c_void_p),
                ("ptn_freq", ct.c_void_p), ("ptn_invar", ct.c_void_p), ("tip_states", ct.c_void_p),
                ("ref_triple_tail", ct.c_int), ("asc_n", ct.c_int), ("asc_nsite", ct.c_double)]


def _dp(a):
    return a.ctypes.data_as(ct.POINTER(ct.c_double))


class OracleModel:
    """Owns the arrays an ``orc_model`` points at."""

    def __init__(self, model, patterns, freq, safe=False, invar=None, ref_triple_tail=False, asc=None):
        """asc=(nconst, nsite): the last nconst patterns are +ASC's unobserved
        constant patterns (weight 0), corrected for with nsite sites."""
        self.arrays = dict(
            eval=np.ascontiguousarray(model.eval, np.float64),
            evec=np.ascontiguousarray(model.evec, np.float64),
            inv_evec=np.ascontiguousarray(model.inv_evec, np.float64),
            rates=np.ascontiguousarray(model.rates, np.float64),
            props=np.ascontiguousarray(model.props, np.float64),
            tip_lh=np.ascontiguousarray(model.tip_lh, np.float64),
            ptn_freq=np.ascontiguousarray(freq, np.float64),
            ptn_invar=np.ascontiguousarray(np.zeros(len(freq)) if invar is None else invar, np.float64),
            tip_states=np.ascontiguousarray(patterns, np.uint8),
        )
        a = self.arrays
        self.nstates, self.ncat = model.nstates, model.ncat
        self.nptn, self.ntaxa = patterns.shape[1], patterns.shape[0]
        self.safe = bool(safe)
        self.s = _Model(self.nptn, model.nstates, model.ncat, self.ntaxa, model.state_unknown, int(safe),
                        *[a[k].ctypes.data for k in ("eval", "evec", "inv_evec", "rates", "props",
                                                     "tip_lh", "ptn_freq", "ptn_invar", "tip_states")],
                        int(ref_triple_tail), int(asc[0]) if asc else 0, float(asc[1]) if asc else 0.0)

    @property
    def ptr(self):
        return ct.addressof(self.s)

    @property
    def block(self):
        return self.nstates * self.ncat


class OracleTree:
    """PhyloTree restatement: computeLikelihood / optimizeOneBranch / optimizeAllBranches."""

    def __init__(self, model, patterns, freq, edges, lengths, safe=False, nthreads=0, invar=None,
                 ref_triple_tail=False, asc=None):
        """ref_triple_tail=True reproduces the reference's derivative sum exactly,
        including its double-counted last entry for odd nstates (codon +G4)."""
        self.m = OracleModel(model, patterns, freq, safe=safe, invar=invar, ref_triple_tail=ref_triple_tail,
                             asc=asc)
        self.edges = np.ascontiguousarray(edges, np.int32)
        self.nedge = len(self.edges)
        L = lib()
        self.h = L.orc_tree_new(self.m.ptr, self.edges.ctypes.data_as(ct.POINTER(ct.c_int)), self.nedge,
                                _dp(np.ascontiguousarray(lengths, np.float64)), int(nthreads))
        if not self.h:
            raise ValueError("tree node degree above ORC_MAX_DEG")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_tree_free(self.h)
            self.h = None

    def compute_likelihood(self, want_pattern_lh=False):
        plh = np.zeros(self.m.nptn) if want_pattern_lh else None
        v = lib().orc_tree_compute_likelihood(self.h, _dp(plh) if plh is not None else None)
        return (v, plh) if want_pattern_lh else v

    def optimize_one_branch(self, n1, n2, max_nr_step=100):
        return lib().orc_tree_optimize_one_branch(self.h, n1, n2, max_nr_step)

    def optimize_all_branches(self, iterations=100, tolerance=1e-3, max_nr_step=100):
        st = ct.c_int(0)
        v = lib().orc_tree_optimize_all_branches(self.h, iterations, tolerance, max_nr_step, ct.byref(st))
        if st.value != 0:
            raise RuntimeError("oracle Newton-Raphson failed")
        return v

    def lengths(self):
        out = np.zeros(self.nedge)
        lib().orc_tree_get_lengths(self.h, _dp(out))
        return out

    def set_lengths(self, lengths):
        lib().orc_tree_set_lengths(self.h, _dp(np.ascontiguousarray(lengths, np.float64)))

    def set_bounds(self, min_bl, max_bl):
        lib().orc_tree_set_bounds(self.h, min_bl, max_bl)

    def num_updates(self):
        return lib().orc_tree_num_updates(self.h)

    def derv(self, n1, n2, length):
        df, ddf = ct.c_double(), ct.c_double()
        if lib().orc_tree_derv(self.h, n1, n2, length, ct.byref(df), ct.byref(ddf)):
            raise ValueError("not a branch")
        return df.value, ddf.value

    def lnl_branch(self, node, dad, want_pattern_lh=False):
        plh = np.zeros(self.m.nptn) if want_pattern_lh else None
        v = lib().orc_tree_lnl_branch(self.h, node, dad, _dp(plh) if plh is not None else None)
        return (v, plh) if want_pattern_lh else v

    def partial(self, node, nbr):
        """Partial of directed branch node->nbr in the reference layout [ptn][c][x]."""
        B = self.m.block
        p = np.zeros((self.m.nptn, B))
        s = np.zeros((self.m.nptn, self.m.ncat if self.m.safe else 1), np.uint8)
        rc = lib().orc_tree_get_partial(self.h, node, nbr, _dp(p), s.ctypes.data_as(ct.POINTER(ct.c_uint8)))
        if rc:
            raise ValueError("nbr is a leaf")
        return p, s
