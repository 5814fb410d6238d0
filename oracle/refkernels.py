"""ctypes binding of the reference oracle (test infrastructure only).

``oracle/_ref/libiqref.so`` is IQ-TREE 2's own likelihood kernel templates
(tree/phylokernelnew.h) compiled from a reference checkout by
``oracle/ref/Makefile`` against a stand-in PhyloTree environment
(``oracle/ref/refenv.h``). The tests use it to pin ``oracle/phylo_oracle.c``
to the reference's compiled arithmetic, and ``tests/golden/make_refgolden.py``
writes golden vectors from it. It exists only where a reference checkout is
available; nothing on the product path imports this module.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libiqref.so")
FAST_LIB_PATH = os.path.join(_HERE, "_ref", "libiqref_fast.so")
STAGED = os.path.join(_HERE, "_ref", "src")  # the kernel headers, copied by `make stage`
DEFAULT_REFERENCE = os.environ.get("IQTREE_REFERENCE", "/root/reference")
_lib = None
_fast = None

KIND_SCALAR = 0  # one-lane generic kernels (Vec1d)
KIND_SIMD = 1    # the SIMD kernels the reference installs on this host


def reference_dir():
    """A reference checkout, or the staged copy of its kernel headers."""
    for d in (DEFAULT_REFERENCE, STAGED):
        if os.path.exists(os.path.join(d, "tree", "phylokernelnew.h")):
            return d
    return None


def available():
    return os.path.exists(LIB_PATH) or reference_dir() is not None


def build():
    ref = reference_dir()
    if ref is None:
        raise RuntimeError("no reference checkout: set IQTREE_REFERENCE to an IQ-TREE 2 source tree")
    mk = ["make", "-s", "-C", os.path.join(_HERE, "ref"), f"REFERENCE={os.path.abspath(ref)}"]
    if os.path.abspath(ref) != os.path.abspath(STAGED):
        subprocess.run(mk + ["stage"], check=True)  # the headers travel with the tree to machines without it
    subprocess.run(mk, check=True)


def _bind(path):
    L = ct.CDLL(path)
    vp, dp, ip, u8p = ct.c_void_p, ct.POINTER(ct.c_double), ct.POINTER(ct.c_int), ct.POINTER(ct.c_uint8)
    L.iqref_last_error.restype = ct.c_char_p
    L.iqref_simd_info.argtypes = [ip, ip]
    L.iqref_create.argtypes = [ct.c_int] * 8 + [ct.POINTER(vp)]
    L.iqref_destroy.argtypes = [vp]
    L.iqref_set_model.argtypes = [vp, dp, dp, dp, dp, dp]
    L.iqref_set_tip_lh.argtypes = [vp, dp]
    L.iqref_set_patterns.argtypes = [vp, dp, dp, ct.c_int]
    L.iqref_set_tips.argtypes = [vp, u8p]
    L.iqref_set_tree.argtypes = [vp, ct.c_int, ip, dp]
    L.iqref_set_length.argtypes = [vp, ct.c_int, ct.c_double]
    L.iqref_branch_lnl.argtypes = [vp, ct.c_int, ct.c_int, dp, dp]
    L.iqref_derv.argtypes = [vp, ct.c_int, ct.c_int, dp, dp]
    L.iqref_from_buffer.argtypes = [vp, ct.c_double, dp]
    L.iqref_get_partial.argtypes = [vp, ct.c_int, ct.c_int, dp, u8p]
    return L


def lib(fast=False):
    """The strict build (parity) or, with fast=True, the build with the
    reference's own optimisation and FMA contraction (CPU baseline)."""
    global _lib, _fast
    if (_fast if fast else _lib) is None:
        if reference_dir() is not None:
            build()
        path = FAST_LIB_PATH if fast else LIB_PATH
        if not os.path.exists(path):
            raise RuntimeError("reference oracle not built")
        if fast:
            _fast = _bind(path)
        else:
            _lib = _bind(path)
    return _fast if fast else _lib


def simd_info(fast=False):
    """(vector width, FMA) of the SIMD kernels (kind 1) of a build."""
    v, f = ct.c_int(), ct.c_int()
    lib(fast).iqref_simd_info(ct.byref(v), ct.byref(f))
    return v.value, bool(f.value)


def _dp(a):
    return None if a is None else a.ctypes.data_as(ct.POINTER(ct.c_double))


def _check(rc, L=None):
    if rc:
        raise RuntimeError("reference oracle: " + (L or lib()).iqref_last_error().decode())


class RefTree:
    """The reference's kernels on one tree: branch lnL, derivatives, partials.

    Node numbering and neighbour order follow ``edges`` as in
    ``oracle.OracleTree``: leaves 0..ntaxa-1, a node's neighbours in edge order.
    """

    def __init__(self, model, patterns, freq, edges, lengths, safe=False, kind=KIND_SCALAR, nthreads=1,
                 invar=None, nsite=None, fast=False):
        """fast=True: the build with the reference's optimisation and FMA
        contraction (CPU baseline timing); nthreads > 1 splits patterns into
        OpenMP packets as the reference does (2 per thread)."""
        patterns = np.ascontiguousarray(patterns, np.uint8)
        self.ntaxa, self.nptn = patterns.shape
        self.nstates, self.ncat, self.safe = model.nstates, model.ncat, bool(safe)
        self.edges = np.ascontiguousarray(edges, np.int32)
        self.lengths = np.array(lengths, np.float64)
        self.L = L = lib(fast)
        h = ct.c_void_p()
        _check(L.iqref_create(self.ntaxa, self.nptn, model.nstates, model.ncat, model.state_unknown, int(safe),
                              int(kind), int(nthreads), ct.byref(h)), L)
        self.h = h
        arr = {k: np.ascontiguousarray(getattr(model, k), np.float64)
               for k in ("eval", "evec", "inv_evec", "rates", "props", "tip_lh")}
        _check(L.iqref_set_model(h, *[_dp(arr[k]) for k in ("eval", "evec", "inv_evec", "rates", "props")]), L)
        _check(L.iqref_set_tip_lh(h, _dp(arr["tip_lh"])), L)
        freq = np.ascontiguousarray(freq, np.float64)
        inv = None if invar is None else np.ascontiguousarray(invar, np.float64)
        _check(L.iqref_set_patterns(h, _dp(freq), _dp(inv), int(nsite if nsite is not None else round(freq.sum()))))
        _check(L.iqref_set_tips(h, patterns.ctypes.data_as(ct.POINTER(ct.c_uint8))))
        _check(L.iqref_set_tree(h, len(self.edges), self.edges.ctypes.data_as(ct.POINTER(ct.c_int)),
                                _dp(self.lengths)))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.iqref_destroy(self.h)
            self.h = None

    def set_length(self, edge, length):
        self.lengths[edge] = length
        _check(self.L.iqref_set_length(self.h, int(edge), float(length)), self.L)

    def set_lengths(self, lengths):
        for e, v in enumerate(lengths):
            self.set_length(e, v)

    def branch_lnl(self, node, dad, want_pattern_lh=False):
        v = ct.c_double()
        plh = np.zeros(self.nptn) if want_pattern_lh else None
        _check(self.L.iqref_branch_lnl(self.h, int(node), int(dad), ct.byref(v), _dp(plh)), self.L)
        return (v.value, plh) if want_pattern_lh else v.value

    def derv(self, node1, node2):
        df, ddf = ct.c_double(), ct.c_double()
        _check(self.L.iqref_derv(self.h, int(node1), int(node2), ct.byref(df), ct.byref(ddf)), self.L)
        return df.value, ddf.value

    def from_buffer(self, length):
        v = ct.c_double()
        _check(self.L.iqref_from_buffer(self.h, float(length), ct.byref(v)), self.L)
        return v.value

    def partial(self, dad, node):
        """Partial of the subtree at ``node`` seen from ``dad`` ([ptn][c*n+x],
        eigen space) and its scale counts; ``oracle.OracleTree.partial(dad, node)``
        names the same directed branch."""
        B = self.nstates * self.ncat
        p = np.zeros((self.nptn, B))
        s = np.zeros((self.nptn, self.ncat if self.safe else 1), np.uint8)
        _check(self.L.iqref_get_partial(self.h, int(node), int(dad), _dp(p), s.ctypes.data_as(ct.POINTER(ct.c_uint8))))
        return p, s
