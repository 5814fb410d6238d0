"""The C oracle against IQ-TREE 2's own compiled kernels (reference oracle).

``oracle/_ref/libiqref.so`` is the reference's tree/phylokernelnew.h kernel
templates compiled from a reference checkout (``oracle/ref/``). Its one-lane
kernels (kind 0) and ``oracle/phylo_oracle.c`` (one thread) must agree BIT
FOR BIT: every partial, every scale count, the branch lnL on every edge, the
pattern lnL, the Newton-Raphson derivatives and the lnL from the theta
buffer, NORM and SAFE, on the seeded fixtures, on a tree that underflows
2^-256 and on the reference's own test alignments. The SIMD kernels the
reference installs on this host (kind 1) agree within 1e-12 with identical
scale counts.

Skipped where no reference checkout is available (the reference oracle is
built from its sources).
"""
import numpy as np
import pytest

from helpers import load_golden, rel

refkernels = pytest.importorskip("refkernels")
if not refkernels.available():
    pytest.skip("no reference checkout for the reference oracle", allow_module_level=True)

import refdata  # noqa: E402
from iqtree2_gb300 import simulate  # noqa: E402


def _oriented(edges, ntaxa):
    """(node, dad) of every edge, the dad a leaf where the edge has one."""
    out = []
    for (u, v) in edges:
        u, v = int(u), int(v)
        out.append((u, v) if v < ntaxa else (v, u))
    return out


def _check_bit_exact(oracle_mod, model, patterns, freq, edges, lengths, safe, derv_edges=None,
                     all_partials=True, codon_tail=False):
    ntaxa = patterns.shape[0]
    o = oracle_mod.OracleTree(model, patterns, freq, edges, lengths, safe=safe, nthreads=1,
                              ref_triple_tail=codon_tail)
    r = refkernels.RefTree(model, patterns, freq, edges, lengths, safe=safe, kind=refkernels.KIND_SCALAR)
    # branch lnL on every edge, pattern lnL on the first
    for k, (node, dad) in enumerate(_oriented(edges, ntaxa)):
        if k == 0:
            a, pa = r.branch_lnl(node, dad, want_pattern_lh=True)
            b, pb = o.lnl_branch(node, dad, want_pattern_lh=True)
            assert a == b, (k, a, b)
            np.testing.assert_array_equal(pa, pb)
        else:
            assert r.branch_lnl(node, dad) == o.lnl_branch(node, dad), k
    # partials and scale counts
    if all_partials:
        nnode = 2 * ntaxa - 2
        adj = [[] for _ in range(nnode)]
        for (u, v) in edges:
            adj[int(u)].append(int(v))
            adj[int(v)].append(int(u))
        for u in range(nnode):
            for v in adj[u]:
                if v < ntaxa:
                    continue
                po, so = o.partial(u, v)
                pr, sr = r.partial(u, v)
                np.testing.assert_array_equal(so, sr)
                np.testing.assert_array_equal(po, pr)
    # derivatives and lnL from the theta buffer
    derv_edges = range(len(edges)) if derv_edges is None else derv_edges
    for k in derv_edges:
        u, v = (int(x) for x in edges[k])
        o2 = oracle_mod.OracleTree(model, patterns, freq, edges, lengths, safe=safe, nthreads=1,
                                   ref_triple_tail=codon_tail)
        r2 = refkernels.RefTree(model, patterns, freq, edges, lengths, safe=safe, kind=refkernels.KIND_SCALAR)
        for L in (0.01, 0.3):
            r2.set_length(k, L)
            assert r2.derv(u, v) == o2.derv(u, v, L), (k, L)
            # lnL from the theta buffer at a third length, against a full
            # evaluation by the oracle at that length
            fb = r2.from_buffer(0.11)
        lens = np.array(lengths, np.float64)
        lens[k] = 0.11
        o3 = oracle_mod.OracleTree(model, patterns, freq, edges, lens, safe=safe, nthreads=1)
        node, dad = (v, u) if v >= ntaxa else (u, v)
        assert rel(fb, o3.lnl_branch(node, dad)) < 1e-13


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
@pytest.mark.parametrize("safe", [False, True])
def test_oracle_bit_exact_on_fixtures(oracle_mod, name, safe):
    g = load_golden(name)
    _check_bit_exact(oracle_mod, g.model, g.patterns, g.freq, g.edges, g.lengths, safe,
                     codon_tail=(g.model.nstates % 2 == 1))


@pytest.mark.parametrize("safe", [False, True])
def test_oracle_bit_exact_when_partials_underflow(oracle_mod, safe):
    """150 taxa on long branches: partials fall below 2^-256 and get scaled."""
    ds = simulate.protein_lg_dataset(150, 40, 11, mean_bl=0.5)
    r = refkernels.RefTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, safe=safe)
    leaf_edge = next(e for e in ds.edges if 0 in (int(e[0]), int(e[1])))
    _, s = r.partial(0, int(leaf_edge[0]) + int(leaf_edge[1]))
    assert s.sum() > 0, "the case must exercise the scaling"
    _check_bit_exact(oracle_mod, ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, safe,
                     derv_edges=[0, 5, 77], all_partials=True)


@pytest.mark.parametrize("name", list(refdata.REF_ALIGNMENTS))
@pytest.mark.parametrize("safe", [False, True])
def test_oracle_bit_exact_on_reference_alignments(oracle_mod, name, safe):
    d = refdata.load(name, refkernels.reference_dir())
    _check_bit_exact(oracle_mod, d.model, d.patterns, d.freq, d.edges, d.lengths, safe,
                     derv_edges=[0, d.ntaxa, 2 * d.ntaxa - 4], all_partials=(name != "d59_8"))


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
@pytest.mark.parametrize("safe", [False, True])
def test_simd_kernels_agree(oracle_mod, name, safe):
    """The reference's SIMD kernels for this host (AVX2+FMA Vec4d on x86-64,
    Vec2d elsewhere): lnL within 1e-12, scale counts identical."""
    g = load_golden(name)
    o = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe, nthreads=1)
    r = refkernels.RefTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe, kind=refkernels.KIND_SIMD)
    for node, dad in _oriented(g.edges, g.ntaxa):
        assert rel(r.branch_lnl(node, dad), o.lnl_branch(node, dad)) < 1e-12
    for (u, v) in g.edges[:4]:
        u, v = int(u), int(v)
        if v >= g.ntaxa:
            _, so = o.partial(u, v)
            _, sr = r.partial(u, v)
            np.testing.assert_array_equal(so, sr)


def test_committed_fixtures_match_reference(oracle_mod):
    """tests/golden/ref_*.npz hold what the reference kernels compute now."""
    import os
    from helpers import GOLDEN
    d = np.load(os.path.join(GOLDEN, "ref_example.npz"))
    m = refdata.load("example", refkernels.reference_dir())
    np.testing.assert_array_equal(d["patterns"], m.patterns)
    r = refkernels.RefTree(m.model, m.patterns, m.freq, m.edges, m.lengths)
    node, dad = _oriented(m.edges, m.ntaxa)[0]
    assert r.branch_lnl(node, dad) == float(d["lnl_norm"][0])


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
@pytest.mark.parametrize("safe", [False, True])
def test_oracle_bit_exact_on_multifurcating_trees(oracle_mod, name, safe):
    """Internal edges contracted to nodes of degree 4 to 6: the reference's
    multifurcating update (tree/phylokernelnew.h:1407-1631)."""
    from iqtree2_gb300 import topology
    g = load_golden(name)
    internal = [k for k, (u, v) in enumerate(g.edges) if min(u, v) >= g.ntaxa]
    e2, l2, _ = topology.collapse_edges(g.edges, g.lengths, g.ntaxa, internal[:3])
    assert np.bincount(e2.ravel()).max() >= 4
    _check_bit_exact(oracle_mod, g.model, g.patterns, g.freq, e2, l2, safe,
                     codon_tail=(g.model.nstates % 2 == 1))


@pytest.mark.parametrize("safe", [False, True])
def test_oracle_bit_exact_multifurcating_underflow(oracle_mod, safe):
    from iqtree2_gb300 import topology
    ds = simulate.protein_lg_dataset(150, 40, 11, mean_bl=0.5)
    internal = [k for k, (u, v) in enumerate(ds.edges) if min(u, v) >= ds.ntaxa]
    e2, l2, _ = topology.collapse_edges(ds.edges, ds.lengths, ds.ntaxa, internal[::6])
    _check_bit_exact(oracle_mod, ds.model, ds.patterns, ds.freq, e2, l2, safe, derv_edges=[0, 9])
