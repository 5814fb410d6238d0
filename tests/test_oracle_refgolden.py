"""The C oracle against the reference kernels' committed outputs.

tests/golden/ref_*.npz hold what IQ-TREE 2's own compiled kernels return on
the reference's test alignments and on a tree that underflows 2^-256
(tests/golden/make_refgolden.py). The oracle must reproduce them on any
machine: within 1e-13 relative (bit for bit where libm's exp and log round
as on the machine that wrote the files), scale counts identical.
"""
import numpy as np
import pytest

from helpers import REF_FIXTURES, load_ref_golden, rel

TOL = 1e-13


@pytest.mark.parametrize("name", REF_FIXTURES)
@pytest.mark.parametrize("safe", [False, True])
def test_oracle_reproduces_reference_outputs(oracle_mod, name, safe):
    g = load_ref_golden(name)
    d, tag = g.d, "safe" if safe else "norm"
    o = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe, nthreads=1)
    for k, (node, dad) in enumerate(g.oriented):
        assert rel(o.lnl_branch(node, dad), float(d[f"lnl_{tag}"][k])) < TOL, k
    node, dad = g.oriented[0]
    _, plh = o.lnl_branch(node, dad, want_pattern_lh=True)
    np.testing.assert_allclose(plh, d[f"pattern_lnl_{tag}"], rtol=TOL, atol=0)
    pu, pv = (int(x) for x in d["partial_branch"])
    p, s = o.partial(pu, pv)
    np.testing.assert_array_equal(s, d[f"scale_{tag}"])
    ref_p = d[f"partial_{tag}"]
    scale = np.maximum(np.abs(ref_p).max(axis=1, keepdims=True), 1e-300)
    assert np.max(np.abs(p[:len(ref_p)] - ref_p) / scale) < TOL
    for i, k in enumerate(d["derv_edges"]):
        u, v = (int(x) for x in g.edges[k])
        for j, L in enumerate(d["derv_lengths"]):
            o2 = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths, safe=safe, nthreads=1)
            df, ddf = o2.derv(u, v, float(L))
            rdf, rddf = d[f"derv_{tag}"][i][j]
            assert abs(df - rdf) <= TOL * max(1.0, abs(rdf)) and abs(ddf - rddf) <= TOL * max(1.0, abs(rddf))
