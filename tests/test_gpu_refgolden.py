"""The GPU paths against IQ-TREE 2's own kernel outputs.

tests/golden/ref_*.npz hold what the reference's compiled kernels
(tree/phylokernelnew.h, one-lane build) return on its own test alignments
(example.phy, d59_8.phy, prot_M126_27_269.phy on a seeded tree) and on a
150-taxon tree whose partials underflow 2^-256 (tests/golden/
make_refgolden.py). The FP64 drop-in must match them through the kernel-level
C ABI: branch lnL on every edge within 1e-10 relative (contract 1e-8), the
pattern lnL, the scale counts of the largest partial identical, its values
within 1e-10 of each pattern's largest entry, derivatives within 1e-9 and the
lnL from the theta buffer within 1e-10, NORM and SAFE, on binary trees
and on trees with multifurcating nodes. The mixed paths (FP32, split TF32
for protein) match the reference's lnL within 1e-6, polytomies included.
"""
import numpy as np
import pytest

from helpers import REF_FIXTURES, load_ref_golden, rel
from iqtree2_gb300 import engine
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu


def _engine(g, topo, safe, precision=engine.F64):
    eng = engine.Engine(g.patterns.shape[1], g.model.nstates, g.model.ncat, g.ntaxa, g.model.state_unknown,
                        topo.nslots, safe=safe, precision=precision, max_ops=2 * topo.nslots)
    eng.set_model(g.model)
    eng.set_patterns(g.freq)
    eng.set_tip_states(g.patterns)
    return eng


@pytest.mark.parametrize("name", REF_FIXTURES)
@pytest.mark.parametrize("safe", [False, True])
def test_fp64_matches_reference_kernels(name, safe):
    g = load_ref_golden(name)
    d, tag = g.d, "safe" if safe else "norm"
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    eng = _engine(g, topo, safe)
    eng.compute_partials(topo.all_partials_ops())
    for k, (node, dad) in enumerate(g.oriented):
        lg = eng.branch_lnl(topo.ref(dad, node), topo.ref(node, dad), topo.edge_len(node, dad))
        assert rel(lg, float(d[f"lnl_{tag}"][k])) < 1e-10, (k, lg, float(d[f"lnl_{tag}"][k]))
        if k == 0:
            np.testing.assert_allclose(eng.pattern_lh(), d[f"pattern_lnl_{tag}"], rtol=1e-10, atol=1e-10)
    pu, pv = (int(x) for x in d["partial_branch"])
    p, s = eng.partial(topo.slot[(pu, pv)])
    np.testing.assert_array_equal(s, d[f"scale_{tag}"])
    ref_p = d[f"partial_{tag}"]
    scale = np.maximum(np.abs(ref_p).max(axis=1, keepdims=True), 1e-300)
    assert np.max(np.abs(p[:len(ref_p)] - ref_p) / scale) < 1e-10
    done = set()
    for i, k in enumerate(d["derv_edges"]):
        u, v = (int(x) for x in g.edges[k])
        node, dad = (v, u) if v >= g.ntaxa else (u, v)
        ops = topo.ops_for(dad, node, done) + topo.ops_for(node, dad, done)
        a, b = topo.ref(dad, node), topo.ref(node, dad)
        for j, L in enumerate(d["derv_lengths"]):
            df, ddf = eng.likelihood_derv(ops if j == 0 else [], a, b, float(L), theta_computed=(j > 0))
            rdf, rddf = d[f"derv_{tag}"][i][j]
            assert abs(df - rdf) <= 1e-9 * max(1.0, abs(rdf)), (k, L, df, rdf)
            assert abs(ddf - rddf) <= 1e-9 * max(1.0, abs(rddf)), (k, L, ddf, rddf)
            assert rel(eng.lnl_from_buffer(float(L)), float(d[f"from_buffer_{tag}"][i][j])) < 1e-10


@pytest.mark.parametrize("name", REF_FIXTURES)
def test_tree_drivers_and_mixed_paths_match_reference(name):
    g = load_ref_golden(name)
    ref = float(g.d["lnl_norm"][0])
    t = engine.GpuTree(g.model, g.patterns, g.freq, g.edges, g.lengths)
    assert rel(t.compute_likelihood(), ref) < 1e-10
    precisions = [engine.F32] + ([engine.TF32X3] if g.model.nstates == 20 else [])
    for prec in precisions:
        tm = engine.GpuTree(g.model, g.patterns, g.freq, g.edges, g.lengths, precision=prec)
        lm = tm.compute_likelihood()
        assert rel(lm, ref) < 1e-6, (prec, lm, ref)
