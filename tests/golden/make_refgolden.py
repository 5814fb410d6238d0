"""Golden vectors from IQ-TREE 2's own compiled likelihood kernels.

Runs the reference oracle (``oracle/_ref/libiqref.so``: the reference's
tree/phylokernelnew.h templates compiled from a reference checkout, one-lane
kernels) on

* the reference's own test alignments (test_scripts/test_data/example.phy,
  d59_8.phy and prot_M126_27_269.phy, read in place and compressed to
  patterns by ``tests/refdata.py``) on a seeded random tree with fixed
  GTR+G4 / LG+G4 models, and
* ``underflow150``: a seeded 150-taxon protein alignment on a long-branch
  tree whose partials fall below 2^-256, so NORM and SAFE scale counts are
  exercised,
* ``example_polytomy`` and ``underflow150_polytomy``: the same with internal
  edges contracted, so multifurcating nodes (degree 4 and more) run the
  reference's multifurcating update,

and writes ``ref_<name>.npz`` here: the inputs (patterns, weights, tree,
the model's eigen arrays) and the reference kernels' outputs (branch lnL on
every edge, pattern lnL, derivatives and lnL-from-buffer on chosen branches,
the partial of all taxa but one with its scale counts, NORM and SAFE). The GPU tests
check the FP64 drop-in against these files on a machine without the
reference checkout.

Run from the repository root, where a reference checkout exists:
``python tests/golden/make_refgolden.py [/path/to/iqtree2]``.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(HERE)):
    sys.path.insert(0, p)

from iqtree2_gb300 import simulate, topology  # noqa: E402
import refdata  # noqa: E402
import refkernels  # noqa: E402

DERV_LENGTHS = (0.02, 0.7)
PARTIAL_PATTERNS = 64  # partial values kept for the first patterns only (scale counts for all)


def underflow150():
    ds = simulate.protein_lg_dataset(150, 40, 11, mean_bl=0.5)
    from types import SimpleNamespace
    return SimpleNamespace(name="underflow150", patterns=ds.patterns, freq=ds.freq, edges=np.asarray(ds.edges),
                           lengths=np.asarray(ds.lengths, np.float64), model=ds.model, ntaxa=ds.ntaxa,
                           nsites=int(round(float(np.sum(ds.freq)))))


def polytomy(d, ncollapse, name):
    """d with ncollapse internal edges contracted: nodes of degree 4 and more
    (the reference's multifurcating update, tree/phylokernelnew.h:1407-1631)."""
    from types import SimpleNamespace
    internal = [k for k, (u, v) in enumerate(d.edges) if min(int(u), int(v)) >= d.ntaxa]
    rng = np.random.default_rng(5)
    pick = sorted(rng.choice(internal, size=ncollapse, replace=False).tolist())
    e2, l2, _ = topology.collapse_edges(d.edges, d.lengths, d.ntaxa, pick)
    return SimpleNamespace(name=name, patterns=d.patterns, freq=d.freq, edges=e2, lengths=l2, model=d.model,
                           ntaxa=d.ntaxa, nsites=d.nsites)


def branches(d):
    """(node, dad) per edge with the dad a leaf where the edge has one, and a
    few branches for the derivatives: edge 0 and two internal ones."""
    nd = []
    for (u, v) in d.edges:
        u, v = int(u), int(v)
        nd.append((u, v) if v < d.ntaxa else (v, u))
    internal = [k for k, (u, v) in enumerate(d.edges) if min(u, v) >= d.ntaxa]
    return nd, [0] + internal[:2]


def run(d):
    out = dict(patterns=d.patterns, freq=d.freq, edges=d.edges.astype(np.int32), lengths=d.lengths,
               nstates=d.model.nstates, eval=d.model.eval, evec=d.model.evec, inv_evec=d.model.inv_evec,
               rates=d.model.rates, props=d.model.props, tip_lh=d.model.tip_lh, pi=d.model.pi,
               nsites=d.nsites, derv_lengths=np.array(DERV_LENGTHS))
    nd, derv_edges = branches(d)
    out["derv_edges"] = np.array(derv_edges, np.int32)
    # the largest partial: the subtree of every taxon but one, seen from that
    # leaf (where scale counts accumulate most)
    e0 = next(k for k, (u, v) in enumerate(d.edges) if 0 in (int(u), int(v)))
    pu, pv = 0, int(d.edges[e0][0]) + int(d.edges[e0][1])
    out["partial_branch"] = np.array([pu, pv], np.int32)
    for safe in (False, True):
        tag = "safe" if safe else "norm"
        r = refkernels.RefTree(d.model, d.patterns, d.freq, d.edges, d.lengths, safe=safe, kind=0,
                               nsite=d.nsites)
        lnl = np.array([r.branch_lnl(node, dad) for (node, dad) in nd])
        node, dad = nd[0]
        _, plh = r.branch_lnl(node, dad, want_pattern_lh=True)
        dv, fb = [], []
        for k in derv_edges:
            r2 = refkernels.RefTree(d.model, d.patterns, d.freq, d.edges, d.lengths, safe=safe, kind=0,
                                    nsite=d.nsites)
            u, v = (int(x) for x in d.edges[k])
            row, fbrow = [], []
            for L in DERV_LENGTHS:
                r2.set_length(k, L)
                df, ddf = r2.derv(u, v)
                row.append((df, ddf))
                fbrow.append(r2.from_buffer(L))
            dv.append(row)
            fb.append(fbrow)
        part, scale = r.partial(pu, pv)
        out[f"lnl_{tag}"] = lnl
        out[f"pattern_lnl_{tag}"] = plh
        out[f"derv_{tag}"] = np.array(dv)          # [edge][length][df, ddf]
        out[f"from_buffer_{tag}"] = np.array(fb)   # [edge][length]
        out[f"partial_{tag}"] = part[:PARTIAL_PATTERNS]
        out[f"scale_{tag}"] = scale
        print(f"  {d.name} {tag}: lnL {lnl[0]:.10f}, scale counts in the partial: {int(scale.sum())}")
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else refkernels.reference_dir()
    if not ref:
        raise SystemExit("no reference checkout (pass its path or set IQTREE_REFERENCE)")
    os.environ["IQTREE_REFERENCE"] = ref
    sets = [refdata.load(name, ref) for name in refdata.REF_ALIGNMENTS] + [underflow150()]
    sets += [polytomy(sets[0], 10, "example_polytomy"), polytomy(sets[3], 25, "underflow150_polytomy")]
    for d in sets:
        out = run(d)
        np.savez_compressed(os.path.join(HERE, f"ref_{d.name}.npz"), **out)
        print(f"wrote ref_{d.name}.npz ({os.path.getsize(os.path.join(HERE, f'ref_{d.name}.npz'))} bytes)")


if __name__ == "__main__":
    main()
