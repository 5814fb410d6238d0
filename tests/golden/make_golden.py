"""Generate the committed golden fixtures in this directory.

The reference has no golden vectors for its likelihood kernels, so these
fixtures pin the path with values that do not come from the code under test:

* ``kat_jc.npz`` -- closed-form JC69 likelihoods of two observed taxa joined
  through a third, fully unknown taxon (its tip vector is all ones, so the
  likelihood is that of the pair at distance t0+t1), for one rate category
  and for +G4, plus the closed-form ML distance -3/4 ln(1 - 4p/3).
* ``dna16.npz``, ``prot12.npz``, ``codon8.npz`` -- small seeded datasets
  (tree, model arrays, patterns) with the lnL of an independent
  standard-basis pruning (scipy ``expm`` of Q, no eigen-decomposition).

Run from the repository root: ``python tests/golden/make_golden.py``.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from iqtree2_gb300 import models, simulate  # noqa: E402
import stdbasis  # noqa: E402


def jc_pair_lnl(pairs, freq, d, rates, props):
    same = np.zeros_like(d, dtype=float)
    diff = np.zeros_like(d, dtype=float)
    for r, p in zip(rates, props):
        e = np.exp(-4.0 * r * d / 3.0)
        same += p * (0.25 + 0.75 * e)
        diff += p * (0.25 - 0.25 * e)
    P = np.where(pairs[0] == pairs[1], same, diff)
    return float(np.sum(freq * np.log(0.25 * P)))


def kat_jc():
    rng = np.random.default_rng(7)
    s0, s1 = np.meshgrid(np.arange(4), np.arange(4), indexing="ij")
    pairs = np.stack([s0.ravel(), s1.ravel()])
    freq = rng.integers(1, 30, size=16).astype(np.float64)
    freq[pairs[0] == pairs[1]] += 60.0  # mostly identical sites
    patterns = np.stack([pairs[0], pairs[1], np.full(16, 18)]).astype(np.uint8)
    edges = np.array([[3, 0], [3, 1], [3, 2]], np.int32)
    lengths = np.array([0.07, 0.11, 0.3])
    out = dict(patterns=patterns, freq=freq, edges=edges, lengths=lengths)
    for tag, alpha, ncat in (("g1", 1.0, 1), ("g4", 0.5, 4)):
        m = models.gtr_model(np.ones(6), np.full(4, 0.25), alpha, ncat=ncat)
        out[f"rates_{tag}"] = m.rates
        out[f"lnl_{tag}"] = jc_pair_lnl(pairs, freq, lengths[0] + lengths[1], m.rates, m.props)
    p_hat = float(freq[pairs[0] != pairs[1]].sum() / freq.sum())
    out["ml_distance_g1"] = -0.75 * np.log(1.0 - 4.0 * p_hat / 3.0)
    np.savez(os.path.join(HERE, "kat_jc.npz"), **out)


def dataset_fixture(name, ds):
    m = ds.model
    lnl, plh = stdbasis.tree_lnl(m, ds.patterns, ds.freq, ds.edges, ds.lengths, ds.ntaxa)
    np.savez(os.path.join(HERE, f"{name}.npz"), patterns=ds.patterns, freq=ds.freq, edges=ds.edges,
             lengths=ds.lengths, nstates=m.nstates, Q=m.Q, pi=m.pi, rates=m.rates, props=m.props,
             eval=m.eval, evec=m.evec, inv_evec=m.inv_evec, tip_lh=m.tip_lh, lnl_std=lnl, pattern_lnl_std=plh)


def main():
    kat_jc()
    dataset_fixture("dna16", simulate.dna_gtr_dataset(16, 1000, 1))
    dataset_fixture("prot12", simulate.protein_lg_dataset(12, 300, 2))
    dataset_fixture("codon8", simulate.codon_gy94_dataset(8, 200, 3))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
