"""The FP64 drop-in's work-spreading kernels against the oracle, across the
category counts each one takes:

* k_traverse_f64_lanes (4 states on short alignments, one lane per
  (category, state)): 1, 2, 3 and 8 categories = 4, 8, 16 and 32 lanes per
  pattern;
* k_traverse_f64_wide (20 states, up to 4 categories, a warp per state): 1, 2
  and 3 categories;
* k_traverse_f64_cat (21-64 states in SAFE, a CTA per category): 1 and 2
  categories (partials held to 1e-6 there: see its test);

NORM and SAFE where the kernel takes both, on trees long enough that
partials underflow 2^-256. Each forms its sums in the order of the kernel it
stands for, so every partial is within 1e-10 of each pattern's largest entry,
scale counts are identical, branch lnL within 1e-10 relative and the
derivatives within 1e-9.
"""
import dataclasses

import numpy as np
import pytest

from helpers import rel
from iqtree2_gb300 import engine, models, simulate
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu


def _with_ncat(model, ncat, alpha=0.6):
    rates, props = models.gamma_rates_mean(alpha, ncat)
    return dataclasses.replace(model, rates=np.asarray(rates, np.float64), props=np.asarray(props, np.float64))


def _check(oracle_mod, ds, model, safe, partial_tol=1e-10, invar=None):
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    eng = engine.Engine(ds.nptn, model.nstates, model.ncat, ds.ntaxa, model.state_unknown, topo.nslots,
                        safe=safe, max_ops=2 * topo.nslots, flags=engine.FLAG_SAFE_AS_GIVEN)
    eng.set_model(model)
    eng.set_patterns(ds.freq, invar)
    eng.set_tip_states(ds.patterns)
    eng.compute_partials(topo.all_partials_ops())
    orc = oracle_mod.OracleTree(model, ds.patterns, ds.freq, ds.edges, ds.lengths, safe=safe, invar=invar)
    scaled = 0
    for (u, v), slot in topo.slot.items():
        gp, gs = eng.partial(slot)
        op, os_ = orc.partial(u, v)
        np.testing.assert_array_equal(gs, os_)
        if invar is not None:  # a pattern with an invariant-site term is never rescaled
            assert not gs[np.asarray(invar)[:len(gs)] > 0].any(), (u, v)
        scaled += int(gs.sum())
        scale = np.maximum(np.abs(op).max(axis=1, keepdims=True), 1e-300)
        assert np.max(np.abs(gp - op) / scale) < partial_tol, (u, v)
    for (u, v) in ds.edges[:5]:
        u, v = int(u), int(v)
        node, dad = (v, u) if v >= ds.ntaxa else (u, v)
        lg = eng.branch_lnl(topo.ref(dad, node), topo.ref(node, dad), topo.edge_len(node, dad))
        assert rel(lg, orc.lnl_branch(node, dad)) < 1e-10, (u, v, lg)
    n1, n2 = next((int(u), int(v)) for (u, v) in ds.edges if min(int(u), int(v)) >= ds.ntaxa)
    ops = topo.branch_ops(n2, n1)
    df, ddf = eng.likelihood_derv(ops, topo.ref(n1, n2), topo.ref(n2, n1), 0.07)
    odf, oddf = oracle_mod.OracleTree(model, ds.patterns, ds.freq, ds.edges, ds.lengths, safe=safe,
                                      invar=invar).derv(n1, n2, 0.07)
    assert abs(df - odf) <= 1e-9 * max(1.0, abs(odf)) and abs(ddf - oddf) <= 1e-9 * max(1.0, abs(oddf))
    return scaled


@pytest.mark.parametrize("ncat", [1, 2, 3, 8])
@pytest.mark.parametrize("safe", [False, True])
def test_lane_kernel_category_counts(oracle_mod, ncat, safe):
    ds = simulate.dna_gtr_dataset(250, 500, 81, mean_bl=0.5)  # short alignment, long branches
    scaled = _check(oracle_mod, ds, _with_ncat(ds.model, ncat), safe)
    assert scaled > 0  # the 2^-256 path ran


@pytest.mark.parametrize("ncat", [1, 2, 3])
@pytest.mark.parametrize("safe", [False, True])
def test_wide_kernel_category_counts(oracle_mod, ncat, safe):
    ds = simulate.protein_lg_dataset(100, 700, 82, mean_bl=0.5)
    scaled = _check(oracle_mod, ds, _with_ncat(ds.model, ncat), safe)
    assert scaled > 0


@pytest.mark.parametrize("ncat", [1, 2])
def test_category_kernel_counts(oracle_mod, ncat):
    """61 states on a deep long-branch tree: the eigen-space sums cancel, and
    summation orders differ at 1e-7 of a pattern's largest entry (the
    reference's own SIMD and one-lane kernels do on such partials), so the
    partials are held to 1e-6 there; scale counts, lnL and derivatives as
    above."""
    ds = simulate.codon_gy94_dataset(60, 300, 83, mean_bl=0.5)
    scaled = _check(oracle_mod, ds, _with_ncat(ds.model, ncat), True, partial_tol=1e-6)
    assert scaled > 0


def test_category_kernel_invariant_sites(oracle_mod):
    """Codon +I+G4 in SAFE on the per-category kernel: a pattern with an
    invariant-site term is never rescaled (the reference's condition
    lh_max < 2^-256 && ptn_invar == 0), while the others' counts grow; every
    count identical to the oracle, partials, lnL and derivatives as above."""
    ds = simulate.codon_gy94_dataset(60, 300, 84, mean_bl=0.5)
    r, p = models.gamma_invar_rates(0.5, 0.3, 4)
    m = dataclasses.replace(ds.model, rates=np.asarray(r, np.float64), props=np.asarray(p, np.float64))
    inv = models.invariant_site_lh(ds.patterns, m.pi, 0.3, m.nstates)
    assert (inv > 0).sum() > 0
    assert _check(oracle_mod, ds, m, True, partial_tol=1e-6, invar=inv) > 0
