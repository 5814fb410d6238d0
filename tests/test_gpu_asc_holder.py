"""Holder's +ASC for variant sites with missing data (ASC_VARIANT_MISSING)
against the FP64 numpy pruning: every pattern's likelihood from
``stdbasis.tree_lnl`` on the pattern list with the unobserved patterns
appended, then the correction of tree/phylokernelnew.h:3175-3196 (lnL) and
its derivative counterpart (:2580-2617, checked by central differences).

Tolerances: FP64 lnL 1e-10 relative, derivatives 1e-6 relative with a floor
of 1e-6 per site (the central differences' own error); mixed paths lnL 1e-6,
derivatives 1e-4 / 1e-3 relative with a floor of 1e-5 per site.
"""
import numpy as np
import pytest

import stdbasis
from helpers import rel
from iqtree2_gb300 import engine, models, simulate
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu


def _data(kind, seed):
    ds = (simulate.dna_gtr_dataset(12, 800, seed) if kind == "dna"
          else simulate.protein_lg_dataset(10, 400, seed))
    rng = np.random.default_rng(seed)
    pat = ds.patterns.copy()
    pat[rng.random(pat.shape) < 0.15] = ds.model.state_unknown  # missing data
    return ds, pat


def _holder_lnl(m, pat_ext, freq_ext, nobs, edges, lengths, ntaxa):
    _, plh = stdbasis.tree_lnl(m, pat_ext, freq_ext, edges, lengths, ntaxa)
    pc = np.exp(plh[nobs:]).reshape(m.nstates, nobs).sum(axis=0)
    corr = np.log(1.0 - pc)
    return float(((plh[:nobs] - corr) * freq_ext[:nobs]).sum()), plh[:nobs] - corr


@pytest.mark.parametrize("kind,precision,safe", [("dna", engine.F64, False), ("dna", engine.F64, True),
                                                 ("dna", engine.F32, False), ("protein", engine.F64, False),
                                                 ("protein", engine.TF32X3, False)])
def test_asc_holder_lnl_and_derivatives(kind, precision, safe):
    ds, pat = _data(kind, 81)
    m = ds.model
    pat_ext, freq_ext, nobs = models.asc_holder_patterns(pat, ds.freq, m.nstates)
    assert pat_ext.shape[1] == nobs * (m.nstates + 1)
    f64 = precision == engine.F64
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    e = engine.Engine(pat_ext.shape[1], m.nstates, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots,
                      precision=precision, safe=safe)
    try:
        e.set_model(m)
        e.set_patterns(freq_ext)
        e.set_tip_states(pat_ext)
        e.set_asc_holder(nobs)
        k = next(i for i, ed in enumerate(ds.edges) if min(ed) >= ds.ntaxa)
        n1, n2 = map(int, ds.edges[k])
        ops = e.ops_array(topo.ops_for(n1, n2, set()) + topo.ops_for(n2, n1, set()))
        a, b = topo.ref(n1, n2), topo.ref(n2, n1)
        want, pwant = _holder_lnl(m, pat_ext, freq_ext, nobs, ds.edges, ds.lengths, ds.ntaxa)
        got = e.compute_likelihood(ops, a, b, ds.lengths[k])
        assert rel(got, want) < (1e-10 if f64 else 1e-6), (got, want)
        plh = e.pattern_lh()[:nobs]
        np.testing.assert_allclose(plh, pwant, atol=1e-8 if f64 else 1e-4)

        def lnl_at(x):
            lens = ds.lengths.copy()
            lens[k] = x
            return _holder_lnl(m, pat_ext, freq_ext, nobs, ds.edges, lens, ds.ntaxa)[0]
        nsite = float(ds.freq.sum())
        h = 1e-5
        for x in (0.05, 0.3):
            df, ddf = e.likelihood_derv(ops, a, b, x)
            l0, lp, lm = lnl_at(x), lnl_at(x + h), lnl_at(x - h)
            fd1, fd2 = (lp - lm) / (2 * h), (lp - 2 * l0 + lm) / h ** 2
            r1, r2, floor = (1e-6, 1e-3, 1e-6) if f64 else (1e-4, 1e-2, 1e-5)
            assert abs(df - fd1) <= r1 * abs(fd1) + floor * nsite, (df, fd1)
            assert abs(ddf - fd2) <= r2 * abs(fd2) + 1e-5 * nsite, (ddf, fd2)
            assert rel(e.lnl_from_buffer(x), l0) < (1e-10 if f64 else 1e-6)
    finally:
        e.close()


def test_asc_holder_argument_checks():
    ds, pat = _data("dna", 82)
    m = ds.model
    pat_ext, freq_ext, nobs = models.asc_holder_patterns(pat, ds.freq, m.nstates)
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    e = engine.Engine(pat_ext.shape[1], m.nstates, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots)
    try:
        with pytest.raises(engine.EngineError, match="Holder"):
            e.set_asc_holder(nobs + 1)  # the pattern count does not split as nobs * (nstates + 1)
        e.set_asc_holder(nobs)
        with pytest.raises(engine.EngineError):
            engine.Group([e])           # +ASC engines cannot join a group
    finally:
        e.close()


@pytest.mark.parametrize("precision", [engine.F64, engine.F32])
def test_asc_informative(precision):
    """+ASC for informative sites (ASC_INFORMATIVE): Lewis's formula over all
    7,012 uninformative DNA patterns of 12 taxa, appended with weight 0;
    lnL against the numpy pruning, derivatives against its central
    differences."""
    ds = simulate.dna_gtr_dataset(12, 800, 83)
    m = ds.model
    un = models.asc_informative_patterns(ds.ntaxa, m.nstates)
    pat_ext = np.ascontiguousarray(np.concatenate([ds.patterns, un], axis=1))
    freq_ext = np.concatenate([ds.freq, np.zeros(un.shape[1])])
    nsite = float(ds.freq.sum())
    nobs = ds.patterns.shape[1]
    f64 = precision == engine.F64
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)

    def want_at(lens):
        _, plh = stdbasis.tree_lnl(m, pat_ext, freq_ext, ds.edges, lens, ds.ntaxa)
        return float(plh[:nobs] @ ds.freq) - nsite * np.log(1.0 - np.exp(plh[nobs:]).sum())

    e = engine.Engine(pat_ext.shape[1], m.nstates, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots,
                      precision=precision)
    try:
        e.set_model(m)
        e.set_patterns(freq_ext)
        e.set_tip_states(pat_ext)
        e.set_asc(un.shape[1], nsite)
        k = next(i for i, ed in enumerate(ds.edges) if min(ed) >= ds.ntaxa)
        n1, n2 = map(int, ds.edges[k])
        ops = e.ops_array(topo.ops_for(n1, n2, set()) + topo.ops_for(n2, n1, set()))
        a, b = topo.ref(n1, n2), topo.ref(n2, n1)
        got = e.compute_likelihood(ops, a, b, ds.lengths[k])
        assert rel(got, want_at(ds.lengths)) < (1e-10 if f64 else 1e-6)
        h = 1e-5
        for x in (0.05, 0.3):
            lens = [ds.lengths.copy() for _ in range(3)]
            for L, d in zip(lens, (0.0, h, -h)):
                L[k] = x + d
            l0, lp, lm = (want_at(L) for L in lens)
            fd1, fd2 = (lp - lm) / (2 * h), (lp - 2 * l0 + lm) / h ** 2
            df, ddf = e.likelihood_derv(ops, a, b, x)
            r1, floor = (1e-6, 1e-6) if f64 else (1e-4, 1e-5)
            assert abs(df - fd1) <= r1 * abs(fd1) + floor * nsite, (df, fd1)
            assert abs(ddf - fd2) <= 1e-2 * abs(fd2) + 1e-5 * nsite, (ddf, fd2)
            assert rel(e.lnl_from_buffer(x), l0) < (1e-10 if f64 else 1e-6)
    finally:
        e.close()
