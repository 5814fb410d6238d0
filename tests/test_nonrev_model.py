"""Host side of non-reversible models: the UNREST-style builder, its
normalisation and complex eigen system, and the op flag layout."""
import numpy as np
from scipy.linalg import expm

from iqtree2_gb300 import engine, models


def test_unrest_model_normalised_and_eigen_consistent():
    for n, seed in ((4, 1), (20, 2), (61, 3)):
        m = models.unrest_model(n, seed, 0.7)
        assert np.abs(m.Q - m.Q.T).max() > 1e-3                     # not reversible
        assert np.allclose(m.Q.sum(axis=1), 0.0, atol=1e-12)        # rate matrix
        assert abs(m.pi.sum() - 1.0) < 1e-12 and (m.pi > 0).all()
        assert np.abs(m.pi @ m.Q).max() < 1e-12                      # stationary
        assert abs(-(m.pi * np.diag(m.Q)).sum() - 1.0) < 1e-12       # one substitution per unit length
        for t in (0.01, 0.3, 2.0):
            P = m.trans_matrix(t)
            assert np.abs(P - expm(m.Q * t)).max() < 1e-10
            assert np.abs(P.sum(axis=1) - 1.0).max() < 1e-10
        assert m.tip_vec.shape == (m.state_unknown + 1, n)
        assert (m.tip_vec[m.state_unknown] == 1.0).all()


def test_op_flags_layout():
    arr = engine.Engine.ops_array([(3, 0, -2, 0.1, 0.2, engine.OP_TRANSPOSE1 | engine.OP_ROOTLEAF1),
                                   (4, 3, 5, 0.3, 0.4)])
    assert arr["flags"].tolist() == [engine.OP_TRANSPOSE1 | engine.OP_ROOTLEAF1, 0]
    assert engine.OP_DTYPE.itemsize == 32


def test_asc_holder_patterns_layout():
    su = models.STATE_UNKNOWN[4]
    pat = np.array([[0, 3, su], [2, su, 1], [su, 5, 1]], np.uint8)  # DNA; 5 is an ambiguity code
    ext, freq, nobs = models.asc_holder_patterns(pat, np.array([2.0, 1.0, 3.0]), 4)
    assert nobs == 3 and ext.shape == (3, 15) and freq.tolist() == [2.0, 1.0, 3.0] + [0.0] * 12
    # block s = 2, observed pattern 0 (taxa 0 and 1 have data, taxon 2 is missing)
    assert ext[:, 3 + 2 * 3 + 0].tolist() == [2, 2, su]
    # ambiguity codes (>= nstates) count as missing, as in the reference
    assert ext[:, 3 + 1 * 3 + 1].tolist() == [1, su, su]


def test_asc_informative_patterns_are_uninformative_and_distinct():
    p = models.asc_informative_patterns(6, 4)
    cols = {tuple(c) for c in p.T}
    assert len(cols) == p.shape[1]                        # no pattern twice
    for c in p.T:                                         # at most one state occurs twice or more
        counts = np.bincount(c, minlength=4)
        assert (counts >= 2).sum() <= 1
