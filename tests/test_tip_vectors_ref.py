"""models.tip_vectors against the reference's own tip-likelihood rules, read
from its sources as text (skipped without a reference checkout):

* ModelDNA::computeTipLikelihood (model/modeldna.cpp:462-474): states below
  num_states and from 18 on go to ModelSubst; states 4..17 are the bitmask
  state - num_states + 1 over A, C, G, T;
* ModelProtein::computeTipLikelihood (model/modelprotein.cpp:1149-1165): the
  ambi_aa pairs for the three states after the 20 amino acids (B, Z, J);
* ModelSubst::computeTipLikelihood (model/modelsubst.cpp:196-206): a unit
  vector for a plain state, all ones otherwise.
"""
import os
import re

import numpy as np
import pytest

from iqtree2_gb300 import models

REF = os.environ.get("IQTREE_REFERENCE", "/root/reference")

pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(REF, "model", "modeldna.cpp")),
                                reason="no reference checkout")


def _function(path, name):
    src = open(os.path.join(REF, path)).read()
    i = src.index(name)
    j = src.index("{", i)
    depth, k = 0, j
    while True:
        if src[k] == "{":
            depth += 1
        elif src[k] == "}":
            depth -= 1
            if depth == 0:
                return src[j:k + 1]
        k += 1


def _strip_comments(s):
    return re.sub(r"//[^\n]*", "", re.sub(r"/\*.*?\*/", "", s, flags=re.S))


def test_dna_ambiguity_bitmask_matches_reference():
    body = _strip_comments(_function("model/modeldna.cpp", "void ModelDNA::computeTipLikelihood"))
    assert re.search(r"state\s*<\s*num_states\s*\|\|\s*state\s*>=\s*18", body)
    assert re.search(r"cstate\s*=\s*state\s*-\s*num_states\s*\+\s*1", body)
    assert re.search(r"\(\s*cstate\s*\)\s*&\s*\(\s*1\s*<<\s*i\s*\)", body)
    T = models.tip_vectors(4)
    for s in range(4, 18):
        want = [1.0 if ((s - 4 + 1) >> i) & 1 else 0.0 for i in range(4)]
        np.testing.assert_array_equal(T[s], want)


def test_protein_ambiguity_pairs_match_reference():
    body = _strip_comments(_function("model/modelprotein.cpp", "void ModelProtein::computeTipLikelihood"))
    table = re.search(r"ambi_aa\[\]\s*=\s*\{([^}]*)\}", body).group(1)
    pairs = [int(v) for v in re.findall(r"\d+", table)]
    assert len(pairs) == 6
    assert re.search(r"cstate\s*=\s*state\s*-\s*num_states", body)
    T = models.tip_vectors(20)
    for k in range(3):
        want = np.zeros(20)
        want[pairs[2 * k]] = want[pairs[2 * k + 1]] = 1.0
        np.testing.assert_array_equal(T[20 + k], want)


def test_plain_and_unknown_states_match_reference():
    body = _strip_comments(_function("model/modelsubst.cpp", "void ModelSubst::computeTipLikelihood"))
    assert re.search(r"if\s*\(\s*state\s*<\s*num_states\s*\)", body)
    assert re.search(r"state_lk\[\s*state\s*\]\s*=\s*1\.0", body)          # a plain state: unit vector
    assert re.search(r"state_lk\[\s*i\s*\]\s*=\s*1\.0", body)              # otherwise all ones
    for n in (4, 20, 61):
        T = models.tip_vectors(n)
        np.testing.assert_array_equal(T[:n], np.eye(n))
        np.testing.assert_array_equal(T[-1], np.ones(n))  # STATE_UNKNOWN
