"""Shared test helpers: golden fixtures and model wrappers."""
import os
from types import SimpleNamespace

import numpy as np

from iqtree2_gb300 import models

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def model_from_arrays(d):
    n = int(d["nstates"])
    return SimpleNamespace(
        nstates=n, ncat=len(d["rates"]), state_unknown=models.STATE_UNKNOWN.get(n, n),
        eval=np.asarray(d["eval"]), evec=np.asarray(d["evec"]), inv_evec=np.asarray(d["inv_evec"]),
        rates=np.asarray(d["rates"]), props=np.asarray(d["props"]), tip_lh=np.asarray(d["tip_lh"]),
        Q=np.asarray(d["Q"]), pi=np.asarray(d["pi"]))


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return SimpleNamespace(model=model_from_arrays(d), patterns=d["patterns"], freq=d["freq"],
                           edges=d["edges"], lengths=d["lengths"], ntaxa=d["patterns"].shape[0],
                           lnl_std=float(d["lnl_std"]), pattern_lnl_std=d["pattern_lnl_std"])


def jc_model(ncat, alpha):
    return models.gtr_model(np.ones(6), np.full(4, 0.25), alpha, ncat=ncat)


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


REF_FIXTURES = ["example", "d59_8", "prot_M126_27_269", "underflow150", "example_polytomy",
                "underflow150_polytomy"]


def load_ref_golden(name):
    """tests/golden/ref_<name>.npz: inputs and IQ-TREE's own kernel outputs
    (written by tests/golden/make_refgolden.py)."""
    d = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    n = int(d["nstates"])
    model = SimpleNamespace(
        nstates=n, ncat=len(d["rates"]), state_unknown=models.STATE_UNKNOWN.get(n, n),
        eval=np.asarray(d["eval"]), evec=np.asarray(d["evec"]), inv_evec=np.asarray(d["inv_evec"]),
        rates=np.asarray(d["rates"]), props=np.asarray(d["props"]), tip_lh=np.asarray(d["tip_lh"]),
        pi=np.asarray(d["pi"]))
    ntaxa = d["patterns"].shape[0]
    oriented = [(int(u), int(v)) if int(v) < ntaxa else (int(v), int(u)) for (u, v) in d["edges"]]
    return SimpleNamespace(name=name, model=model, patterns=d["patterns"], freq=d["freq"], edges=d["edges"],
                           lengths=d["lengths"], ntaxa=ntaxa, oriented=oriented, d=d)
