"""The reference's own test alignments as likelihood problems (test helper).

Reads PHYLIP files in place from a reference checkout, converts characters to
IQ-TREE's state codes (Alignment::convertState, alignment/alignment.cpp:
1415-1500: DNA A/C/G/T(U) = 0..3, IUPAC ambiguity codes 4..17 as 3 + the
bitmask of the allowed nucleotides, gaps and N = STATE_UNKNOWN 18; protein
in IQ-TREE's amino-acid order, B/Z/J = 20/21/22, gaps, X, *, U, O = 23),
compresses the columns to patterns with counts, and puts them on a seeded
random tree with a fixed model (DNA GTR+G4, protein LG+G4 with the
alignment's empirical frequencies). Used by tests/golden/make_refgolden.py
and by the CPU tests against the reference oracle.
"""
from __future__ import annotations

import os
from types import SimpleNamespace

import numpy as np

from iqtree2_gb300 import models, simulate

PROTEIN_ORDER = "ARNDCQEGHILKMFPSTWYV"  # IQ-TREE's symbols_protein
DNA_CODES = {"A": 0, "C": 1, "G": 2, "T": 3, "U": 3,
             "R": 3 + 1 + 4, "Y": 3 + 2 + 8, "W": 3 + 1 + 8, "S": 3 + 2 + 4, "M": 3 + 1 + 2,
             "K": 3 + 4 + 8, "B": 3 + 2 + 4 + 8, "H": 3 + 1 + 2 + 8, "D": 3 + 1 + 4 + 8,
             "V": 3 + 1 + 2 + 4}
UNKNOWN_CHARS = set("?-.~")

REF_ALIGNMENTS = {
    "example": ("test_scripts/test_data/example.phy", 4),
    "d59_8": ("test_scripts/test_data/d59_8.phy", 4),
    "prot_M126_27_269": ("test_scripts/test_data/prot_M126_27_269.phy", 20),
}


def read_phylip(path):
    """Sequential or interleaved PHYLIP: names and upper-case sequences."""
    with open(path) as f:
        lines = [ln.rstrip("\n") for ln in f if ln.strip()]
    ntaxa, nsites = map(int, lines[0].split()[:2])
    names, seqs = [], []
    for ln in lines[1:1 + ntaxa]:
        parts = ln.split()
        names.append(parts[0])
        seqs.append("".join(parts[1:]))
    k = 1 + ntaxa
    while any(len(s) < nsites for s in seqs) and k < len(lines):
        for i in range(ntaxa):
            seqs[i] += "".join(lines[k + i].split())
        k += ntaxa
    seqs = [s.upper() for s in seqs]
    if any(len(s) != nsites for s in seqs):
        raise ValueError(f"{path}: sequence lengths differ from {nsites}")
    return names, seqs


def convert_states(seqs, nstates):
    su = models.STATE_UNKNOWN[nstates]
    out = np.empty((len(seqs), len(seqs[0])), np.uint8)
    for i, s in enumerate(seqs):
        for j, ch in enumerate(s):
            if ch in UNKNOWN_CHARS:
                v = su
            elif nstates == 4:
                v = DNA_CODES.get(ch, su)
            else:
                if ch == "B":
                    v = 20
                elif ch == "Z":
                    v = 21
                elif ch == "J":
                    v = 22
                elif ch in PROTEIN_ORDER:
                    v = PROTEIN_ORDER.index(ch)
                else:
                    v = su
            out[i, j] = v
    return out


def compress(states):
    """Unique columns (in order of first appearance) and their counts."""
    cols = np.ascontiguousarray(states.T)
    _, first, inv, counts = np.unique(cols.view([("", cols.dtype)] * cols.shape[1]).ravel(),
                                      return_index=True, return_inverse=True, return_counts=True)
    order = np.argsort(first)
    patterns = states[:, first[order]]
    return np.ascontiguousarray(patterns), counts[order].astype(np.float64)


def empirical_freqs(patterns, freq, nstates):
    cnt = np.zeros(nstates)
    for s in range(nstates):
        cnt[s] = ((patterns == s) * freq[None, :]).sum()
    cnt += 1.0
    return cnt / cnt.sum()


def load(name, reference_dir, seed=17, mean_bl=0.1):
    rel_path, nstates = REF_ALIGNMENTS[name]
    names, seqs = read_phylip(os.path.join(reference_dir, rel_path))
    states = convert_states(seqs, nstates)
    patterns, freq = compress(states)
    ntaxa = len(names)
    rng = np.random.default_rng(seed)
    edges, lengths = simulate.yule_tree(ntaxa, mean_bl, rng)
    if nstates == 4:
        model = models.gtr_model(np.array([1.3, 3.1, 0.8, 1.1, 4.2, 1.0]),
                                 empirical_freqs(patterns, freq, 4), 0.5)
    else:
        model = models.lg_model(empirical_freqs(patterns, freq, 20), 0.8)
    return SimpleNamespace(name=name, nstates=nstates, patterns=patterns, freq=freq, edges=np.asarray(edges),
                           lengths=np.asarray(lengths, np.float64), model=model, ntaxa=ntaxa,
                           nsites=int(states.shape[1]))
