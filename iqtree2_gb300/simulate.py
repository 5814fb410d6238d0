"""Seeded synthetic alignments for tests and benchmarks.

IQ-TREE's benchmarks here have no public dataset: inputs are simulated under
the named model on a random Yule tree, then compressed into site patterns the
way ``Alignment::addPattern`` does (alignment/alignment.cpp:1126) -- each
distinct column once, with its count as the pattern frequency.

Tree convention used across the engine, the oracle and the tests: an
unrooted binary tree with leaves ``0..ntaxa-1`` and internal nodes
``ntaxa..2*ntaxa-3``, given as an edge list ``edges[k] = (u, v)`` with
``lengths[k]``. A node's neighbour order is the order its edges appear in the
list; traversal tie-breaks follow that order.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import models


def yule_tree(ntaxa, mean_bl, rng):
    """Unrooted tree from a pure-birth (Yule) topology with Exp(mean_bl) branches."""
    if ntaxa < 3:
        raise ValueError("need at least 3 taxa")
    # rooted growth: lineages are (node tokens); split a random lineage each step
    children = {0: []}
    lineages = [0]
    nxt = 1
    parent = {}
    while len(lineages) < ntaxa:
        i = int(rng.integers(len(lineages)))
        node = lineages[i]
        a, b = nxt, nxt + 1
        nxt += 2
        children[node] = [a, b]
        children[a] = []
        children[b] = []
        parent[a] = node
        parent[b] = node
        lineages[i:i + 1] = [a, b]
    # relabel: leaves 0..n-1 in lineage order, internal nodes after
    leaves = lineages
    internal = [t for t in range(nxt) if children[t]]
    label = {t: k for k, t in enumerate(leaves)}
    # root (token 0) is dropped when unrooting; its two children get joined
    root_kids = children[0]
    inner = [t for t in internal if t != 0]
    for k, t in enumerate(inner):
        label[t] = ntaxa + k
    edges = []
    for t in range(1, nxt):
        p = parent[t]
        if p == 0:
            continue
        edges.append((label[p], label[t]))
    edges.append((label[root_kids[0]], label[root_kids[1]]))
    edges = np.array(edges, dtype=np.int32)
    lengths = rng.exponential(mean_bl, size=len(edges))
    assert len(edges) == 2 * ntaxa - 3
    return edges, lengths


def adjacency(ntaxa, edges):
    nnode = 2 * ntaxa - 2
    adj = [[] for _ in range(nnode)]
    for k, (u, v) in enumerate(edges):
        adj[u].append((v, k))
        adj[v].append((u, k))
    return adj


def simulate_alignment(ntaxa, edges, lengths, model, nsites, rng):
    """Evolve ``nsites`` sites down the tree; returns uint8 states (ntaxa, nsites)."""
    n = model.nstates
    adj = adjacency(ntaxa, edges)
    root = ntaxa  # first internal node
    cat = rng.integers(model.ncat, size=nsites) if model.ncat > 1 else np.zeros(nsites, np.int64)
    cum_pi = np.cumsum(model.pi)
    states = {root: np.minimum(np.searchsorted(cum_pi, rng.random(nsites) * cum_pi[-1]), n - 1)}
    stack = [(root, -1)]
    offs = np.arange(n, dtype=np.float64)[:, None]
    while stack:
        node, dad = stack.pop()
        for (nb, k) in adj[node]:
            if nb == dad:
                continue
            parent_states = states[node]
            child = np.empty(nsites, dtype=np.int64)
            for c in range(model.ncat):
                idx = np.nonzero(cat == c)[0]
                if idx.size == 0:
                    continue
                P = model.trans_matrix(model.rates[c] * lengths[k])
                P = np.clip(P, 0.0, None)
                P /= P.sum(axis=1, keepdims=True)
                cum = np.cumsum(P, axis=1)
                cum[:, -1] = 1.0
                flat = (cum + offs).ravel()
                ps = parent_states[idx]
                pos = np.searchsorted(flat, rng.random(idx.size) + ps, side="right")
                child[idx] = np.minimum(pos - ps * n, n - 1)
            states[nb] = child
            stack.append((nb, node))
    return np.stack([states[t] for t in range(ntaxa)]).astype(np.uint8)


def compress_patterns(aln):
    """Distinct columns (ntaxa, nptn) and their counts as float64 weights."""
    cols, counts = np.unique(np.ascontiguousarray(aln.T), axis=0, return_counts=True)
    return np.ascontiguousarray(cols.T.astype(np.uint8)), counts.astype(np.float64)


@dataclass
class Dataset:
    name: str
    ntaxa: int
    nsites: int
    edges: np.ndarray
    lengths: np.ndarray
    model: models.SubstModel
    patterns: np.ndarray  # (ntaxa, nptn) uint8
    freq: np.ndarray      # (nptn,) float64

    @property
    def nptn(self):
        return self.patterns.shape[1]

    @property
    def n_internal(self):
        return self.ntaxa - 2


def dna_gtr_dataset(ntaxa, nsites, seed, mean_bl=0.1, alpha=0.5):
    """DNA GTR+G4: exchangeabilities ~U(0.5,3), pi ~ Dirichlet(5,5,5,5)."""
    rng = np.random.default_rng(seed)
    exch = rng.uniform(0.5, 3.0, size=6)
    pi = rng.dirichlet([5.0, 5.0, 5.0, 5.0])
    model = models.gtr_model(exch, pi, alpha)
    edges, lengths = yule_tree(ntaxa, mean_bl, rng)
    aln = simulate_alignment(ntaxa, edges, lengths, model, nsites, rng)
    pats, freq = compress_patterns(aln)
    return Dataset(f"dna{ntaxa}x{nsites}", ntaxa, nsites, edges, lengths, model, pats, freq)


def partitioned_dna_datasets(ntaxa, sizes, seed, mean_bl=0.1):
    """Partitions on one shared tree (edge-linked, equal branch lengths), each
    with its own GTR+G4 (exchangeabilities, frequencies, alpha) and site count:
    the shape of a PhyloSuperTree with separate models per partition."""
    rng = np.random.default_rng(seed)
    edges, lengths = yule_tree(ntaxa, mean_bl, rng)
    out = []
    for k, nsites in enumerate(sizes):
        exch = rng.uniform(0.5, 3.0, size=6)
        pi = rng.dirichlet([5.0, 5.0, 5.0, 5.0])
        model = models.gtr_model(exch, pi, float(rng.uniform(0.3, 1.5)))
        aln = simulate_alignment(ntaxa, edges, lengths, model, int(nsites), rng)
        pats, freq = compress_patterns(aln)
        out.append(Dataset(f"part{k}_dna{ntaxa}x{nsites}", ntaxa, int(nsites), edges, lengths, model, pats, freq))
    return out


def protein_lg_dataset(ntaxa, nsites, seed, mean_bl=0.05, alpha=0.8):
    """LG+G4 simulated with LG frequencies; the model then uses the empirical
    frequencies of the sampled alignment (the reference's +F)."""
    rng = np.random.default_rng(seed)
    _, lg_pi = models.lg_exchangeabilities()
    sim_model = models.lg_model(lg_pi, alpha)
    edges, lengths = yule_tree(ntaxa, mean_bl, rng)
    aln = simulate_alignment(ntaxa, edges, lengths, sim_model, nsites, rng)
    counts = np.bincount(aln.ravel(), minlength=20)[:20].astype(np.float64) + 1e-3
    model = models.lg_model(counts / counts.sum(), alpha)
    pats, freq = compress_patterns(aln)
    return Dataset(f"prot{ntaxa}x{nsites}", ntaxa, nsites, edges, lengths, model, pats, freq)


def codon_gy94_dataset(ntaxa, ncodons, seed, mean_bl=0.1, alpha=0.5, kappa=2.0, omega=0.3):
    """GY94+G4 over 61 sense codons with F3x4 frequencies drawn from the seed."""
    rng = np.random.default_rng(seed)
    nt = np.stack([rng.dirichlet([5.0] * 4) for _ in range(3)])
    pi = models.f3x4_frequencies(nt)
    model = models.gy94_model(kappa, omega, pi, alpha)
    edges, lengths = yule_tree(ntaxa, mean_bl, rng)
    aln = simulate_alignment(ntaxa, edges, lengths, model, ncodons, rng)
    pats, freq = compress_patterns(aln)
    return Dataset(f"codon{ntaxa}x{ncodons}", ntaxa, ncodons, edges, lengths, model, pats, freq)


def bootstrap_weights(freq, nreps, rng):
    """UFBoot replicate weights: multinomial(nsites) over sites mapped to patterns
    (Alignment::createBootstrapAlignment, alignment/alignment.cpp:3795-3830)."""
    nsites = int(round(freq.sum()))
    p = freq / freq.sum()
    return rng.multinomial(nsites, p, size=nreps).astype(np.float32)


def _preorder_edges(ntaxa, edges):
    """Edges oriented away from the first internal node, in preorder."""
    adj = adjacency(ntaxa, edges)
    root = ntaxa
    par, ch, order = [], [], []
    stack = [(root, -1)]
    while stack:
        node, dad = stack.pop()
        for (nb, k) in adj[node]:
            if nb == dad:
                continue
            par.append(node)
            ch.append(nb)
            order.append(k)
            stack.append((nb, node))
    return np.array(par, np.int32), np.array(ch, np.int32), np.array(order)


def device_alignment(ntaxa, edges, lengths, model, nsites, seed, device=0):
    """Simulate on the GPU (iqgpu_simulate); returns uint8 states (ntaxa, nsites)."""
    import ctypes as ct

    from . import engine
    par, ch, order = _preorder_edges(ntaxa, edges)
    n, C = model.nstates, model.ncat
    cum = np.empty((len(order), C, n, n), np.float32)
    for j, k in enumerate(order):
        for c in range(C):
            P = np.clip(model.trans_matrix(model.rates[c] * lengths[k]), 0.0, None)
            P /= P.sum(axis=1, keepdims=True)
            cp = np.cumsum(P, axis=1)
            cp[:, -1] = 1.0
            cum[j, c] = cp
    cpi = np.cumsum(model.pi).astype(np.float32)
    cpi[-1] = 1.0
    out = np.empty((ntaxa, nsites), np.uint8)
    L = engine.lib()
    f = L.iqgpu_simulate
    f.argtypes = [ct.c_int32, ct.c_int64, ct.c_int32, ct.c_int32, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                  ct.c_void_p, ct.c_uint64, ct.c_int32, ct.c_void_p]
    f.restype = ct.c_int
    engine._check(f(ntaxa, nsites, n, C, par.ctypes.data, ch.ctypes.data, cum.ctypes.data, cpi.ctypes.data,
                    int(seed) & 0xFFFFFFFFFFFFFFFF, device, out.ctypes.data))
    return out


def serving_dataset(kind, ntaxa, nsites, seed, compress_below=20000):
    """A serving request: DNA GTR+G4 or protein LG+G4 simulated on the device.
    Alignments up to ``compress_below`` sites are compressed into patterns;
    larger ones keep one pattern per site (weight 1), the same likelihood."""
    rng = np.random.default_rng(seed)
    if kind == "dna":
        model = models.gtr_model(rng.uniform(0.5, 3.0, size=6), rng.dirichlet([5.0] * 4), 0.5)
        mean_bl = 0.1
    else:
        _, lg_pi = models.lg_exchangeabilities()
        model = models.lg_model(lg_pi, 0.8)
        mean_bl = 0.05
    edges, lengths = yule_tree(ntaxa, mean_bl, rng)
    aln = device_alignment(ntaxa, edges, lengths, model, nsites, int(rng.integers(1 << 62)))
    if nsites <= compress_below:
        pats, freq = compress_patterns(aln)
    else:
        pats, freq = aln, np.ones(nsites)
    return Dataset(f"{kind}{ntaxa}x{nsites}", ntaxa, nsites, edges, lengths, model, pats, freq)
