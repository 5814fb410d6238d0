"""Slot numbering and post-order traversal lists over the kernel-level C ABI.

Slots follow the engine's tree driver: directed partial (u -> v) with v
internal gets a slot, numbered by node then neighbour order. Tip v is
referenced as -1 - v.
"""
import numpy as np


class Topology:
    def __init__(self, edges, lengths, ntaxa):
        self.ntaxa = ntaxa
        self.nnode = 2 * ntaxa - 2
        self.adj = [[] for _ in range(self.nnode)]
        for k, (u, v) in enumerate(edges):
            self.adj[int(u)].append((int(v), k))
            self.adj[int(v)].append((int(u), k))
        self.lengths = np.asarray(lengths, np.float64)
        self.slot = {}
        for u in range(self.nnode):
            for (v, _) in self.adj[u]:
                if v >= ntaxa:
                    self.slot[(u, v)] = len(self.slot)
        self.nslots = len(self.slot)

    def ref(self, u, v):
        return -1 - v if v < self.ntaxa else self.slot[(u, v)]

    def ops_for(self, dad, node, done=None):
        """Post-order ops computing partial dad->node (and everything below)."""
        done = set() if done is None else done
        ops = []

        def rec(d, n):
            if n < self.ntaxa or (d, n) in done:
                return
            kids = [(c, k) for (c, k) in self.adj[n] if c != d]
            for (c, _) in kids:
                rec(n, c)
            (c0, k0), (c1, k1) = kids
            ops.append((self.slot[(d, n)], self.ref(n, c0), self.ref(n, c1), self.lengths[k0], self.lengths[k1]))
            done.add((d, n))

        rec(dad, node)
        return ops

    def branch_ops(self, node, dad):
        done = set()
        return self.ops_for(dad, node, done) + self.ops_for(node, dad, done)

    def edge_len(self, u, v):
        for (w, k) in self.adj[u]:
            if w == v:
                return self.lengths[k]
        raise KeyError
