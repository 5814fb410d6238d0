"""Slot numbering and post-order traversal lists over the kernel-level C ABI.

Slots follow the engine's tree driver: directed partial (u -> v) with v
internal gets a slot, numbered by node then neighbour order. Tip v is
referenced as -1 - v.
"""
import numpy as np


NO_CHILD = -(2 ** 31)  # absent second child of a multifurcating node's last record
OP_MORE = 16           # more records of the same multifurcating node follow


class Topology:
    def __init__(self, edges, lengths, ntaxa):
        self.ntaxa = ntaxa
        self.nnode = int(np.max(edges)) + 1
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
            # two children per record; a multifurcating node continues over
            # records flagged OP_MORE (tree/phylokernelnew.h:1407-1631)
            if len(kids) == 2:
                (c0, k0), (c1, k1) = kids
                ops.append((self.slot[(d, n)], self.ref(n, c0), self.ref(n, c1), self.lengths[k0],
                            self.lengths[k1]))
            else:
                for i in range(0, len(kids), 2):
                    c0, k0 = kids[i]
                    last = i + 2 >= len(kids)
                    if i + 1 < len(kids):
                        c1, k1 = kids[i + 1]
                        r1, l1 = self.ref(n, c1), self.lengths[k1]
                    else:
                        r1, l1 = NO_CHILD, 0.0
                    ops.append((self.slot[(d, n)], self.ref(n, c0), r1, self.lengths[k0], l1,
                                0 if last else OP_MORE))
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

    def all_partials_ops(self):
        """Ops that make every directed partial of the tree current."""
        done, ops = set(), []
        for (u, v) in sorted(self.slot):
            ops += self.ops_for(u, v, done)
        return ops

    def nni_candidates(self, nmax):
        """Both NNI swaps of internal branches (reference: PhyloTree::getBestNNIForBran,
        tree/phylotree.cpp:4069-4320), up to nmax, as dicts: branch (u, v); n1 = the two
        subtrees at u after the swap, n2 = the two at v."""
        out = []
        for (u, v) in sorted(self.slot):
            if u < self.ntaxa or v < self.ntaxa or u > v:
                continue
            a_, b_ = [w for (w, _) in self.adj[u] if w != v]
            c_, d_ = [w for (w, _) in self.adj[v] if w != u]
            for (x, y) in ((b_, c_), (b_, d_)):  # x leaves u for v, y leaves v for u
                keep_u = a_ if x == b_ else b_
                keep_v = d_ if y == c_ else c_
                out.append(dict(u=u, v=v, n1=(keep_u, y), n2=(x, keep_v)))
                if len(out) == nmax:
                    return out
        return out

    def nni_batch_entries(self, cands, first_scratch):
        """Engine.nni_batch entries for candidates: the four subtree partials with
        their own branch lengths, two scratch slots per candidate starting at
        first_scratch, and the current central length."""
        arr = []
        for k, c in enumerate(cands):
            u, v = c["u"], c["v"]
            old_of = {w: u for (w, _) in self.adj[u]}
            old_of.update({w: v for (w, _) in self.adj[v]})
            subs, lens = [], []
            for s in (c["n1"][0], c["n1"][1], c["n2"][0], c["n2"][1]):
                subs.append(self.ref(old_of[s], s))
                lens.append(self.edge_len(old_of[s], s))
            arr.append((tuple(subs), (first_scratch + 2 * k, first_scratch + 2 * k + 1), tuple(lens),
                        self.edge_len(u, v)))
        return arr


def collapse_edges(edges, lengths, ntaxa, collapse):
    """Contract the internal edges listed in ``collapse`` (edge indices): their
    end nodes merge, so nodes of degree 4, 5, ... (polytomies) appear.
    Returns (edges, lengths, nnode) with internal nodes renumbered ntaxa..;
    neighbour order follows the remaining edges' order."""
    edges = [(int(u), int(v)) for (u, v) in edges]
    parent = {}

    def find(x):
        while parent.get(x, x) != x:
            x = parent[x]
        return x

    for k in collapse:
        u, v = edges[k]
        if u < ntaxa or v < ntaxa:
            raise ValueError("only internal edges can be collapsed")
        a, b = find(u), find(v)
        if a != b:
            parent[max(a, b)] = min(a, b)
    keep = [k for k in range(len(edges)) if k not in set(collapse)]
    label = {}
    out_e, out_l = [], []
    for k in keep:
        u, v = find(edges[k][0]), find(edges[k][1])
        for w in (u, v):
            if w >= ntaxa and w not in label:
                label[w] = ntaxa + len(label)
        out_e.append((label.get(u, u), label.get(v, v)))
        out_l.append(float(lengths[k]))
    return np.asarray(out_e, np.int32), np.asarray(out_l), ntaxa + len(label)
