"""Independent standard-basis Felsenstein pruning in numpy (test helper).

Uses P(t) = expm(Q*r*t) from scipy instead of the eigen-decomposition, stores
partials in the standard basis and rescales every node by its per-pattern
maximum, tracking the log of the factor. It shares no code with the oracle
or the engine, so agreement pins both to the textbook likelihood.
"""
import numpy as np
from scipy.linalg import expm


def tree_lnl(model, patterns, freq, edges, lengths, ntaxa, root=None, invar=None):
    nnode = 2 * ntaxa - 2
    adj = [[] for _ in range(nnode)]
    for k, (u, v) in enumerate(edges):
        adj[u].append((v, k))
        adj[v].append((u, k))
    tips = np.asarray(__import__("iqtree2_gb300.models", fromlist=["x"]).tip_vectors(model.nstates))
    nptn = patterns.shape[1]
    C = model.ncat

    def partial(node, dad):
        # returns (C, nptn, n) standard-basis partial and per-pattern log scale
        if node < ntaxa:
            v = tips[patterns[node]]  # (nptn, n)
            return np.broadcast_to(v, (C, nptn, model.nstates)).copy(), np.zeros(nptn)
        out = np.ones((C, nptn, model.nstates))
        logs = np.zeros(nptn)
        for (ch, k) in adj[node]:
            if ch == dad:
                continue
            cp, cl = partial(ch, node)
            for c in range(C):
                P = expm(model.Q * model.rates[c] * lengths[k])
                out[c] *= cp[c] @ P.T
            logs += cl
        mx = out.max(axis=(0, 2))
        mx = np.where(mx > 0, mx, 1.0)
        out /= mx[None, :, None]
        return out, logs + np.log(mx)

    r = ntaxa if root is None else root
    out = np.ones((C, nptn, model.nstates))
    logs = np.zeros(nptn)
    for (ch, k) in adj[r]:
        cp, cl = partial(ch, r)
        for c in range(C):
            P = expm(model.Q * model.rates[c] * lengths[k])
            out[c] *= cp[c] @ P.T
        logs += cl
    lh = np.einsum("cpx,x,c->p", out, model.pi, model.props)
    if invar is not None:  # +I: the invariant-site term, in the same scaled units
        lh = lh + np.asarray(invar) * np.exp(-logs)
    plh = np.log(lh) + logs
    return float(plh @ freq), plh


def tree_lnl_mixture(mix, patterns, freq, edges, lengths, ntaxa, root=None):
    """Mixture-model pruning in the standard basis: category c uses the Q and
    the root frequencies of its class; lh = sum_c p_c sum_x pi_m(c)[x] L_c[x]."""
    nnode = 2 * ntaxa - 2
    adj = [[] for _ in range(nnode)]
    for k, (u, v) in enumerate(edges):
        adj[u].append((v, k))
        adj[v].append((u, k))
    tips = np.asarray(__import__("iqtree2_gb300.models", fromlist=["x"]).tip_vectors(mix.nstates))
    nptn = patterns.shape[1]
    C, cls, rates = mix.ncat, mix.cat_class, mix.rates
    Qs = [c.Q for c in mix.classes]

    def partial(node, dad):
        if node < ntaxa:
            v = tips[patterns[node]]
            return np.broadcast_to(v, (C, nptn, mix.nstates)).copy(), np.zeros(nptn)
        out = np.ones((C, nptn, mix.nstates))
        logs = np.zeros(nptn)
        for (ch, k) in adj[node]:
            if ch == dad:
                continue
            cp, cl = partial(ch, node)
            for c in range(C):
                P = expm(Qs[cls[c]] * rates[c] * lengths[k])
                out[c] *= cp[c] @ P.T
            logs += cl
        mx = out.max(axis=(0, 2))
        mx = np.where(mx > 0, mx, 1.0)
        out /= mx[None, :, None]
        return out, logs + np.log(mx)

    r = ntaxa if root is None else root
    out = np.ones((C, nptn, mix.nstates))
    logs = np.zeros(nptn)
    for (ch, k) in adj[r]:
        cp, cl = partial(ch, r)
        for c in range(C):
            P = expm(Qs[cls[c]] * rates[c] * lengths[k])
            out[c] *= cp[c] @ P.T
        logs += cl
    lh = np.einsum("cpx,cx,c->p", out, mix.pi[cls], mix.props)
    plh = np.log(lh) + logs
    return float(plh @ freq), plh


def branch_lnl_nonrev(model, patterns, freq, edges, lengths, ntaxa, dad, node, weights=None, blen=None,
                      derivatives=False):
    """lnL of a non-reversible model evaluated on branch (dad, node): per
    pattern sum_c p_c sum_x w_x A_c[x] (P_c(t) B_c)[x], A the conditional
    likelihood of dad's side (edges directed away from dad), B node's side,
    P_c(t) = expm(Q r_c t) straight from the rate matrix (no eigen system).
    w defaults to the stationary frequencies (the unrooted convention);
    ``blen`` overrides the branch's length. With ``derivatives`` also the
    Newton-Raphson sums df = sum f lh'/lh and ddf = sum f (lh''/lh -
    (lh'/lh)^2), dP/dt = r Q P and d2P/dt2 = (r Q)^2 P."""
    from iqtree2_gb300 import models
    w = model.pi if weights is None else np.asarray(weights, np.float64)
    T = models.tip_vectors(model.nstates)
    adj = [[] for _ in range(2 * ntaxa - 2)]
    for k, (u, v) in enumerate(edges):
        adj[int(u)].append((int(v), k))
        adj[int(v)].append((int(u), k))
    lengths = np.asarray(lengths, np.float64).copy()
    Ps = {}

    def P(c, t):
        key = (c, t)
        if key not in Ps:
            Ps[key] = expm(model.Q * (model.rates[c] * t))
        return Ps[key]

    def cond(n, d):  # [C, nptn, n] conditional likelihood of n's subtree seen from d
        if n < ntaxa:
            v = T[patterns[n]]
            return np.broadcast_to(v, (model.ncat,) + v.shape).copy()
        out = None
        for (c, k) in adj[n]:
            if c == d:
                continue
            L = cond(c, n)
            m = np.stack([L[ci] @ P(ci, lengths[k]).T for ci in range(model.ncat)])
            out = m if out is None else out * m
        return out

    k_b = next(k for (c, k) in adj[dad] if c == node)
    t = lengths[k_b] if blen is None else blen
    A, B = cond(dad, node), cond(node, dad)
    lh, d1, d2 = (np.zeros(patterns.shape[1]) for _ in range(3))
    for ci in range(model.ncat):
        Pt = P(ci, t)
        rQ = model.Q * model.rates[ci]
        Aw = A[ci] * w[None, :]
        lh += model.props[ci] * (Aw * (B[ci] @ Pt.T)).sum(axis=1)
        d1 += model.props[ci] * (Aw * (B[ci] @ (rQ @ Pt).T)).sum(axis=1)
        d2 += model.props[ci] * (Aw * (B[ci] @ (rQ @ rQ @ Pt).T)).sum(axis=1)
    lnl = float((np.log(lh) * freq).sum())
    if not derivatives:
        return lnl
    return lnl, float((freq * d1 / lh).sum()), float((freq * (d2 / lh - (d1 / lh) ** 2)).sum())
