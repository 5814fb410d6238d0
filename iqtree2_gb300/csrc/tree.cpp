// PhyloTree drivers over the kernel-level C ABI.
//
// This is the host half of the drop-in: the same control flow as IQ-TREE 2's
// PhyloTree around its kernel function pointers, restated in C++ on top of
// iqgpu_compute_likelihood / iqgpu_likelihood_derv / iqgpu_lnl_from_buffer:
//   traversal of stale partials   tree/phylotree.cpp:5918-6028 and
//                                 tree/phylokernelnew.h:1145-1200
//   computeLikelihood             tree/phylotree.cpp:1233-1280
//   computeFuncDerv               tree/phylotree.cpp:2529-2536
//   optimizeOneBranch             tree/phylotree.cpp:2594-2644
//   optimizeAllBranches           tree/phylotree.cpp:2698-2774
//   computeBestTraversal          tree/phylotree.cpp:2689 with
//   findFarthestLeaf / getPreOrderBranches  tree/mtree.cpp:3040-3082
//   minimizeNewton                utils/optimization.cpp:422-499
//   clearReversePartialLh         tree/phylonode.cpp:22-33
// Every directed partial of an internal subtree owns one HBM slot (three per
// internal node), so a branch-length change only recomputes the partials it
// invalidates, as with the reference's per-neighbour partial_lh buffers.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/iqgpu.h"

namespace iqg {
void set_error(const std::string &msg);
bool newton_on_device(const iqgpu_engine *e);
bool pass_served(const iqgpu_engine *e);
int run_pass(iqgpu_engine *e, const iqgpu_op *ops, const int32_t *edges, const int32_t *off, const int32_t *ab,
             const int32_t *bedge, int nb, const double *lengths, int nedge, double x1, double x2, double xacc,
             int max_steps, double *res);
}

// largest node degree (a multifurcating node of degree d has d - 1 children)
constexpr int kMaxDeg = 32;

struct iqgpu_tree {
    iqgpu_engine *e;
    int64_t nptn;
    int ntaxa, nnode, nedge;
    std::vector<int> deg;
    std::vector<int> nbr, edge;        // [node*kMaxDeg + j]
    std::vector<uint8_t> computed;     // [node*kMaxDeg + j]: partial of node->nbr valid (and resident)
    std::vector<double> len;
    std::vector<int> height;
    std::vector<iqgpu_op> ops;         // records not yet executed
    std::vector<int32_t> op_edge;      // [2 per record]: the edge of each child's length (-1: none)
    int64_t nupdates = 0;
    double min_bl = 1e-6, max_bl = 10.0;
    int cur1 = -1, cur2 = -1;  // current_it: cur1 -> cur2
    bool theta_computed = false;
    // minimizeNewton through iqgpu_newton_branch where the engine serves it:
    // 1 whole passes of optimizeAllBranches on the device, 2 one branch at a time
    int device_newton = 1;
    int last_rc = IQGPU_OK;

    // HBM slots. A tree may have more directed internal partials than its
    // engine has slots (a job larger than its memory): partials then share the
    // slots least-recently-used first, as MemSlotVector does under LM_MEM_SAVE
    // (tree/memslot.h:44-74, tree/phylotree.cpp:967-1027), and are recomputed
    // when needed again. A slot is never reassigned while an op that is not
    // yet executed reads or writes it (pending) or an op that is not yet built
    // will read it (pins); subtrees are walked larger first, so only about
    // log2(ntaxa) partials are pinned at once.
    int nslots = 0;
    std::vector<int> slot_of;          // [node*kMaxDeg + j]: slot holding that partial, or -1
    std::vector<int> owner;            // [slot]: the directed partial it holds, or -1
    std::vector<int64_t> stamp;        // [slot]: last use
    std::vector<int> pins;             // [slot]
    std::vector<uint8_t> pending;      // [slot]
    std::vector<int> free_slots;
    std::vector<int> leaves;           // [node*kMaxDeg + j]: leaves behind that directed edge (0 = not yet known)
    int64_t tick = 0;
    int walk_rc = IQGPU_OK;

    bool leaf(int u) const { return u < ntaxa; }
    int idx(int u, int v) const {
        for (int j = 0; j < deg[u]; j++)
            if (nbr[u * kMaxDeg + j] == v) return j;
        return -1;
    }
    double &blen(int u, int v) { return len[edge[u * kMaxDeg + idx(u, v)]]; }
    int leaves_behind(int dad, int node) {
        if (leaf(node)) return 1;
        int &c = leaves[dad * kMaxDeg + idx(dad, node)];
        if (c == 0)
            for (int q = 0; q < deg[node]; q++)
                if (nbr[node * kMaxDeg + q] != dad) c += leaves_behind(node, nbr[node * kMaxDeg + q]);
        return c;
    }
    void evict(int s) {
        if (owner[s] >= 0) {
            computed[owner[s]] = 0;
            slot_of[owner[s]] = -1;
            owner[s] = -1;
        }
    }
    int take_slot(int d) {
        if (slot_of[d] >= 0) return slot_of[d];
        int s = -1;
        if (!free_slots.empty()) {
            s = free_slots.back();
            free_slots.pop_back();
        } else {
            for (int k = 0; k < nslots; k++)
                if (pins[k] == 0 && !pending[k] && (s < 0 || stamp[k] < stamp[s])) s = k;
            if (s < 0) return -1;
            evict(s);
        }
        owner[s] = d;
        slot_of[d] = s;
        return s;
    }
    int flush() {
        if (ops.empty()) return IQGPU_OK;
        const int rc = iqgpu_compute_partials(e, ops.data(), (int32_t)ops.size());
        nupdates += (int64_t)ops.size() * nptn;
        settled(rc);
        return rc;
    }
    void unpin(int ref) {
        if (ref >= 0 && pins[ref] > 0) pins[ref]--;
    }
    void settled(int rc) {  // the evaluation launch executed the pending records (or failed)
        ops.clear();
        op_edge.clear();
        std::fill(pending.begin(), pending.end(), 0);
        if (rc) std::fill(computed.begin(), computed.end(), 0);  // nothing of a failed launch is valid
    }

    // post-order list of stale partials (tree/phylotree.cpp:5918-6028); returns
    // the partial of node seen from dad (a slot, pinned for the caller, or a
    // tip). A node with more than two children becomes consecutive records
    // flagged IQGPU_OP_MORE (two children each, IQGPU_NO_CHILD closing an odd
    // count); children keep the neighbour order in the records.
    int traverse(int dad, int node) {
        if (leaf(node)) return -1 - node;
        const int d = dad * kMaxDeg + idx(dad, node);
        if (computed[d]) {
            const int s = slot_of[d];
            pins[s]++;
            stamp[s] = ++tick;
            return s;
        }
        int kid_q[kMaxDeg], order[kMaxDeg], refs[kMaxDeg];
        int k = 0;
        for (int q = 0; q < deg[node]; q++)
            if (nbr[node * kMaxDeg + q] != dad) kid_q[k++] = q;
        for (int i = 0; i < k; i++) order[i] = i;
        std::stable_sort(order, order + k, [&](int x, int y) {
            return leaves_behind(node, nbr[node * kMaxDeg + kid_q[x]]) > leaves_behind(node, nbr[node * kMaxDeg + kid_q[y]]);
        });
        for (int i = 0; i < k; i++) refs[order[i]] = traverse(node, nbr[node * kMaxDeg + kid_q[order[i]]]);
        if (walk_rc) return 0;
        int s = take_slot(d);
        if (s < 0) {
            if ((walk_rc = flush())) return 0;
            s = take_slot(d);
        }
        if (s < 0) {
            iqg::set_error("too few partial slots for this tree (every slot holds a partial still needed)");
            walk_rc = IQGPU_ERR_OOM;
            return 0;
        }
        for (int i = 0; i < k; i += 2) {
            iqgpu_op op;
            std::memset(&op, 0, sizeof(op));
            op.dad_slot = s;
            op.child[0] = refs[i];
            op.len[0] = len[edge[node * kMaxDeg + kid_q[i]]];
            op.child[1] = i + 1 < k ? refs[i + 1] : IQGPU_NO_CHILD;
            op.len[1] = i + 1 < k ? len[edge[node * kMaxDeg + kid_q[i + 1]]] : 0.0;
            op.flags = i + 2 < k ? IQGPU_OP_MORE : 0;
            ops.push_back(op);
            op_edge.push_back(edge[node * kMaxDeg + kid_q[i]]);
            op_edge.push_back(i + 1 < k ? edge[node * kMaxDeg + kid_q[i + 1]] : -1);
        }
        for (int i = 0; i < k; i++)
            if (refs[i] >= 0) {
                unpin(refs[i]);
                pending[refs[i]] = 1;
            }
        pending[s] = 1;
        stamp[s] = ++tick;
        computed[d] = 1;
        pins[s]++;
        return s;
    }
    // both partials of branch dad-node, pinned until the branch is evaluated
    int collect(int node, int dad, int *a, int *b) {
        walk_rc = IQGPU_OK;
        *a = traverse(dad, node); /* dad_branch: dad -> node */
        *b = traverse(node, dad); /* node_branch: node -> dad */
        return walk_rc;
    }
    int farthest_leaf(int node, int dad) {
        if (dad >= 0 && leaf(node)) { height[node] = 0; return node; }
        int res = -1;
        height[node] = 0;
        for (int q = 0; q < deg[node]; q++) {
            const int ch = nbr[node * kMaxDeg + q];
            if (ch == dad) continue;
            const int lf = farthest_leaf(ch, node);
            if (height[node] < height[ch] + 1) {
                height[node] = height[ch] + 1;
                res = lf;
            }
        }
        return res;
    }
    void clear_reverse(int node, int dad) {
        for (int q = 0; q < deg[node]; q++) {
            const int x = nbr[node * kMaxDeg + q];
            if (x == dad) continue;
            computed[x * kMaxDeg + idx(x, node)] = 0;  // stale; its slot is reused when it is recomputed
            clear_reverse(x, node);
        }
    }
    void preorder(int node, int dad, std::vector<int> &n1, std::vector<int> &n2) {
        if (dad >= 0) { n1.push_back(node); n2.push_back(dad); }
        int order[kMaxDeg], d = deg[node];
        for (int q = 0; q < d; q++) order[q] = nbr[node * kMaxDeg + q];
        for (int i = 0; i < d; i++)
            for (int k = i + 1; k < d; k++)
                if (height[order[i]] > height[order[k]]) std::swap(order[i], order[k]);
        for (int q = 0; q < d; q++)
            if (order[q] != dad) preorder(order[q], node, n1, n2);
    }
};

namespace {

int64_t nptn_of(const iqgpu_tree *t) { return t->nptn; }

// computeLikelihoodBranch(dad_branch = dad->node, dad)
int lnl_branch(iqgpu_tree *t, int node, int dad, double *lnl) {
    if (t->leaf(node)) std::swap(node, dad);
    int a, b;
    int rc = t->collect(node, dad, &a, &b);
    if (!rc) rc = iqgpu_compute_likelihood(t->e, t->ops.data(), (int32_t)t->ops.size(), a, b, t->blen(node, dad), lnl);
    t->nupdates += (int64_t)t->ops.size() * nptn_of(t);
    t->settled(rc);
    t->unpin(a);
    t->unpin(b);
    return rc;
}

// computeFuncDerv: f = -df, df = -ddf on the current branch
int func_derv(iqgpu_tree *t, double value, double *f, double *df) {
    const int n1 = t->cur1, n2 = t->cur2;
    t->blen(n1, n2) = value;
    int node = n2, dad = n1;
    if (t->leaf(node)) std::swap(node, dad);
    int a, b;
    int rc = t->collect(node, dad, &a, &b);
    double d1 = 0.0, d2 = 0.0;
    if (!rc)
        rc = iqgpu_likelihood_derv(t->e, t->ops.data(), (int32_t)t->ops.size(), a, b, value,
                                   t->theta_computed ? 1 : 0, &d1, &d2);
    t->nupdates += (int64_t)t->ops.size() * nptn_of(t);
    t->settled(rc);
    t->unpin(a);
    t->unpin(b);
    if (rc) return rc;
    t->theta_computed = true;
    *f = -d1;
    *df = -d2;
    return IQGPU_OK;
}

int from_buffer(iqgpu_tree *t, double *lnl) { return iqgpu_lnl_from_buffer(t->e, t->blen(t->cur1, t->cur2), lnl); }

// Optimization::minimizeNewton (utils/optimization.cpp:422-499)
int minimize_newton(iqgpu_tree *t, double x1, double xguess, double x2, double xacc, int max_nr_step, double *out) {
    double f, df, dx, temp, xh, xl, rts, rts_old;
    int rc;
    rts = xguess;
    if (rts < x1) rts = x1;
    if (rts > x2) rts = x2;
    if ((rc = func_derv(t, rts, &f, &df))) return rc;
    if (!std::isfinite(f) || !std::isfinite(df)) { iqg::set_error("Wrong computeFuncDerv"); return IQGPU_ERR_NEWTON; }
    if (df >= 0.0 && std::fabs(f) < xacc) { *out = rts; return IQGPU_OK; }
    if (f < 0.0) { xl = rts; xh = x2; } else { xh = rts; xl = x1; }
    dx = std::fabs(xh - xl);
    for (int j = 1; j <= max_nr_step; j++) {
        rts_old = rts;
        if ((df <= 0.0) || (((rts - xh) * df - f) * ((rts - xl) * df - f) >= 0.0)) {
            dx = 0.5 * (xh - xl);
            rts = xl + dx;
            if (xl == rts) { *out = rts; return IQGPU_OK; }
        } else {
            dx = f / df;
            temp = rts;
            rts -= dx;
            if (temp == rts) { *out = rts; return IQGPU_OK; }
        }
        if (std::fabs(dx) < xacc || (j == max_nr_step)) { *out = rts_old; return IQGPU_OK; }
        if ((rc = func_derv(t, rts, &f, &df))) return rc;
        if (!std::isfinite(f) || !std::isfinite(df)) { iqg::set_error("Wrong computeFuncDerv"); return IQGPU_ERR_NEWTON; }
        if (df > 0.0 && std::fabs(f) < xacc) { *out = rts; return IQGPU_OK; }
        if (f < 0.0) xl = rts;
        else if (f > 0.0) xh = rts;
    }
    iqg::set_error("Maximum number of iterations exceeded in minimizeNewton");
    return IQGPU_ERR_NEWTON;
}

// minimizeNewton as one device kernel (iqgpu_newton_branch): the same
// control flow, with one host wait per branch instead of one per step
int minimize_newton_device(iqgpu_tree *t, double x1, double xguess, double x2, double xacc, int max_nr_step,
                           double *out) {
    int node = t->cur2, dad = t->cur1;
    if (t->leaf(node)) std::swap(node, dad);
    int a, b;
    double last = xguess;
    int rc = t->collect(node, dad, &a, &b);
    if (!rc)
        rc = iqgpu_newton_branch(t->e, t->ops.data(), (int32_t)t->ops.size(), a, b, t->theta_computed ? 1 : 0, x1,
                                 xguess, x2, xacc, max_nr_step, out, nullptr, &last, nullptr);
    t->nupdates += (int64_t)t->ops.size() * nptn_of(t);
    t->settled(rc);
    t->unpin(a);
    t->unpin(b);
    if (rc) return rc;
    t->theta_computed = true;
    t->blen(t->cur1, t->cur2) = last;  // the branch holds the last evaluated length, as after computeFuncDerv
    return IQGPU_OK;
}

// One pass of optimizeAllBranches (tree/phylotree.cpp:2698-2774) on the
// device: the pass's op lists are built here first, as the branch-by-branch
// driver builds them when every branch's length changes (each branch then
// clears the partials behind it, tree/phylotree.cpp:2635-2640), and
// iqg::run_pass rebuilds, forms theta and solves branch after branch with the
// lengths kept on the device. Recomputing a partial whose branch kept its
// length gives the same values, so the pass matches the branch-by-branch
// driver's results. It stands when every solve returned an optimum below
// 0.95 max_bl; otherwise (the reference's lnL comparison at the bound, or an
// error) the lengths go back to the pass's start, every partial is marked
// stale and *done is false, for the branch-by-branch driver to take the pass.
// Served when every directed internal partial has its own slot (no eviction).
int device_pass(iqgpu_tree *t, const std::vector<int> &n1, const std::vector<int> &n2, int max_nr_step,
                bool *done) {
    *done = false;
    const std::vector<double> saved = t->len;
    std::vector<iqgpu_op> ops;
    std::vector<int32_t> edges, off{0}, ab, bedge;
    for (size_t j = 0; j < n1.size(); j++) {
        int node = n2[j], dad = n1[j];
        if (t->leaf(node)) std::swap(node, dad);
        int a, b;
        int rc = t->collect(node, dad, &a, &b);
        if (rc) {
            t->settled(rc);
            t->unpin(a);
            t->unpin(b);
            return rc;
        }
        ops.insert(ops.end(), t->ops.begin(), t->ops.end());
        edges.insert(edges.end(), t->op_edge.begin(), t->op_edge.end());
        off.push_back((int32_t)ops.size());
        t->nupdates += (int64_t)t->ops.size() * nptn_of(t);
        t->settled(IQGPU_OK);
        t->unpin(a);
        t->unpin(b);
        if (a < 0) std::swap(a, b);
        ab.push_back(a);
        ab.push_back(b);
        bedge.push_back(t->edge[n1[j] * kMaxDeg + t->idx(n1[j], n2[j])]);
        t->clear_reverse(n1[j], n2[j]);
        t->clear_reverse(n2[j], n1[j]);
    }
    std::vector<double> res(4 * n1.size());
    int rc = iqg::run_pass(t->e, ops.data(), edges.data(), off.data(), ab.data(), bedge.data(), (int)n1.size(),
                           t->len.data(), t->nedge, t->min_bl, t->max_bl, t->min_bl, max_nr_step, res.data());
    if (rc) {
        t->settled(rc);
        return rc;
    }
    bool ok = true;
    for (size_t j = 0; j < n1.size() && ok; j++) {
        ok = ((int)res[4 * j + 1] & 15) == 0 && !(res[4 * j] > t->max_bl * 0.95);
        t->len[bedge[j]] = res[4 * j];
    }
    if (!ok) {
        t->len = saved;
        std::fill(t->computed.begin(), t->computed.end(), 0);
        t->theta_computed = false;
        return IQGPU_OK;
    }
    t->cur1 = n1.back();
    t->cur2 = n2.back();
    t->theta_computed = true;
    *done = true;
    return IQGPU_OK;
}

// every directed partial of an internal node has a slot of its own
bool slots_for_all(const iqgpu_tree *t) {
    long long need = 0;
    for (int u = t->ntaxa; u < t->nnode; u++) need += t->deg[u];
    return need <= t->nslots;
}

}  // namespace

extern "C" {

int iqgpu_tree_create_n(iqgpu_engine *e, int32_t nedge, const int32_t *edges, const double *lengths,
                        iqgpu_tree **out) {
    if (!e || !edges || !lengths || !out) { iqg::set_error("null argument"); return IQGPU_ERR_ARG; }
    *out = nullptr;
    iqgpu_config cfgv;
    int rc0 = iqgpu_get_config(e, &cfgv);
    if (rc0) return rc0;
    const iqgpu_config *cfg = &cfgv;
    if (nedge < cfg->ntaxa || nedge > 2 * cfg->ntaxa - 3) {
        iqg::set_error("an unrooted tree on ntaxa leaves has between ntaxa and 2*ntaxa-3 edges");
        return IQGPU_ERR_ARG;
    }
    iqgpu_tree *t = new iqgpu_tree();
    t->e = e;
    t->nptn = cfg->nptn;
    t->ntaxa = cfg->ntaxa;
    t->nedge = nedge;
    t->nnode = nedge + 1;  // a tree
    t->deg.assign(t->nnode, 0);
    t->nbr.assign((size_t)t->nnode * kMaxDeg, -1);
    t->edge.assign((size_t)t->nnode * kMaxDeg, -1);
    t->slot_of.assign((size_t)t->nnode * kMaxDeg, -1);
    t->leaves.assign((size_t)t->nnode * kMaxDeg, 0);
    t->computed.assign((size_t)t->nnode * kMaxDeg, 0);
    t->height.assign(t->nnode, 0);
    t->len.assign(lengths, lengths + t->nedge);
    for (int k = 0; k < t->nedge; k++) {
        const int u = edges[2 * k], v = edges[2 * k + 1];
        if (u < 0 || v < 0 || u >= t->nnode || v >= t->nnode || u == v || t->deg[u] >= kMaxDeg ||
            t->deg[v] >= kMaxDeg || !(lengths[k] >= 0.0)) {
            delete t;
            iqg::set_error("edge list is not an unrooted tree on nedge+1 nodes (node degree <= 32)");
            return IQGPU_ERR_ARG;
        }
        t->nbr[u * kMaxDeg + t->deg[u]] = v;
        t->edge[u * kMaxDeg + t->deg[u]++] = k;
        t->nbr[v * kMaxDeg + t->deg[v]] = u;
        t->edge[v * kMaxDeg + t->deg[v]++] = k;
    }
    for (int u = 0; u < t->nnode; u++) {
        if ((t->leaf(u) && t->deg[u] != 1) || (!t->leaf(u) && t->deg[u] < 3)) {
            delete t;
            iqg::set_error("leaves need degree 1 and internal nodes degree 3 or more");
            return IQGPU_ERR_ARG;
        }
    }
    int ns = 0;  // directed internal partials
    for (int u = 0; u < t->nnode; u++)
        for (int j = 0; j < t->deg[u]; j++)
            if (!t->leaf(t->nbr[u * kMaxDeg + j])) ns++;
    // fewer slots than partials: recycling; it needs the partials pinned along
    // one root path (larger subtrees first: about log2(ntaxa)) plus the branch
    int lg = 1;
    while ((1 << lg) < t->ntaxa) lg++;
    const int min_slots = std::min(ns, 2 * lg + 4);
    if (cfg->nslots < min_slots || cfg->max_ops < 2 * t->ntaxa) {
        delete t;
        iqg::set_error("engine needs nslots >= " + std::to_string(min_slots) + " (" + std::to_string(ns) +
                       " for every directed internal partial at once) and max_ops >= 2*ntaxa");
        return IQGPU_ERR_ARG;
    }
    t->nslots = std::min(cfg->nslots, ns);
    t->owner.assign(t->nslots, -1);
    t->stamp.assign(t->nslots, 0);
    t->pins.assign(t->nslots, 0);
    t->pending.assign(t->nslots, 0);
    for (int k = t->nslots - 1; k >= 0; k--) t->free_slots.push_back(k);
    *out = t;
    return IQGPU_OK;
}

int iqgpu_tree_create(iqgpu_engine *e, const int32_t *edges, const double *lengths, iqgpu_tree **out) {
    iqgpu_config cfg;
    int rc = e ? iqgpu_get_config(e, &cfg) : IQGPU_ERR_ARG;
    if (rc) {
        if (!e) iqg::set_error("null argument");
        return rc;
    }
    return iqgpu_tree_create_n(e, 2 * cfg.ntaxa - 3, edges, lengths, out);
}

int iqgpu_tree_destroy(iqgpu_tree *t) {
    delete t;
    return IQGPU_OK;
}

int iqgpu_tree_compute_likelihood(iqgpu_tree *t, double *lnl, double *pattern_lh) {
    if (!t || !lnl) { iqg::set_error("null argument"); return IQGPU_ERR_ARG; }
    if (t->cur1 < 0) {
        const int lf = t->farthest_leaf(0, -1);  // root is taxon 0, a leaf
        t->cur1 = lf;
        t->cur2 = t->nbr[lf * kMaxDeg];
    }
    int rc = lnl_branch(t, t->cur2, t->cur1, lnl);
    if (rc) return rc;
    if (pattern_lh) rc = iqgpu_get_pattern_lh(t->e, pattern_lh);
    return rc;
}

int iqgpu_tree_optimize_one_branch(iqgpu_tree *t, int32_t node1, int32_t node2, int32_t max_nr_step) {
    if (!t || node1 < 0 || node2 < 0 || node1 >= t->nnode || node2 >= t->nnode || t->idx(node1, node2) < 0) {
        iqg::set_error("not a branch");
        return IQGPU_ERR_ARG;
    }
    t->cur1 = node1;
    t->cur2 = node2;
    const double current_len = t->blen(node1, node2);
    t->theta_computed = false;
    double optx = current_len;
    int rc = t->device_newton && iqg::newton_on_device(t->e)
                 ? minimize_newton_device(t, t->min_bl, current_len, t->max_bl, t->min_bl, max_nr_step, &optx)
                 : minimize_newton(t, t->min_bl, current_len, t->max_bl, t->min_bl, max_nr_step, &optx);
    if (rc) return rc;
    if (optx > t->max_bl * 0.95) {
        // at the length of the last derivative evaluation, as the reference
        // (current_it->length, tree/phylotree.cpp:2619-2621)
        double opt_lh, orig_lh;
        if ((rc = from_buffer(t, &opt_lh))) return rc;
        t->blen(node1, node2) = current_len;
        if ((rc = from_buffer(t, &orig_lh))) return rc;
        if (orig_lh > opt_lh) optx = current_len;
    }
    t->blen(node1, node2) = optx;
    if (current_len != optx) {
        t->clear_reverse(node1, node2);
        t->clear_reverse(node2, node1);
    }
    return IQGPU_OK;
}

int iqgpu_tree_optimize_all_branches(iqgpu_tree *t, int32_t iterations, double tolerance, int32_t max_nr_step,
                                     double *lnl) {
    if (!t || !lnl) { iqg::set_error("null argument"); return IQGPU_ERR_ARG; }
    std::vector<int> n1, n2;
    const int farleaf = t->farthest_leaf(0, -1);
    t->farthest_leaf(farleaf, -1);
    t->preorder(farleaf, -1, n1, n2);
    double tree_lh;
    int rc = lnl_branch(t, n2[0], n1[0], &tree_lh);
    if (rc) return rc;
    std::vector<double> saved;
    const bool on_device = t->device_newton == 1 && iqg::pass_served(t->e) && slots_for_all(t) && !n1.empty();
    for (int it = 0; it < iterations; it++) {
        saved = t->len;
        bool done = false;
        if (on_device && (rc = device_pass(t, n1, n2, max_nr_step, &done))) return rc;
        for (size_t j = 0; j < n1.size() && !done; j++)
            if ((rc = iqgpu_tree_optimize_one_branch(t, n1[j], n2[j], max_nr_step))) return rc;
        double new_lh;
        if ((rc = from_buffer(t, &new_lh))) return rc;
        if (new_lh < tree_lh - tolerance * 0.1) {
            // log-likelihood decreased: restore and stop
            t->len = saved;
            std::fill(t->computed.begin(), t->computed.end(), 0);
            return iqgpu_tree_compute_likelihood(t, lnl, nullptr);
        }
        if (tree_lh <= new_lh && new_lh <= tree_lh + tolerance) {
            *lnl = new_lh;
            return IQGPU_OK;
        }
        tree_lh = new_lh;
    }
    *lnl = tree_lh;
    return IQGPU_OK;
}

int iqgpu_tree_get_lengths(iqgpu_tree *t, double *lengths) {
    if (!t || !lengths) { iqg::set_error("null argument"); return IQGPU_ERR_ARG; }
    std::memcpy(lengths, t->len.data(), sizeof(double) * t->nedge);
    return IQGPU_OK;
}

int iqgpu_tree_set_lengths(iqgpu_tree *t, const double *lengths) {
    if (!t || !lengths) { iqg::set_error("null argument"); return IQGPU_ERR_ARG; }
    for (int k = 0; k < t->nedge; k++)
        if (!(lengths[k] >= 0.0)) { iqg::set_error("negative branch length"); return IQGPU_ERR_ARG; }
    t->len.assign(lengths, lengths + t->nedge);
    std::fill(t->computed.begin(), t->computed.end(), 0);  // clearAllPartialLH
    t->theta_computed = false;
    return IQGPU_OK;
}

int iqgpu_tree_set_bounds(iqgpu_tree *t, double min_bl, double max_bl) {
    if (!t || !(min_bl > 0.0) || !(max_bl > min_bl)) { iqg::set_error("bad bounds"); return IQGPU_ERR_ARG; }
    t->min_bl = min_bl;
    t->max_bl = max_bl;
    return IQGPU_OK;
}

int iqgpu_tree_set_device_newton(iqgpu_tree *t, int32_t on) {
    if (!t) { iqg::set_error("null argument"); return IQGPU_ERR_ARG; }
    t->device_newton = on < 0 || on > 2 ? 1 : on;
    return IQGPU_OK;
}

int iqgpu_tree_num_updates(iqgpu_tree *t, int64_t *updates) {
    if (!t || !updates) { iqg::set_error("null argument"); return IQGPU_ERR_ARG; }
    *updates = t->nupdates;
    return IQGPU_OK;
}

}  // extern "C"
