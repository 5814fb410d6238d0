/*
 * Reference oracle: IQ-TREE 2's own likelihood kernels, compiled from the
 * reference checkout's tree/phylokernelnew.h (read in place, never copied
 * into this repository) against the stand-in environment of refenv.h, behind
 * a small C API for the tests.
 *
 * Test infrastructure only. The tests use it to pin oracle/phylo_oracle.c (the
 * C restatement that the GPU parity tests check against) to the reference's
 * compiled kernels, and tests/golden/make_refgolden.py to write golden vectors
 * from it. Nothing on the product path links it.
 *
 * Kernels instantiated (tree/phylotreesse.cpp:91-199, tree/phylokernelfma.cpp,
 * tree/phylokernelsse.cpp choose among the same templates):
 *   kind 0: the one-lane generic kernels (Vec1d), the path the reference
 *           installs when built without SIMD (tree/phylotreesse.cpp:186-191);
 *   kind 1: the SIMD kernels the reference installs on this host: Vec4d with
 *           FMA (setLikelihoodKernelFMA) where AVX2+FMA are compiled in, else
 *           Vec2d (setLikelihoodKernelSSE, also the Arm NEON build through
 *           sse2neon); fixed-state templates for 4 and 20 states, the generic
 *           ones otherwise.
 *
 * What this file restates rather than compiles (host code of
 * tree/phylotree.cpp, which cannot be linked without the rest of IQ-TREE):
 * the subtree walk that fills traversal_info (computeTraversalInfo(
 * PhyloNeighbor*, PhyloNode*, double*&), tree/phylotree.cpp:5918-6028, with
 * one partial slot per directed internal branch as in LM_PER_NODE) and the
 * buffer size of getBufferPartialLhSize (tree/phylotree.cpp:864-891).
 */
#include "refenv.h"

#include "tree/phylokernelnew.h"
#define KERNEL_FIX_STATES
#include "tree/phylokernelnew.h"

#include <algorithm>
#include <map>
#include <memory>

VerboseMode verbose_mode = VB_MIN;

Params &Params::getInstance() {
    static Params p;
    return p;
}

struct iqref_failure : std::runtime_error {
    using std::runtime_error::runtime_error;
};

void iqref_fail(const char *what, const char *file, int line) {
    char buf[512];
    snprintf(buf, sizeof buf, "%s (%s:%d)", what, file, line);
    throw iqref_failure(buf);
}

#if INSTRSET >= 8 && defined(__FMA__)
typedef Vec4d SimdVec;
static const bool kSimdFMA = true;
#else
typedef Vec2d SimdVec;
static const bool kSimdFMA = false;
#endif

/* ------------------------------------------------------------------------ */

size_t PhyloTree::getBufferPartialLhSize() {
    const size_t V = 8;
    size_t nstates = aln->num_states;
    size_t ncat_mix = site_rate->getNRate() * (model_factory->fused_mix_rate ? 1 : model->getNMixtures());
    size_t block = nstates * ncat_mix;
    size_t size = 0;
    /* echildren and leaf tables of every traversal entry */
    size += get_safe_upper_limit(block * nstates * 2) * aln->getNSeq();
    size += get_safe_upper_limit(block * (aln->STATE_UNKNOWN + 1)) * aln->getNSeq();
    /* per-branch scratch the kernels carve from the front and the back */
    size += get_safe_upper_limit(block * (aln->STATE_UNKNOWN + 1));
    size += (block * 2 + nstates) * V * num_packets;
    size += get_safe_upper_limit(block) * (aln->STATE_UNKNOWN + 1) * 2;
    size += block * 2 * V * num_packets;
    size += get_safe_upper_limit(3 * block * nstates);
    return size;
}

bool PhyloTree::computeTraversalInfo(PhyloNeighbor *dad_branch, PhyloNode *dad, double *&buffer) {
    PhyloNode *node = (PhyloNode *)dad_branch->node;
    if ((dad_branch->partial_lh_computed & 1) || node->isLeaf()) return false;
    /* children first, larger subtrees first */
    vector<pair<int, PhyloNeighbor *>> kids;
    size_t num_leaves = 0;
    FOR_NEIGHBOR_IT(node, dad, it) {
        PhyloNeighbor *nei = (PhyloNeighbor *)*it;
        kids.push_back({nei->node->computeSize(node), nei});
        if (nei->node->isLeaf()) num_leaves++;
    }
    std::stable_sort(kids.begin(), kids.end(), [](auto &a, auto &b) { return a.first > b.first; });
    for (auto &k : kids) computeTraversalInfo(k.second, node, buffer);
    dad_branch->partial_lh_computed |= 1;

    TraversalInfo info(dad_branch, dad);
    size_t nstates = aln->num_states;
    size_t block = nstates * (model_factory->fused_mix_rate ? site_rate->getNRate()
                                                            : site_rate->getNRate() * model->getNMixtures());
    info.echildren = buffer;
    buffer += get_safe_upper_limit(block * nstates * (node->degree() - 1));
    if (num_leaves) {
        info.partial_lh_leaves = buffer;
        buffer += get_safe_upper_limit((aln->STATE_UNKNOWN + 1) * block * num_leaves);
    }
    traversal_info.push_back(info);
    return false;
}

/* ------------------------------------------------------------------------ */

namespace {

typedef void (PhyloTree::*PartialFn)(TraversalInfo &, size_t, size_t, int);
typedef double (PhyloTree::*BranchFn)(PhyloNeighbor *, PhyloNode *, bool);
typedef void (PhyloTree::*DervFn)(PhyloNeighbor *, PhyloNode *, double *, double *);
typedef double (PhyloTree::*FromBufferFn)();
typedef void (PhyloTree::*TraverseFn)(PhyloNode *, PhyloNode *, bool);

struct Kernels {
    PartialFn partial;
    BranchFn branch;
    DervFn derv;
    FromBufferFn from_buffer;
    TraverseFn traverse;
    int vsize;
};

template <class VC, bool SAFE, bool FMA> Kernels generic_kernels() {
    return {&PhyloTree::computePartialLikelihoodGenericSIMD<VC, SAFE, FMA>,
            &PhyloTree::computeLikelihoodBranchGenericSIMD<VC, SAFE, FMA>,
            &PhyloTree::computeLikelihoodDervGenericSIMD<VC, SAFE, FMA>,
            &PhyloTree::computeLikelihoodFromBufferGenericSIMD<VC, FMA>,
            &PhyloTree::computeTraversalInfo<VC>,
            VC::size()};
}

template <class VC, bool SAFE, int N, bool FMA> Kernels fixed_kernels() {
    return {&PhyloTree::computePartialLikelihoodSIMD<VC, SAFE, N, FMA>,
            &PhyloTree::computeLikelihoodBranchSIMD<VC, SAFE, N, FMA>,
            &PhyloTree::computeLikelihoodDervSIMD<VC, SAFE, N, FMA>,
            &PhyloTree::computeLikelihoodFromBufferSIMD<VC, N, FMA>,
            &PhyloTree::computeTraversalInfo<VC, N>,
            VC::size()};
}

Kernels pick_kernels(int kind, bool safe, int nstates) {
    if (kind == 0) return safe ? generic_kernels<Vec1d, true, false>() : generic_kernels<Vec1d, false, false>();
    if (nstates == 4)
        return safe ? fixed_kernels<SimdVec, true, 4, kSimdFMA>() : fixed_kernels<SimdVec, false, 4, kSimdFMA>();
    if (nstates == 20)
        return safe ? fixed_kernels<SimdVec, true, 20, kSimdFMA>() : fixed_kernels<SimdVec, false, 20, kSimdFMA>();
    return safe ? generic_kernels<SimdVec, true, kSimdFMA>() : generic_kernels<SimdVec, false, kSimdFMA>();
}

template <class T> struct Aligned {
    T *p = nullptr;
    size_t n = 0;
    // zeroed unless `lazy` (partials and scale counts: written before they are
    // read, so pages of slots a traversal never touches are never committed)
    void alloc(size_t count, bool lazy = false) {
        release();
        n = count;
        p = aligned_alloc<T>(count ? count : 1);
        if (!lazy) memset(p, 0, sizeof(T) * (count ? count : 1));
    }
    void release() {
        if (p) free(p);
        p = nullptr;
    }
    ~Aligned() { release(); }
};

}  // namespace

struct iqref {
    PhyloTree tree;
    Alignment aln;
    ModelSubst model;
    RateHeterogeneity rates;
    ModelFactory factory;
    Params params;
    Kernels k;
    int ntaxa, nptn, nptn_pad, nstates, ncat, safe, kind;
    Aligned<double> eval, evec, inv_evec, tip_lh, freq, invar, buffer, theta, scale_all, pattern_lh, pattern_lh_cat;
    vector<vector<UBYTE>> tip_rows;
    vector<std::unique_ptr<PhyloNode>> nodes;
    vector<std::unique_ptr<PhyloNeighbor>> neis;
    vector<Aligned<double>> partials;
    vector<Aligned<UBYTE>> scales;
    vector<pair<PhyloNeighbor *, PhyloNeighbor *>> edge_nei; /* per edge: a->b side, b->a side */
    std::string err;
};

static thread_local std::string g_err;

#define IQREF_TRY(...)                        \
    try {                                      \
        __VA_ARGS__;                           \
        return 0;                              \
    } catch (const std::exception &ex) {       \
        g_err = ex.what();                     \
        return 1;                              \
    }

extern "C" {

const char *iqref_last_error(void) { return g_err.c_str(); }

/* Which SIMD kernel kind 1 is on this build: vector width and FMA. */
int iqref_simd_info(int *vsize, int *fma) {
    *vsize = SimdVec::size();
    *fma = kSimdFMA ? 1 : 0;
    return 0;
}

int iqref_create(int ntaxa, int nptn, int nstates, int ncat, int state_unknown, int safe, int kind, int nthreads,
                 iqref **out) {
    IQREF_TRY({
        if (ntaxa < 3 || nptn < 1 || nstates < 2 || ncat < 1 || (kind != 0 && kind != 1))
            iqref_fail("bad arguments", __FILE__, __LINE__);
        iqref *r = new iqref();
        r->ntaxa = ntaxa;
        r->nptn = nptn;
        r->nstates = nstates;
        r->ncat = ncat;
        r->safe = safe;
        r->kind = kind;
        r->k = pick_kernels(kind, safe != 0, nstates);
        r->nptn_pad = roundUpToMultiple(nptn, r->k.vsize);
        r->aln.num_states = nstates;
        r->aln.STATE_UNKNOWN = state_unknown;
        r->aln.nseq = ntaxa;
        r->aln.resize(nptn);
        r->model.num_states = nstates;
        r->rates.rate.assign(ncat, 1.0);
        r->rates.prop.assign(ncat, 1.0 / ncat);
        r->params.num_threads = nthreads < 1 ? 1 : nthreads;
        Params::getInstance().num_threads = r->params.num_threads;
        PhyloTree &t = r->tree;
        t.aln = &r->aln;
        t.model = &r->model;
        t.site_rate = &r->rates;
        t.model_factory = &r->factory;
        t.params = &r->params;
        t.num_threads = r->params.num_threads;
        t.num_packets = t.num_threads == 1 ? 1 : t.num_threads * 2;
        t.computePartialLikelihoodPointer = r->k.partial;
        size_t block = (size_t)nstates * ncat;
        r->eval.alloc(get_safe_upper_limit(nstates));
        r->evec.alloc(get_safe_upper_limit((size_t)nstates * nstates));
        r->inv_evec.alloc(get_safe_upper_limit((size_t)nstates * nstates));
        r->tip_lh.alloc(get_safe_upper_limit((size_t)(state_unknown + 1) * nstates));
        r->freq.alloc(get_safe_upper_limit(r->nptn_pad));
        r->invar.alloc(get_safe_upper_limit(r->nptn_pad));
        r->theta.alloc((size_t)r->nptn_pad * block);
        r->scale_all.alloc(get_safe_upper_limit(r->nptn_pad));
        r->pattern_lh.alloc(get_safe_upper_limit(r->nptn_pad));
        r->pattern_lh_cat.alloc((size_t)r->nptn_pad * ncat);
        r->model.eval = r->eval.p;
        r->model.evec = r->evec.p;
        r->model.inv_evec = r->inv_evec.p;
        t.tip_partial_lh = r->tip_lh.p;
        t.ptn_freq = r->freq.p;
        t.ptn_invar = r->invar.p;
        t.theta_all = r->theta.p;
        t.buffer_scale_all = r->scale_all.p;
        t._pattern_lh = r->pattern_lh.p;
        t._pattern_lh_cat = r->pattern_lh_cat.p;
        r->buffer.alloc(t.getBufferPartialLhSize());
        t.buffer_partial_lh = r->buffer.p;
        r->tip_rows.assign(ntaxa, vector<UBYTE>(r->nptn_pad, (UBYTE)state_unknown));
        for (int i = 0; i < ntaxa; i++) t.tip_state_rows.push_back(r->tip_rows[i].data());
        *out = r;
    })
}

int iqref_destroy(iqref *r) {
    delete r;
    return 0;
}

/* eval[n], evec[n*n], inv_evec[n*n] row-major; rates, props [ncat]. */
int iqref_set_model(iqref *r, const double *eval, const double *evec, const double *inv_evec, const double *rates,
                    const double *props) {
    IQREF_TRY({
        size_t n = r->nstates;
        memcpy(r->eval.p, eval, sizeof(double) * n);
        memcpy(r->evec.p, evec, sizeof(double) * n * n);
        memcpy(r->inv_evec.p, inv_evec, sizeof(double) * n * n);
        r->rates.rate.assign(rates, rates + r->ncat);
        r->rates.prop.assign(props, props + r->ncat);
        r->tree.theta_computed = false;
    })
}

/* Eigen-space tip vectors [(state_unknown+1) x n] (tip_partial_lh). */
int iqref_set_tip_lh(iqref *r, const double *tip_lh) {
    IQREF_TRY(memcpy(r->tip_lh.p, tip_lh, sizeof(double) * (r->aln.STATE_UNKNOWN + 1) * r->nstates))
}

int iqref_set_patterns(iqref *r, const double *freq, const double *invar, int nsite) {
    IQREF_TRY({
        for (int p = 0; p < r->nptn; p++) {
            r->freq.p[p] = freq[p];
            r->invar.p[p] = invar ? invar[p] : 0.0;
        }
        r->aln.nsite = nsite;
    })
}

/* Tip states, ntaxa x nptn bytes. */
int iqref_set_tips(iqref *r, const uint8_t *states) {
    IQREF_TRY({
        for (int i = 0; i < r->ntaxa; i++) memcpy(r->tip_rows[i].data(), states + (size_t)i * r->nptn, r->nptn);
    })
}

/* Unrooted tree: edges[2k], edges[2k+1] join nodes (leaves 0..ntaxa-1, any
 * internal ids above), a node's neighbour order is edge order. Every directed
 * internal branch gets its own partial and scale buffer. */
int iqref_set_tree(iqref *r, int nedges, const int *edges, const double *lengths) {
    IQREF_TRY({
        int nnodes = 0;
        for (int e = 0; e < 2 * nedges; e++) nnodes = std::max(nnodes, edges[e] + 1);
        r->nodes.clear();
        r->neis.clear();
        r->partials.clear();
        r->scales.clear();
        r->edge_nei.clear();
        for (int i = 0; i < nnodes; i++) {
            r->nodes.emplace_back(new PhyloNode());
            r->nodes.back()->id = i;
        }
        size_t block = (size_t)r->nstates * r->ncat;
        size_t scale_n = r->safe ? (size_t)r->nptn_pad * r->ncat : (size_t)r->nptn_pad;
        size_t ninternal_dir = 0;
        for (int e = 0; e < nedges; e++) {
            int a = edges[2 * e], b = edges[2 * e + 1];
            PhyloNeighbor *ab = new PhyloNeighbor(), *ba = new PhyloNeighbor();
            ab->node = r->nodes[b].get(); /* a's neighbour pointing to b: partial of b's side */
            ba->node = r->nodes[a].get();
            ab->length = ba->length = lengths[e];
            ab->id = ba->id = e;
            r->nodes[a]->neighbors.push_back(ab);
            r->nodes[b]->neighbors.push_back(ba);
            r->neis.emplace_back(ab);
            r->neis.emplace_back(ba);
            r->edge_nei.push_back({ab, ba});
        }
        for (auto &nei : r->neis) {
            if (nei->node->isLeaf()) continue;
            ninternal_dir++;
        }
        r->partials.resize(ninternal_dir);
        r->scales.resize(ninternal_dir);
        size_t k = 0;
        for (auto &nei : r->neis) {
            if (nei->node->isLeaf()) continue;
            r->partials[k].alloc((size_t)r->nptn_pad * block, true);
            r->scales[k].alloc(scale_n, true);
            nei->partial_lh = r->partials[k].p;
            nei->scale_num = r->scales[k].p;
            k++;
        }
        r->tree.central_partial_lh = r->partials.empty() ? nullptr : r->partials[0].p;
        r->tree.root = r->nodes[0].get();
        r->tree.theta_computed = false;
    })
}

static void clear_all(iqref *r) {
    for (auto &nei : r->neis) nei->partial_lh_computed = 0;
    r->tree.theta_computed = false;
}

/* New length of edge e; every partial is recomputed at the next call. */
int iqref_set_length(iqref *r, int e, double len) {
    IQREF_TRY({
        r->edge_nei.at(e).first->length = len;
        r->edge_nei.at(e).second->length = len;
        clear_all(r);
    })
}

static PhyloNeighbor *directed(iqref *r, int node, int dad) {
    PhyloNode *nd = r->nodes.at(node).get(), *dd = r->nodes.at(dad).get();
    PhyloNeighbor *db = (PhyloNeighbor *)dd->findNeighbor(nd);
    if (!db) iqref_fail("not a branch", __FILE__, __LINE__);
    return db;
}

/* computeLikelihoodBranch(dad_branch = dad's neighbour `node`, dad): lnL and,
 * if pattern_lh is not NULL, the pattern lnL (_pattern_lh, nptn doubles). */
int iqref_branch_lnl(iqref *r, int node, int dad, double *lnl, double *pattern_lh) {
    IQREF_TRY({
        clear_all(r);
        PhyloNeighbor *db = directed(r, node, dad);
        *lnl = (r->tree.*(r->k.branch))(db, r->nodes[dad].get(), true);
        if (pattern_lh) memcpy(pattern_lh, r->pattern_lh.p, sizeof(double) * r->nptn);
    })
}

/* computeLikelihoodDerv(current_it = node1's neighbour node2, node1) at the
 * branch's current length, theta rebuilt: the kernel's df and ddf. */
int iqref_derv(iqref *r, int node1, int node2, double *df, double *ddf) {
    IQREF_TRY({
        clear_all(r);
        PhyloNeighbor *db = directed(r, node2, node1);
        r->tree.current_it = db;
        r->tree.current_it_back = (PhyloNeighbor *)r->nodes[node2]->findNeighbor(r->nodes[node1].get());
        (r->tree.*(r->k.derv))(db, r->nodes[node1].get(), df, ddf);
    })
}

/* computeLikelihoodFromBuffer after iqref_derv, with the current branch at
 * length len (theta is kept). */
int iqref_from_buffer(iqref *r, double len, double *lnl) {
    IQREF_TRY({
        if (!r->tree.theta_computed || !r->tree.current_it)
            iqref_fail("no theta buffer: call iqref_derv first", __FILE__, __LINE__);
        r->tree.current_it->length = len;
        r->tree.current_it_back->length = len;
        *lnl = (r->tree.*(r->k.from_buffer))();
    })
}

/* The partial of node `node` seen from neighbour `dad` (the directed branch
 * dad->node), de-interleaved to partial[ptn*B + c*n + x], and its scale counts
 * (NORM: nptn bytes; SAFE: nptn*ncat, pattern-major). Computes it first. */
int iqref_get_partial(iqref *r, int node, int dad, double *partial, uint8_t *scale) {
    IQREF_TRY({
        PhyloNode *nd = r->nodes.at(node).get(), *dd = r->nodes.at(dad).get();
        PhyloNeighbor *db = (PhyloNeighbor *)dd->findNeighbor(nd);
        if (!db || nd->isLeaf()) iqref_fail("not an internal directed branch", __FILE__, __LINE__);
        clear_all(r);
        PhyloTree &t = r->tree;
        /* the reference's two-sided traversal of branch dad-node (both partials) */
        (t.*(r->k.traverse))(nd, dd, true);
        size_t V = r->k.vsize;
        size_t n = r->nstates, B = n * r->ncat;
        if (partial) {
            for (int p = 0; p < r->nptn; p++)
                for (size_t j = 0; j < B; j++)
                    partial[(size_t)p * B + j] = db->partial_lh[(p / V) * B * V + j * V + p % V];
        }
        if (scale) {
            size_t per = r->safe ? r->ncat : 1;
            memcpy(scale, db->scale_num, (size_t)r->nptn * per);
        }
    })
}

}  /* extern "C" */
