/*
 * Stand-in environment for compiling IQ-TREE 2's own likelihood kernel
 * templates (tree/phylokernelnew.h) outside the IQ-TREE build.
 *
 * Test infrastructure only: this header and refkernels.cpp are compiled,
 * together with the reference's tree/phylokernelnew.h and vectorclass/
 * headers read where they lie in a reference checkout, into the reference
 * oracle library (oracle/_ref/). Nothing on the product path links it.
 *
 * tree/phylokernelnew.h defines member templates of PhyloTree and reads the
 * tree, alignment, model and rate objects through a small set of members. The
 * classes below provide exactly those members, with the names and meanings
 * the kernels expect (tree/phylotree.h, tree/node.h, tree/phylonode.h,
 * alignment/alignment.h, model/modelsubst.h, model/rateheterogeneity.h,
 * model/modelfactory.h, utils/tools.h), and nothing of IQ-TREE's own
 * implementation of them. The include guards of the real headers are
 * defined first, so the kernel header's `#include "phylotree.h"` is empty
 * and the kernels compile against these stand-ins.
 */
#ifndef IQREF_ENV_H
#define IQREF_ENV_H

#define PHYLOTREE_H 1

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

using namespace std; /* before vectorf64.h: its scalar max/min resolve to std's */

#include "vectorclass/vectorclass.h"
#include "vectorclass/vectormath_exp.h"
#include "vectorclass/vectorf64.h"

typedef unsigned char UBYTE;
typedef unsigned int UINT;
typedef vector<int> IntVector;

/* ---- constants the kernels test against (tree/phylotree.h:60-80) -------- */
#define SAFE_LH true
#define NORM_LH false
#define SCALING_THRESHOLD_EXP 256
#define SCALING_THRESHOLD 8.636168555094444625386e-78 /* 2^-256 */
#define LOG_SCALING_THRESHOLD -177.4456782233459932741 /* log(2^-256) */

/* ---- utils/tools.h pieces ----------------------------------------------- */
enum VerboseMode { VB_QUIET, VB_MIN, VB_MED, VB_MAX, VB_DEBUG };
extern VerboseMode verbose_mode;
enum LhMemSave { LM_PER_NODE, LM_MEM_SAVE };
enum ASCType { ASC_NONE, ASC_VARIANT, ASC_VARIANT_MISSING, ASC_INFORMATIVE, ASC_INFORMATIVE_MISSING };
const int WT_TAXON_ID = 4, WT_BR_LEN = 8, WT_NEWLINE = 256; /* tree-printing flags (diagnostics only) */
enum RootDirection { UNDEFINED_DIRECTION, TOWARD_ROOT, AWAYFROM_ROOT };

[[noreturn]] void iqref_fail(const char *what, const char *file, int line);
#define ASSERT(e) ((e) ? (void)0 : iqref_fail(#e, __FILE__, __LINE__))
inline void outError(const string &msg) { iqref_fail(msg.c_str(), __FILE__, __LINE__); }
inline void outError(const char *a, const string &b) { outError(string(a) + b); }
inline void outWarning(const string &msg) { cerr << "WARNING: " << msg << endl; }

struct Params {
    double robust_phy_keep = 1.0;
    bool robust_median = false;
    LhMemSave lh_mem_save = LM_PER_NODE;
    bool buffer_mem_save = false;
    int num_threads = 1;
    static Params &getInstance();
};

template <class C, class G> C roundUpToMultiple(C count, G grain) { return ((count + grain - 1) / grain) * grain; }
/* rounded up to a multiple of 8 doubles, as the kernels' buffer carve-up expects */
inline size_t get_safe_upper_limit(size_t cur_limit) { return ((cur_limit + 7) / 8) * 8; }

template <class T> inline T *aligned_alloc(size_t size) {
    void *mem = nullptr;
    if (posix_memalign(&mem, 64, (size ? size : 1) * sizeof(T)) != 0 || !mem) iqref_fail("out of memory", __FILE__, __LINE__);
    return (T *)mem;
}
template <class T> void aligned_free(T *&mem) {
    if (mem) free(mem);
    mem = nullptr;
}

/* ---- tree nodes (tree/node.h, tree/phylonode.h) -------------------------- */
class Node;
class Neighbor {
public:
    Node *node = nullptr;
    double length = 0.0;
    int id = -1;
    virtual ~Neighbor() {}
    double getLength(int) { return length; }
};
typedef vector<Neighbor *> NeighborVec;

class Node {
public:
    int id = -1;
    string name;
    NeighborVec neighbors;
    virtual ~Node() {}
    bool isLeaf() { return neighbors.size() <= 1; }
    int degree() { return (int)neighbors.size(); }
    Neighbor *findNeighbor(Node *n) {
        for (Neighbor *nei : neighbors)
            if (nei->node == n) return nei;
        return nullptr;
    }
    int computeSize(Node *dad) {
        int s = isLeaf() ? 1 : 0;
        for (Neighbor *nei : neighbors)
            if (nei->node != dad) s += nei->node->computeSize(this);
        return s;
    }
};

#define FOR_NEIGHBOR_IT(mynode, mydad, it) \
    for (NeighborVec::iterator it = (mynode)->neighbors.begin(); it != (mynode)->neighbors.end(); it++) \
        if ((*it)->node != (mydad))

class PhyloNeighbor : public Neighbor {
public:
    double *partial_lh = nullptr;
    UBYTE *scale_num = nullptr;
    int partial_lh_computed = 0;
    int size = 0;
    RootDirection direction = UNDEFINED_DIRECTION;
};
class PhyloNode : public Node {};

/* ---- alignment (alignment/alignment.h): only what the kernels read ------- */
typedef vector<int> Pattern;
class Alignment : public vector<Pattern> {
public:
    int num_states = 0;
    int STATE_UNKNOWN = 0;
    int nsite = 0;
    int nseq = 0;
    int getNSite() { return nsite; }
    int getNSeq() { return nseq; }
};

/* ---- model (model/modelsubst.h) and rates (model/rateheterogeneity.h) ---- */
class ModelSubst {
public:
    int num_states = 0;
    int nmix = 1;
    double *eval = nullptr, *evec = nullptr, *inv_evec = nullptr, *freq = nullptr;
    double *mix_weight = nullptr;
    bool reversible = true;
    int getNMixtures() { return nmix; }
    double getMixtureWeight(int m) { return mix_weight ? mix_weight[m] : 1.0; }
    double *getEigenvalues() { return eval; }
    double *getEigenvectors() { return evec; }
    double *getInverseEigenvectors() { return inv_evec; }
    bool useRevKernel() { return reversible; }
    bool isSiteSpecificModel() { return false; }
    void getStateFrequency(double *out, int m = 0) { memcpy(out, freq + (size_t)m * num_states, sizeof(double) * num_states); }
    void writeInfo(ostream &) {}
};

class RateHeterogeneity {
public:
    vector<double> rate, prop;
    int getNRate() { return (int)rate.size(); }
    double getRate(int c) { return rate[c]; }
    double getProp(int c) { return prop[c]; }
    void writeInfo(ostream &) {}
};

class ModelFactory {
public:
    bool fused_mix_rate = false;
    vector<Pattern> unobserved_ptns;
    ASCType ASC_type = ASC_NONE;
    ASCType getASC() { return ASC_type; }
    void computeTransMatrix(double, double *, int = 0, int = -1) { iqref_fail("non-reversible models are not wired", __FILE__, __LINE__); }
};

/* ---- memory slots (tree/memslot.h): LM_PER_NODE only ---------------------- */
class MemSlotVector : public vector<int> {
public:
    bool lock(PhyloNeighbor *) { return false; }
    void unlock(PhyloNeighbor *) {}
    vector<int>::iterator findNei(PhyloNeighbor *) { return begin(); }
};

/* ---- TraversalInfo (tree/phylotree.h:320-333) ----------------------------- */
class TraversalInfo {
public:
    PhyloNeighbor *dad_branch;
    PhyloNode *dad;
    double *echildren;
    double *partial_lh_leaves;
    TraversalInfo(PhyloNeighbor *db, PhyloNode *d) : dad_branch(db), dad(d), echildren(nullptr), partial_lh_leaves(nullptr) {}
};

/* ---- PhyloTree: the members the kernel templates read and the member
 * templates they define (declarations with the signatures of
 * tree/phylotree.h:851-1320) ---------------------------------------------- */
class PhyloTree {
public:
    Alignment *aln = nullptr;
    ModelSubst *model = nullptr;
    RateHeterogeneity *site_rate = nullptr;
    ModelFactory *model_factory = nullptr;
    Params *params = nullptr;
    Node *root = nullptr;

    double *tip_partial_lh = nullptr;
    int tip_partial_lh_computed = 1;
    double *ptn_freq = nullptr;
    double *ptn_invar = nullptr;
    bool ptn_freq_computed = true;
    double *buffer_partial_lh = nullptr;
    double *central_partial_lh = nullptr;
    double *theta_all = nullptr;
    double *buffer_scale_all = nullptr;
    bool theta_computed = false;
    double *_pattern_lh = nullptr;
    double *_site_lh = nullptr;
    double *_pattern_lh_cat = nullptr;
    double *_pattern_scaling = nullptr;
    bool safe_numeric = false;
    PhyloNeighbor *current_it = nullptr, *current_it_back = nullptr;
    int num_threads = 1;
    int num_packets = 1;
    vector<TraversalInfo> traversal_info;
    MemSlotVector mem_slots;
    vector<const UBYTE *> tip_state_rows;  /* per taxon: converted sequence (one state per pattern) */

    void (PhyloTree::*computePartialLikelihoodPointer)(TraversalInfo &, size_t, size_t, int) = nullptr;

    /* non-template helpers the kernels call (restated in refkernels.cpp) */
    void computeTipPartialLikelihood() {}
    void computePtnFreq() {}
    void computePtnInvar() {}
    void initializeAllPartialLh() { iqref_fail("buffers are allocated by the harness", __FILE__, __LINE__); }
    bool isRootLeaf(Node *) { return false; }
    bool isMixlen() { return false; }
    int getMixlen() { return 1; }
    int getCurMixture() { return 0; }
    size_t getAlnNSite() { return aln->getNSite(); }
    int printTree(ostream &, int) { return 0; }
    void drawTree(ostream &) {}
    size_t getBufferPartialLhSize();
    const UBYTE *getConvertedSequenceByNumber(int seq) { return tip_state_rows[seq]; }
    ModelSubst *getModel() { return model; }
    RateHeterogeneity *getRate() { return site_rate; }
    void computePartialLikelihood(TraversalInfo &info, size_t lo, size_t hi, int packet) {
        (this->*computePartialLikelihoodPointer)(info, lo, hi, packet);
    }
    bool computeTraversalInfo(PhyloNeighbor *dad_branch, PhyloNode *dad, double *&buffer);

    template <class VectorClass> void computeTraversalInfo(PhyloNode *node, PhyloNode *dad, bool compute_partial_lh);
    template <class VectorClass, const int nstates>
    void computeTraversalInfo(PhyloNode *node, PhyloNode *dad, bool compute_partial_lh);
    template <class VectorClass>
    void computePartialInfo(TraversalInfo &info, VectorClass *buffer, double *echildren = NULL, double *partial_lh_leaves = NULL);
    template <class VectorClass, const int nstates>
    void computePartialInfo(TraversalInfo &info, VectorClass *buffer, double *echildren = NULL, double *partial_lh_leaves = NULL);

    template <class VectorClass, const bool SAFE_NUMERIC, const int nstates, const bool FMA = false, const bool SITE_MODEL = false>
    void computePartialLikelihoodSIMD(TraversalInfo &info, size_t ptn_lower, size_t ptn_upper, int thread_id);
    template <class VectorClass, const bool SAFE_NUMERIC, const bool FMA = false, const bool SITE_MODEL = false>
    void computePartialLikelihoodGenericSIMD(TraversalInfo &info, size_t ptn_lower, size_t ptn_upper, int thread_id);

    template <class VectorClass, const bool SAFE_NUMERIC, const int nstates, const bool FMA = false, const bool SITE_MODEL = false>
    double computeLikelihoodBranchSIMD(PhyloNeighbor *dad_branch, PhyloNode *dad, bool save_log_value = true);
    template <class VectorClass, const bool SAFE_NUMERIC, const bool FMA = false, const bool SITE_MODEL = false>
    double computeLikelihoodBranchGenericSIMD(PhyloNeighbor *dad_branch, PhyloNode *dad, bool save_log_value = true);

    template <class VectorClass, const int nstates, const bool FMA = false, const bool SITE_MODEL = false>
    double computeLikelihoodFromBufferSIMD();
    template <class VectorClass, const bool FMA = false, const bool SITE_MODEL = false>
    double computeLikelihoodFromBufferGenericSIMD();

    template <class VectorClass, const bool SAFE_NUMERIC, const int nstates, const bool FMA = false, const bool SITE_MODEL = false>
    void computeLikelihoodBufferSIMD(PhyloNeighbor *dad_branch, PhyloNode *dad, size_t ptn_lower, size_t ptn_upper, int thread_id);
    template <class VectorClass, const bool SAFE_NUMERIC, const bool FMA = false, const bool SITE_MODEL = false>
    void computeLikelihoodBufferGenericSIMD(PhyloNeighbor *dad_branch, PhyloNode *dad, size_t ptn_lower, size_t ptn_upper, int thread_id);

    template <class VectorClass, const bool SAFE_NUMERIC, const int nstates, const bool FMA = false, const bool SITE_MODEL = false>
    void computeLikelihoodDervSIMD(PhyloNeighbor *dad_branch, PhyloNode *dad, double *df, double *ddf);
    template <class VectorClass, const bool SAFE_NUMERIC, const bool FMA = false, const bool SITE_MODEL = false>
    void computeLikelihoodDervGenericSIMD(PhyloNeighbor *dad_branch, PhyloNode *dad, double *df, double *ddf);

    template <class VectorClass, const bool SAFE_NUMERIC, const int nstates, const bool FMA = false, const bool SITE_MODEL = false>
    void computeLikelihoodDervMixlenSIMD(PhyloNeighbor *dad_branch, PhyloNode *dad, double &df, double &ddf);
    template <class VectorClass, const bool SAFE_NUMERIC, const bool FMA = false, const bool SITE_MODEL = false>
    void computeLikelihoodDervMixlenGenericSIMD(PhyloNeighbor *dad_branch, PhyloNode *dad, double &df, double &ddf);
};

#endif
