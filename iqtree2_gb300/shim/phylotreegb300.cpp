/*
 * IQ-TREE 2 side of the drop-in boundary: PhyloTree's kernel function
 * pointers backed by the GB300 likelihood engine (libiqgpu, include/iqgpu.h).
 *
 * This translation unit is compiled inside an IQ-TREE 2 build that carries
 * the two patches beside it:
 *   phylotree_h.patch     declares the members below in class PhyloTree
 *                         (tree/phylotree.h), guarded by IQTREE_GB300;
 *   phylotreesse_cpp.patch makes PhyloTree::setLikelihoodKernel
 *                         (tree/phylotreesse.cpp:91) install them when the
 *                         environment asks for the engine (IQTREE_GB300=fp64,
 *                         or =mixed for the FP32 / split-TF32 paths), right
 *                         after the reference has chosen NORM or SAFE.
 * Link the build with -liqgpu. Callers (computeLikelihood, optimizeOneBranch,
 * optimizeAllBranches, NNI, UFBoot, ModelFinder) are unchanged: they call
 * the same four pointers (tree/phylotree.h:899-901, 947-948, 1000-1001,
 * 1342-1343), whose signatures the static_asserts below check.
 *
 * Partials live in HBM. A PhyloNeighbor's partial_lh pointer stays what the
 * reference makes it (a block of central_partial_lh, or of nni_partial_lh)
 * and names the engine slot with the same index, so the reference's own slot
 * management (LM_PER_NODE, reorientPartialLh, and the MemSlotVector recycling
 * of LM_MEM_SAVE, tree/memslot.h:44-74) decides which partial occupies which
 * slot; the host blocks are never read or written on this path. The host
 * traversal is the reference's own computeTraversalInfo(PhyloNeighbor*,
 * PhyloNode*, double*&) (tree/phylotree.cpp:5918-6028): the resulting
 * traversal_info becomes one op list and one engine launch.
 */
#include "tree/phylotree.h"

#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "iqgpu.h"

static_assert(std::is_same<decltype(&PhyloTree::computePartialLikelihoodGB300),
                           PhyloTree::ComputePartialLikelihoodType>::value,
              "computePartialLikelihoodPointer signature (tree/phylotree.h:899-901)");
static_assert(std::is_same<decltype(&PhyloTree::computeLikelihoodBranchGB300),
                           PhyloTree::ComputeLikelihoodBranchType>::value,
              "computeLikelihoodBranchPointer signature (tree/phylotree.h:947-948)");
static_assert(std::is_same<decltype(&PhyloTree::computeLikelihoodDervGB300),
                           PhyloTree::ComputeLikelihoodDervType>::value,
              "computeLikelihoodDervPointer signature (tree/phylotree.h:1342-1343)");
static_assert(std::is_same<decltype(&PhyloTree::computeLikelihoodFromBufferGB300),
                           PhyloTree::ComputeLikelihoodFromBufferType>::value,
              "computeLikelihoodFromBufferPointer signature (tree/phylotree.h:1000-1001)");

// A non-OK engine status ends the run the way the reference's own kernels
// do: outError (utils/tools.h) with the engine's message.
static void gpuCheck(int rc, const char *what) {
    if (rc == IQGPU_OK) return;
    string msg = string("GB300 likelihood engine (") + what + "): " + iqgpu_last_error();
    if (rc == IQGPU_ERR_NONFINITE) msg += ". Run again with the safe likelihood kernel via `-safe` option";
    outError(msg);
}

// cheap signature of an input array: re-upload only when the reference changed it
static uint64_t gpuSignature(const double *v, size_t n) {
    uint64_t h = 1469598103934665603ULL;
    for (size_t i = 0; i < n; i++) {
        uint64_t b;
        memcpy(&b, &v[i], sizeof b);
        h = (h ^ b) * 1099511628211ULL;
    }
    return h ^ n;
}

bool PhyloTree::isGB300() { return gpu_engine != nullptr || gpu_precision >= 0; }

void PhyloTree::setLikelihoodKernelGB300(int precision) {
    // safe_numeric was set by setLikelihoodKernel (tree/phylotreesse.cpp:95-96)
    if (model_factory && !model_factory->model->isReversible())
        outError("GB300 likelihood engine: non-reversible models are not wired into this binding yet");
    if (model_factory && model_factory->model->isSiteSpecificModel())
        outError("GB300 likelihood engine: site-specific models are not supported");
    gpu_precision = precision;
    computePartialLikelihoodPointer = &PhyloTree::computePartialLikelihoodGB300;
    computeLikelihoodBranchPointer = &PhyloTree::computeLikelihoodBranchGB300;
    computeLikelihoodDervPointer = &PhyloTree::computeLikelihoodDervGB300;
    computeLikelihoodFromBufferPointer = &PhyloTree::computeLikelihoodFromBufferGB300;
    computeLikelihoodDervMixlenPointer = nullptr;
    num_packets = 1;  // one launch covers every pattern
    if (gpu_engine) {
        iqgpu_destroy(gpu_engine);
        gpu_engine = nullptr;
    }
}

void PhyloTree::releaseGB300() {
    if (gpu_engine) iqgpu_destroy(gpu_engine);
    gpu_engine = nullptr;
}

// Patterns as the engine sees them: the alignment's, then +ASC's unobserved
// ones (which the reference keeps after a padded gap).
size_t PhyloTree::gpuPatternCount() { return aln->size() + model_factory->unobserved_ptns.size(); }

void PhyloTree::ensureEngineGB300() {
    if (!central_partial_lh) initializeAllPartialLh();
    if (gpu_engine) return;
    iqgpu_config cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.nptn = (int32_t)gpuPatternCount();
    cfg.nstates = aln->num_states;
    cfg.ncat = site_rate->getNRate() * (model_factory->fused_mix_rate ? 1 : model->getNMixtures());
    cfg.ntaxa = aln->getNSeq();
    cfg.state_unknown = aln->STATE_UNKNOWN;
    gpu_central_slots = (int32_t)max_lh_slots;
    cfg.nslots = gpu_central_slots + 2;  // + nni_partial_lh's two blocks
    cfg.safe = safe_numeric ? 1 : 0;
    cfg.precision = gpu_precision;
    cfg.device = 0;
    cfg.max_ops = 2 * (int32_t)nodeNum;
    // exactly the reference's kernel: its NORM/SAFE choice and its derivative sum
    cfg.flags = IQGPU_FLAG_SAFE_AS_GIVEN | IQGPU_FLAG_REF_TRIPLE_TAIL;
    if (const char *dev = getenv("IQTREE_GB300_DEVICE")) cfg.device = atoi(dev);
    gpuCheck(iqgpu_create(&cfg, &gpu_engine), "create");

    // tip states, taxon-major (getConvertedSequenceByNumber, tree/phylotree.cpp:3251)
    const size_t nptn = aln->size(), ntot = gpuPatternCount();
    vector<uint8_t> states((size_t)cfg.ntaxa * ntot);
    for (int t = 0; t < cfg.ntaxa; t++) {
        const char *row = getConvertedSequenceByNumber(t);
        uint8_t *dst = &states[(size_t)t * ntot];
        for (size_t p = 0; p < nptn; p++) dst[p] = (uint8_t)(row ? row[p] : (aln->at(p))[t]);
        for (size_t k = 0; k < ntot - nptn; k++) dst[nptn + k] = (uint8_t)model_factory->unobserved_ptns[k][t];
    }
    gpuCheck(iqgpu_set_tip_states(gpu_engine, states.data()), "tip states");
    gpu_model_sig = gpu_freq_sig = 0;
}

// Model and pattern inputs, uploaded when the reference has changed them.
void PhyloTree::syncInputsGB300() {
    ensureEngineGB300();
    if ((tip_partial_lh_computed & 1) == 0) computeTipPartialLikelihood();
    const int n = aln->num_states, nmix = model->getNMixtures();
    const int nrate = site_rate->getNRate();
    const int ncat = nrate * (model_factory->fused_mix_rate ? 1 : nmix);
    vector<double> rates(ncat), props(ncat);
    for (int c = 0; c < ncat; c++) {
        const int m = model_factory->fused_mix_rate ? c : c / nrate;
        rates[c] = site_rate->getRate(c % nrate);
        props[c] = site_rate->getProp(c % nrate) * model->getMixtureWeight(m);
    }
    uint64_t sig = gpuSignature(model->getEigenvalues(), (size_t)n * nmix) ^
                   gpuSignature(model->getEigenvectors(), (size_t)n * n * nmix) ^
                   gpuSignature(rates.data(), ncat) ^ gpuSignature(props.data(), ncat) ^
                   gpuSignature(tip_partial_lh, (size_t)(aln->STATE_UNKNOWN + 1) * n * nmix);
    if (sig != gpu_model_sig) {
        if (nmix > 1) {
            vector<double> freq((size_t)nmix * n);
            for (int m = 0; m < nmix; m++) model->getStateFrequency(&freq[(size_t)m * n], m);
            gpuCheck(iqgpu_set_mixture(gpu_engine, nmix, model->getEigenvalues(), model->getEigenvectors(),
                                       model->getInverseEigenvectors(), rates.data(), props.data(),
                                       tip_partial_lh, freq.data()),
                     "mixture");
        } else {
            vector<double> freq(n);
            model->getStateFrequency(freq.data());
            gpuCheck(iqgpu_set_model(gpu_engine, model->getEigenvalues(), model->getEigenvectors(),
                                     model->getInverseEigenvectors(), rates.data(), props.data()),
                     "model");
            gpuCheck(iqgpu_set_state_freq(gpu_engine, freq.data()), "state frequencies");
            gpuCheck(iqgpu_set_tip_partials(gpu_engine, tip_partial_lh), "tip vectors");
        }
        gpu_model_sig = sig;
    }
    if (!ptn_freq_computed) computePtnFreq();
    // compact the reference's padded layout: observed patterns, then +ASC's
    const size_t nptn = aln->size(), nunobs = model_factory->unobserved_ptns.size();
    const size_t pad = get_safe_upper_limit(nptn);
    vector<double> f(nptn + nunobs), inv(nptn + nunobs);
    for (size_t p = 0; p < nptn; p++) {
        f[p] = ptn_freq[p];
        inv[p] = ptn_invar[p];
    }
    for (size_t k = 0; k < nunobs; k++) {
        f[nptn + k] = ptn_freq[pad + k];
        inv[nptn + k] = ptn_invar[pad + k];
    }
    sig = gpuSignature(f.data(), f.size()) ^ (gpuSignature(inv.data(), inv.size()) * 3);
    if (sig != gpu_freq_sig) {
        gpuCheck(iqgpu_set_patterns(gpu_engine, f.data(), inv.data()), "pattern weights");
        // the engine copies pinned caller memory asynchronously: wait before f and inv go
        gpuCheck(iqgpu_sync(gpu_engine), "pattern weights");
        ASCType asc = model_factory->getASC();
        if (asc == ASC_VARIANT || asc == ASC_INFORMATIVE)
            gpuCheck(iqgpu_set_asc(gpu_engine, (int32_t)nunobs, (double)aln->getNSite()), "+ASC");
        else if (asc == ASC_VARIANT_MISSING)
            gpuCheck(iqgpu_set_asc_holder(gpu_engine, (int32_t)nptn), "+ASC (Holder)");
        gpu_freq_sig = sig;
    }
}

// The engine's name for the partial of the subtree behind `nei`: its HBM
// slot, from the block its partial_lh pointer names, or the tip taxon.
int32_t PhyloTree::gpuRef(PhyloNeighbor *nei) {
    if (nei->node->isLeaf()) return -1 - nei->node->id;
    const size_t block = getPartialLhSize();
    if (nei->partial_lh >= central_partial_lh &&
        nei->partial_lh < central_partial_lh + (size_t)gpu_central_slots * block)
        return (int32_t)((nei->partial_lh - central_partial_lh) / block);
    if (nni_partial_lh && nei->partial_lh >= nni_partial_lh && nei->partial_lh < nni_partial_lh + 2 * block)
        return gpu_central_slots + (int32_t)((nei->partial_lh - nni_partial_lh) / block);
    outError("GB300 likelihood engine: a partial outside the slot blocks");
    return 0;
}

// One traversal entry as engine op records: two children per record; a
// multifurcating node continues over records flagged IQGPU_OP_MORE.
void PhyloTree::appendOpsGB300(TraversalInfo &info, vector<iqgpu_op> &ops) {
    PhyloNode *node = (PhyloNode *)info.dad_branch->node;
    vector<int32_t> ref;
    vector<double> len;
    FOR_NEIGHBOR_IT(node, info.dad, it) {
        ref.push_back(gpuRef((PhyloNeighbor *)*it));
        len.push_back((*it)->length);
    }
    const int32_t dad = gpuRef(info.dad_branch);
    for (size_t k = 0; k < ref.size(); k += 2) {
        iqgpu_op op;
        memset(&op, 0, sizeof op);
        op.dad_slot = dad;
        op.child[0] = ref[k];
        op.len[0] = len[k];
        op.child[1] = k + 1 < ref.size() ? ref[k + 1] : IQGPU_NO_CHILD;
        op.len[1] = k + 1 < ref.size() ? len[k + 1] : 0.0;
        op.flags = k + 2 < ref.size() ? IQGPU_OP_MORE : 0;
        ops.push_back(op);
    }
}

// The reference's host traversal for both sides of branch dad-node, as ops.
void PhyloTree::traversalOpsGB300(PhyloNeighbor *dad_branch, PhyloNode *dad, vector<iqgpu_op> &ops) {
    PhyloNode *node = (PhyloNode *)dad_branch->node;
    PhyloNeighbor *node_branch = (PhyloNeighbor *)node->findNeighbor(dad);
    traversal_info.clear();
    double *unused = buffer_partial_lh;  // the walk carves host echild buffers the engine does not use
    bool dad_locked = computeTraversalInfo(dad_branch, dad, unused);
    bool node_locked = computeTraversalInfo(node_branch, node, unused);
    if (params->lh_mem_save == LM_MEM_SAVE) {  // as computeTraversalInfo<VC> (tree/phylokernelnew.h:1183-1188)
        if (dad_locked) mem_slots.unlock(dad_branch);
        if (node_locked) mem_slots.unlock(node_branch);
    }
    for (TraversalInfo &info : traversal_info) appendOpsGB300(info, ops);
    traversal_info.clear();
}

void PhyloTree::computePartialLikelihoodGB300(TraversalInfo &info, size_t ptn_lower, size_t ptn_upper,
                                              int packet_id) {
    // one call computes every pattern; the other packets have nothing to do
    if (packet_id != 0 || ptn_lower != 0) return;
    syncInputsGB300();
    vector<iqgpu_op> ops;
    appendOpsGB300(info, ops);
    gpuCheck(iqgpu_compute_partials(gpu_engine, ops.data(), (int32_t)ops.size()), "partials");
}

double PhyloTree::computeLikelihoodBranchGB300(PhyloNeighbor *dad_branch, PhyloNode *dad, bool save_log_value) {
    syncInputsGB300();
    PhyloNode *node = (PhyloNode *)dad_branch->node;
    PhyloNeighbor *node_branch = (PhyloNeighbor *)node->findNeighbor(dad);
    if (node->isLeaf()) {  // the leaf side becomes dad (tree/phylokernelnew.h:2652-2660)
        std::swap(node, dad);
        std::swap(dad_branch, node_branch);
    }
    vector<iqgpu_op> ops;
    traversalOpsGB300(dad_branch, dad, ops);
    double lnl = 0.0;
    gpuCheck(iqgpu_compute_likelihood(gpu_engine, ops.data(), (int32_t)ops.size(), gpuRef(dad_branch),
                                      gpuRef(node_branch), dad_branch->length, &lnl),
             "branch lnL");
    // _pattern_lh (UFBoot, AU tests, -wsl): copied back with every saved evaluation
    if (save_log_value) gpuCheck(iqgpu_get_pattern_lh(gpu_engine, _pattern_lh), "pattern lnL");
    return lnl;
}

void PhyloTree::computeLikelihoodDervGB300(PhyloNeighbor *dad_branch, PhyloNode *dad, double *df, double *ddf) {
    syncInputsGB300();
    PhyloNode *node = (PhyloNode *)dad_branch->node;
    PhyloNeighbor *node_branch = (PhyloNeighbor *)node->findNeighbor(dad);
    if (node->isLeaf()) {
        std::swap(node, dad);
        std::swap(dad_branch, node_branch);
    }
    vector<iqgpu_op> ops;
    if (!theta_computed) traversalOpsGB300(dad_branch, dad, ops);
    gpuCheck(iqgpu_likelihood_derv(gpu_engine, ops.data(), (int32_t)ops.size(), gpuRef(dad_branch),
                                   gpuRef(node_branch), dad_branch->length, theta_computed ? 1 : 0, df, ddf),
             "derivatives");
    theta_computed = true;
}

/* Optimization::minimizeNewton (utils/optimization.cpp:422-499) over
   computeFuncDerv (tree/phylotree.cpp:2529-2536) for the current branch of
   optimizeOneBranch (:2611), as one device kernel: the traversal and every
   Newton or bisection step run on the GPU with one host wait. Leaves the
   branch at the last evaluated length, as computeFuncDerv does. False when
   the engine keeps the host loop (mixed precision, non-reversible, +ASC,
   theta buffers above IQGPU_NEWTON_MAX_ENTRIES, super trees, mixlen). */
bool PhyloTree::minimizeNewtonGB300(double x1, double xguess, double x2, double xacc, double &d2l, int maxNRStep,
                                    double &optx) {
    int32_t supported = 0;
    if (!gpu_engine || isSuperTree() || getMixlen() > 1) return false;
    gpuCheck(iqgpu_newton_supported(gpu_engine, &supported), "Newton-Raphson");
    if (!supported) return false;
    syncInputsGB300();
    PhyloNeighbor *dad_branch = current_it, *node_branch = current_it_back;
    PhyloNode *dad = (PhyloNode *)current_it_back->node, *node = (PhyloNode *)current_it->node;
    if (node->isLeaf()) {
        std::swap(node, dad);
        std::swap(dad_branch, node_branch);
    }
    vector<iqgpu_op> ops;
    if (!theta_computed) traversalOpsGB300(dad_branch, dad, ops);
    double last = xguess;
    gpuCheck(iqgpu_newton_branch(gpu_engine, ops.data(), (int32_t)ops.size(), gpuRef(dad_branch),
                                 gpuRef(node_branch), theta_computed ? 1 : 0, x1, xguess, x2, xacc, maxNRStep, &optx,
                                 &d2l, &last, nullptr),
             "Newton-Raphson");
    theta_computed = true;
    current_it->length = last;
    current_it_back->length = last;
    return true;
}

double PhyloTree::computeLikelihoodFromBufferGB300() {
    double lnl = 0.0;
    gpuCheck(iqgpu_lnl_from_buffer(gpu_engine, current_it->length, &lnl), "lnL from buffer");
    gpuCheck(iqgpu_get_pattern_lh(gpu_engine, _pattern_lh), "pattern lnL");
    return lnl;
}
