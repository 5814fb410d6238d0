/*
 * iqgpu -- GB300 (sm_103a) Felsenstein-pruning likelihood engine, C ABI.
 *
 * This is the drop-in boundary for IQ-TREE 2's likelihood kernels. The
 * PhyloTree binding in iqtree2_gb300/shim/phylotreegb300.cpp binds these entry
 * points in place of the function pointers that PhyloTree::setLikelihoodKernel
 * installs (tree/phylotreesse.cpp:91-199):
 *
 *   computePartialLikelihoodPointer      -> iqgpu_compute_partials
 *   computeLikelihoodBranchPointer       -> iqgpu_branch_lnl / iqgpu_compute_likelihood
 *   computeLikelihoodDervPointer         -> iqgpu_likelihood_derv
 *   computeLikelihoodFromBufferPointer   -> iqgpu_lnl_from_buffer
 *
 * and reads the model through the same arrays as ModelSubst
 * (getEigenvalues/getEigenvectors/getInverseEigenvectors,
 * model/modelsubst.h:360-372) and RateHeterogeneity (getRate/getProp,
 * model/rategamma.h:106,120).
 *
 * Above the kernel level, iqgpu_tree_* is a C++ restatement of the PhyloTree
 * drivers that call those pointers (computeLikelihood, optimizeOneBranch,
 * optimizeAllBranches, computePatternLikelihood), so a caller that owns only
 * a tree and a model can use the engine without IQ-TREE's host code.
 *
 * Conventions. Plain pointers and sizes; every pointer argument is host
 * memory unless its name ends in _dev. Every entry point returns an int
 * status (IQGPU_OK or an IQGPU_ERR_* code); iqgpu_last_error() describes the
 * last failure on the calling thread. One engine owns one CUDA stream and is
 * used from one host thread at a time; different engines may be driven
 * concurrently from different threads (PhyloSuperTree calls partitions from
 * OpenMP threads, tree/phylosupertree.cpp:716-723).
 *
 * Host inputs. The setters (iqgpu_set_model, iqgpu_set_state_freq,
 * iqgpu_set_tip_partials, iqgpu_set_patterns, ...) take a copy of the
 * caller's arrays before they return and send it in stream order, so a
 * caller may overwrite or free its buffers at once (pinned memory included)
 * while the engine's stream is still busy. (Arrays of 16 KB or more in
 * page-locked memory are copied to the device from where they are, and the
 * setter returns once that copy has run.)
 *
 * Partial references. A directed partial (the reference's PhyloNeighbor
 * partial_lh: the subtree at `node` seen from `dad`) is named by an int32:
 * r >= 0 is an HBM slot, r < 0 is tip taxon (-1 - r).
 */
#ifndef IQGPU_H
#define IQGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define IQGPU_OK 0
#define IQGPU_ERR_ARG 1        /* bad argument or size */
#define IQGPU_ERR_OOM 2        /* device allocation or admission refused */
#define IQGPU_ERR_CUDA 3       /* CUDA runtime error */
#define IQGPU_ERR_NONFINITE 4  /* non-finite lnL/derivative (reference: outError "use -safe") */
#define IQGPU_ERR_TIMEOUT 5    /* a bounded device wait gave up */
#define IQGPU_ERR_STATE 6      /* call out of order (e.g. from-buffer before derivative) */
#define IQGPU_ERR_NODEV 7      /* no CUDA device, or the device is not sm_103 */
#define IQGPU_ERR_NEWTON 8     /* Newton-Raphson failed (reference: nrerror) */

/* ---- precision of the stored partials ---------------------------------- */
#define IQGPU_F64 0     /* FP64 eigen-space partials, uint8 2^-256 scale counts: the drop-in */
#define IQGPU_F32 1     /* FP32 standard-basis partials, per-pattern power-of-two exponents */
#define IQGPU_TF32X3 2  /* as F32, tensor-core contraction with split-TF32 (3 passes) for
                           16..64 states (fewer states: FP32 CUDA cores) */
#define IQGPU_BF16 3    /* as F32, tensor-core contraction with BF16 operands (1 pass, FP32
                           accumulate and storage) for 16..64 states; about 1e-3 relative
                           per partial, error reported, not a drop-in */

typedef struct {
    int32_t nptn;          /* patterns (aln->size()) */
    int32_t nstates;       /* aln->num_states, <= 64 */
    int32_t ncat;          /* site_rate->getNRate(), <= 16 */
    int32_t ntaxa;         /* leaves */
    int32_t state_unknown; /* aln->STATE_UNKNOWN, <= 255 */
    int32_t nslots;        /* partial-likelihood slots to reserve in HBM */
    int32_t safe;          /* 1 = SAFE (scale count per pattern x category), 0 = NORM; the engine
                              turns SAFE on by the reference's rule unless
                              IQGPU_FLAG_SAFE_AS_GIVEN (see below) */
    int32_t precision;     /* IQGPU_F64 ... */
    int32_t device;        /* CUDA device ordinal */
    int32_t max_ops;       /* largest traversal the engine must accept (>= ntaxa) */
    int32_t flags;         /* IQGPU_FLAG_* */
} iqgpu_config;

/* Reproduce the reference's derivative sum bit for bit: its dotProductTriple
 * (tree/phylokernelnew.h:699-718), called with N = nstates*ncat, adds the last
 * block entry twice when nstates is odd and N is even (codon +G4). Off by
 * default: the engine then returns the exact derivative of lnL. */
#define IQGPU_FLAG_REF_TRIPLE_TAIL 1
/* The reference picks SAFE scaling by itself (PhyloTree::setLikelihoodKernel,
 * tree/phylotreesse.cpp:95-96): with -safe, for trees of 2000 taxa or more
 * (params->numseq_safe_scaling, utils/tools.cpp:1262) and for every model
 * whose state count is not 4 or 20 (codon, binary, morphology). The engine
 * applies the same rule to cfg.safe at creation (iqgpu_get_config returns
 * the result); this flag takes cfg.safe as given instead. */
#define IQGPU_FLAG_SAFE_AS_GIVEN 2

/* One TraversalInfo entry (tree/phylotree.h:320-333): compute the partial of
 * dad_slot from two children with their branch lengths. flags is 0 for
 * reversible models; with a non-reversible model (iqgpu_set_model_nonrev) it
 * carries, per child, the reference's edge direction and root leaf
 * (tree/phylokernelnew.h:932-963): TRANSPOSE uses P(t)^T for a child reached
 * against the edge direction (child->direction == TOWARD_ROOT), ROOTLEAF makes
 * a tip child the root leaf, whose leaf-table rows are P(t) times the root
 * frequencies whatever its states (isRootLeaf). */
typedef struct {
    int32_t dad_slot;
    int32_t child[2];
    int32_t flags;
    double len[2];
} iqgpu_op;
#define IQGPU_OP_TRANSPOSE0 1
#define IQGPU_OP_TRANSPOSE1 2
#define IQGPU_OP_ROOTLEAF0 4
#define IQGPU_OP_ROOTLEAF1 8
/* Multifurcating nodes (node->degree() > 3, tree/phylokernelnew.h:1407-1631):
 * a dad with k > 2 children is given as ceil(k/2) consecutive records with the
 * same dad_slot, two children each, every record but the last flagged
 * IQGPU_OP_MORE; when k is odd the last record's child[1] is IQGPU_NO_CHILD.
 * Children keep the neighbour order of the node (the order of the products).
 * Reversible models; the FP64 drop-in follows the reference's multifurcating
 * update (products of the children's eigen-space sums, the 2^-256 check after
 * every child, one U^-1 transform at the end); mixed-precision engines run
 * such traversals on their fused CUDA-core kernel (a running product rescaled
 * by powers of two after every record). */
#define IQGPU_OP_MORE 16
#define IQGPU_NO_CHILD ((int32_t)0x80000000)

typedef struct iqgpu_engine iqgpu_engine;
typedef struct iqgpu_tree iqgpu_tree;

const char *iqgpu_last_error(void);
/* Bytes of HBM an engine with this config would hold (PhyloTree::getMemoryRequired,
 * tree/phylotree.cpp:967-1027). */
int iqgpu_memory_required(const iqgpu_config *cfg, size_t *bytes);

/* ---- engine lifetime and inputs ----------------------------------------- */
/* replaces initializeAllPartialLh (tree/phylotree.cpp:893-940) */
int iqgpu_create(const iqgpu_config *cfg, iqgpu_engine **out);
/* The same, with every device buffer carved from the caller's 256-byte
 * aligned region of at least iqgpu_memory_required() bytes; the engine then
 * calls no cudaMalloc/cudaFree (its side buffers for the NNI batch and RELL
 * excepted). Used by the serving loop to admit jobs into one HBM arena. */
int iqgpu_create_in(const iqgpu_config *cfg, void *dev_mem, size_t bytes, iqgpu_engine **out);
int iqgpu_destroy(iqgpu_engine *e);
/* The configuration an engine was created with. */
int iqgpu_get_config(const iqgpu_engine *e, iqgpu_config *out);
/* ModelSubst eigen arrays (model/modelsubst.h:360-372) + RateHeterogeneity
 * rates/props (model/rategamma.h:106,120). eval[n], evec[n*n], inv_evec[n*n]
 * row-major, rates[ncat], props[ncat]. A model change invalidates every slot
 * on the caller's side (ModelFactory clears partials, model/modelfactory.cpp:1124-1127). */
int iqgpu_set_model(iqgpu_engine *e, const double *eval, const double *evec, const double *inv_evec,
                    const double *rates, const double *props);
/* State frequencies pi[n] (ModelSubst::getStateFrequency, model/modelsubst.h).
 * The mixed-precision paths keep standard-basis partials and weight the root
 * by pi; the FP64 eigen-space path ignores it (pi is folded into U^-1). */
int iqgpu_set_state_freq(iqgpu_engine *e, const double *state_freq);
/* Eigen-space tip vectors, (state_unknown+1) x nstates
 * (computeTipPartialLikelihood, tree/phylotreesse.cpp:354-375). */
int iqgpu_set_tip_partials(iqgpu_engine *e, const double *tip_lh);
/* Pattern weights and +I constant-site terms (computePtnFreq/computePtnInvar,
 * tree/phylotreesse.cpp:537-612). ptn_invar may be NULL (all zero). */
int iqgpu_set_patterns(iqgpu_engine *e, const double *ptn_freq, const double *ptn_invar);
/* Tip states, ntaxa x nptn, one byte per state
 * (getConvertedSequenceByNumber, tree/phylotree.cpp:3251). */
int iqgpu_set_tip_states(iqgpu_engine *e, const uint8_t *states);

/* ---- kernel-level entry points (the reference's function pointers) ----- */
/* computePartialLikelihoodPointer over a traversal list, all patterns
 * (computePartialLikelihoodGenericSIMD, tree/phylokernelnew.h:1289-2039). */
int iqgpu_compute_partials(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops);
/* computeLikelihoodBranchPointer (tree/phylokernelnew.h:2641-3223): lnL on the
 * branch between partial a (dad_branch) and b (node_branch) of length len. */
int iqgpu_branch_lnl(iqgpu_engine *e, int32_t a, int32_t b, double len, double *lnl);
/* Fused traversal + branch lnL in one launch: the full computeLikelihood path. */
int iqgpu_compute_likelihood(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops,
                             int32_t a, int32_t b, double len, double *lnl);
/* computeLikelihoodDervPointer (tree/phylokernelnew.h:2233-2633). When
 * theta_computed is 0 the traversal runs first and theta (node o dad) is
 * rebuilt (computeLikelihoodBufferGenericSIMD :2048-2231); df and ddf are the
 * derivative sums of lnL in the length, not yet negated. */
int iqgpu_likelihood_derv(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops, int32_t a, int32_t b,
                          double len, int32_t theta_computed, double *df, double *ddf);
/* computeLikelihoodFromBufferPointer (tree/phylokernelnew.h:3232-3428). */
int iqgpu_lnl_from_buffer(iqgpu_engine *e, double len, double *lnl);
/* Optimization::minimizeNewton (utils/optimization.cpp:422-499) of one branch
 * length, with computeFuncDerv (tree/phylotree.cpp:2529-2536: f = -df,
 * df = -ddf) as its function, run as one device kernel: the traversal
 * (when theta_computed is 0, as for iqgpu_likelihood_derv) and every Newton or
 * bisection step happen on the GPU, and the host waits once. x1/xguess/x2/
 * xacc/max_nr_step mean what they mean to minimizeNewton; *optx receives its
 * return value, *d2l its d2l output (the last second-derivative value of
 * computeFuncDerv), *last_len the length of the last derivative evaluation
 * (where the reference leaves the branch: computeLikelihoodFromBuffer after
 * minimizeNewton reads it) and *steps the iterations taken; d2l, last_len
 * and steps may be NULL. Errors as the
 * reference's: IQGPU_ERR_NONFINITE for a non-finite NORM derivative,
 * IQGPU_ERR_NEWTON for "Wrong computeFuncDerv" or the iteration limit.
 * Reversible FP64 engines without +ASC whose theta buffer holds at most
 * IQGPU_NEWTON_MAX_ENTRIES doubles (patterns x states x categories); other
 * engines return IQGPU_ERR_ARG before doing anything, and callers iterate
 * iqgpu_likelihood_derv on the host as minimizeNewton does. The theta buffer
 * stays valid for iqgpu_lnl_from_buffer at any length afterwards. */
#define IQGPU_NEWTON_MAX_ENTRIES (1 << 18)
/* *supported = 1 when iqgpu_newton_branch serves this engine, else 0. */
int iqgpu_newton_supported(iqgpu_engine *e, int32_t *supported);
int iqgpu_newton_branch(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops, int32_t a, int32_t b,
                        int32_t theta_computed, double x1, double xguess, double x2, double xacc,
                        int32_t max_nr_step, double *optx, double *d2l, double *last_len, int32_t *steps);
/* Per-pattern lnL of the last branch/from-buffer evaluation (_pattern_lh);
 * with +ASC the observed patterns carry the correction term. */
int iqgpu_get_pattern_lh(iqgpu_engine *e, double *out);
/* +ASC (Lewis ascertainment bias correction, ASC_VARIANT): the last `nconst`
 * patterns of the engine are the unobserved constant patterns IQ-TREE appends
 * with weight 0 (one per state whose taxa all show it and that the alignment
 * lacks: Alignment::getUnobservedConstPatterns, alignment/alignment.cpp:
 * 4140-4156). With P_const the sum of their likelihoods, every lnL entry point
 * returns lnL - nsite * log(1 - P_const) and the observed patterns' lnL drop
 * by log(1 - P_const) (tree/phylokernelnew.h:3198-3222, 3405-3420); the
 * derivative adds nsite * (d1/(1-P)) and nsite * (d2/(1-P) + (d1/(1-P))^2)
 * with d1, d2 the constant patterns' summed derivatives (:2620-2628).
 * The same formula with the uninformative patterns as the unobserved ones is
 * the correction for informative sites (ASC_INFORMATIVE, alignment/alignment.cpp:
 * 4181-4192): nconst may be any count below the number of patterns.
 * nconst = 0 switches it off. The batched NNI, group and on-device RELL entry
 * points refuse +ASC engines (IQGPU_ERR_ARG); iqgpu_rell takes the corrected
 * pattern lnL from iqgpu_get_pattern_lh. */
int iqgpu_set_asc(iqgpu_engine *e, int32_t nconst, double nsite);
/* Holder's +ASC for variant sites with missing data (ASC_VARIANT_MISSING,
 * alignment/alignment.cpp:4158-4180; tree/phylokernelnew.h:3175-3196 for the
 * lnL, :2580-2617 for the derivatives): the first nobs patterns are the
 * observed ones and the last nstates * nobs the unobserved ones with weight 0,
 * block s holding, for observed pattern p, state s at every taxon where p has
 * data and STATE_UNKNOWN elsewhere. Every pattern lnL drops by log(1 - P_p),
 * P_p the sum of its unobserved patterns' likelihoods, the tree lnL by
 * sum_p freq_p log(1 - P_p); the derivatives gain the matching terms.
 * iqgpu_set_asc(e, 0, 0) switches it off. Refused with non-reversible models;
 * the batched NNI, group and on-device RELL entry points refuse +ASC engines. */
int iqgpu_set_asc_holder(iqgpu_engine *e, int32_t nobs);
/* Mixture model (ModelMixture: profile mixtures such as C10-C60, LG4X, ...)
 * on every path: nmix classes, each with its own eigen system
 * and state frequencies; the ncat categories (a multiple of nmix) are class
 * blocks of ncat/nmix rate categories, category c belonging to class
 * c / (ncat/nmix) (tree/phylokernelnew.h:908-918; with fused mix-rate,
 * ncat = nmix and category c is class c). Arrays by class: eval [nmix][n],
 * evec and inv_evec [nmix][n][n], state_freq [nmix][n]; tip_lh
 * [STATE_UNKNOWN+1][nmix][n] (the reference's tip_partial_lh layout); rates
 * and props per category (props = rate proportion x class weight,
 * :2327). iqgpu_set_model goes back to one class. On FP64 engines each
 * category's partial lives in its class's eigen basis, as in the reference's
 * kernels. The batched NNI entry point refuses mixtures (IQGPU_ERR_ARG). */
int iqgpu_set_mixture(iqgpu_engine *e, int32_t nmix, const double *eval, const double *evec, const double *inv_evec,
                      const double *rates, const double *props, const double *tip_lh, const double *state_freq);
/* Non-reversible model (ModelMarkov with is_reversible false: UNREST, NONREV,
 * Lie-Markov; model/modelmarkov.cpp:463-505, 732-756) on every path. The partials stay in the standard basis (the reference's nonrev
 * kernels, tree/phylokernelnonrev.h); P(r_c t) = Re(V diag(exp(lambda r_c t))
 * V^-1) from the complex eigen system of the normalised rate matrix, each
 * array given as real and imaginary parts: ceval [n], cevec and cinv_evec
 * [n][n] row-major. tip_vec [STATE_UNKNOWN+1][n] are the standard-basis tip
 * vectors (the unknown state's row all ones), root_freq [n] the root-leaf
 * vector. The branch lnL and derivatives weigh the dad side by the state
 * frequencies of iqgpu_set_state_freq: the stationary frequencies for an
 * unrooted tree (tree/phylokernelnonrev.h:1117-1130), all ones for a rooted
 * tree whose root leaf carries root_freq. Derivatives use r_c lambda and
 * (r_c lambda)^2 on the same eigen system (Q P and Q^2 P,
 * tree/phylokernelnonrev.h:628-660). On FP64 engines the partials are
 * standard-basis (the traversal's dad transform becomes the identity) with
 * the reference's NORM / SAFE scale counts. Mixtures, +ASC and the batched
 * NNI / group entry points refuse non-reversible models. */
int iqgpu_set_model_nonrev(iqgpu_engine *e, const double *ceval_re, const double *ceval_im, const double *cevec_re,
                           const double *cevec_im, const double *cinv_re, const double *cinv_im,
                           const double *rates, const double *props, const double *tip_vec,
                           const double *root_freq);
/* Copy a slot back in the reference layout: partial[ptn*B + c*n + x] in eigen
 * space (F64) or standard basis (mixed), and scale counts (NORM: nptn bytes,
 * SAFE: nptn*ncat bytes, pattern-major). Either output may be NULL. */
int iqgpu_get_partial(iqgpu_engine *e, int32_t slot, double *partial, uint8_t *scale);
/* Mixed precision: per-pattern power-of-two exponent of a slot (int32, nptn). */
int iqgpu_get_exponent(iqgpu_engine *e, int32_t slot, int32_t *exponent);
/* Wait for all work of this engine. */
int iqgpu_sync(iqgpu_engine *e);
/* Run this engine's work on the caller's CUDA stream (a cudaStream_t passed
 * as void*); NULL returns to the engine's own stream. */
int iqgpu_set_stream(iqgpu_engine *e, void *cuda_stream);
/* Kernel timing with CUDA events on the engine's stream around every
 * traversal launch (the dominant kernel): enable, read (total ms and number
 * of timed launches since the last reset), reset. */
int iqgpu_set_timing(iqgpu_engine *e, int32_t enable);
/* Pattern tile (patterns per CTA, 32/64/128) of the mixed-precision traversal
 * kernel; 0 restores the default. 4-state models also take 1 (one thread per
 * pattern and all its categories) and 2 (as 1, two patterns per thread, level
 * schedule). Chosen by the autotuner in iqtree2_gb300/autotune.py; results do
 * not depend on it. */
int iqgpu_set_tile(iqgpu_engine *e, int32_t patterns_per_cta);
/* Schedule of the mixed-precision traversal: 0 = one fused launch walking the
 * whole op list per pattern tile; 1 = one launch per tree level, all of the
 * level's (op, tile) pairs in flight together; 2 = dataflow: one persistent
 * launch hands out (op, tile) pairs in level order and each waits (bounded)
 * for its children's pairs (4-state one-thread-per-pattern kernel, tile 1;
 * other kernels run fused); 3 = as 1, with the warp-specialised tensor-core
 * kernel (a copy/MMA issuer warp beside four worker warps; other kernels run
 * as 1); 4 = as 1, with the tensor-core kernel that keeps operand A in tensor
 * memory (20-state models in IQGPU_TF32X3; others run as 3); 5 = as 3, and
 * the narrow levels of models up to 32 padded states run as (tile, op,
 * category) items on the tensor cores, as 61-state models always do, instead
 * of on the CUDA-core tail; 6 = dataflow on the tensor cores: leading
 * tip-tip levels as in 1, then every other op in one persistent launch of
 * (tile, op, category) items handed out in level order, each item's copies
 * issued once the items writing its children are done (bounded waits; the
 * level form of 5 when the traversal has more (op, tile) pairs than the
 * engine's pair counters; other kernels run as 3); 7 = as 6 with whole
 * (tile, op) items (every category of the pair in one item); 8 = as 1 on the
 * deep-ring tensor-core kernel (20-state models in IQGPU_TF32X3: one CTA per
 * SM, a ring of six (tile, op, category) stages landed by TMA, operand A
 * split into TF32 hi/lo in tensor memory; the one-op levels near the root on
 * the CUDA-core tail; others run as 3); 9 = as 8, with those one-op levels
 * in one more launch of the same kernel, each CTA taking its pattern tiles
 * through all of them in level order. Results do not depend on it. */
int iqgpu_set_schedule(iqgpu_engine *e, int32_t schedule);
/* Copy depth of the tensor-core traversal (precision IQGPU_TF32X3 / BF16):
 * how many child slices per CTA may be in flight as TMA copies (landing slots
 * of shared memory), 2, 3 or 4; 0 = default (3). A depth whose shared memory
 * does not fit one CTA is lowered. Chosen by the autotuner; results do not
 * depend on it. */
int iqgpu_set_stages(iqgpu_engine *e, int32_t stages);
/* K pieces per copied stage of the tensor-core traversal: 0/1 = a stage
 * carries a category's whole K; 2 = halves (61-state models: half the shared
 * memory per stage, two CTAs per SM instead of one); 4 = quarters with one
 * accumulator buffer per CTA (61-state models on schedule 6: a quarter of the
 * shared memory per stage and half the tensor memory, four CTAs per SM).
 * Ignored where K does not split evenly. Chosen by the autotuner; results do
 * not depend on it. */
int iqgpu_set_kpieces(iqgpu_engine *e, int32_t pieces);
int iqgpu_get_timing(iqgpu_engine *e, double *total_ms, int64_t *launches);
/* Failure detection (no counterpart in the reference, whose kernels cannot
 * wait on each other): the number of polls after which a wait on another
 * CTA's progress -- the dataflow schedule's producer flags -- gives up; the
 * launch then stops, the call returns IQGPU_ERR_TIMEOUT and the engine stays
 * usable (its next call runs normally). 0 restores the built-in limit (about
 * seconds). Waits for the engine's own TMA copies and MMAs keep a fixed
 * limit. */
int iqgpu_set_wait_limit(iqgpu_engine *e, uint32_t polls);
/* Kernel launches issued by this engine so far (all entry points). */
int iqgpu_get_launches(iqgpu_engine *e, int64_t *launches);

/* ---- batched evaluation ------------------------------------------------- */
/* One NNI candidate around a central branch node1-node2 (getBestNNIForBran,
 * tree/phylotree.cpp:4069-4320): after the swap, sub[0] and sub[1] hang off
 * node1 and sub[2], sub[3] off node2 (partial references: slot or tip),
 * len[] are their branch lengths; scratch[] are two slots the engine may
 * overwrite with the candidate's node1/node2 partials (the reference's
 * nni_partial_lh); central is the starting central-branch length. */
typedef struct {
    int32_t sub[4];
    int32_t scratch[2];
    double len[4];
    double central;
} iqgpu_nni_candidate;

/* Evaluate a batch of NNI candidates with one optimised branch each (-nni1):
 * both new partials of every candidate in one traversal launch, then theta,
 * Newton-Raphson on every central branch (minimizeNewton with max_nr_step,
 * xacc = min_bl) and the final lnL in one CUDA graph. lnl[k] and
 * central_len[k] receive each candidate's result. Mixed-precision engines;
 * 2*ncand <= max_ops. */
int iqgpu_nni_batch(iqgpu_engine *e, const iqgpu_nni_candidate *cand, int32_t ncand, int32_t max_nr_step,
                    double min_bl, double max_bl, double *lnl, double *central_len);

/* UFBoot resampled pattern weights, nreps x nptn, kept resident in HBM
 * (Alignment::createBootstrapAlignment, alignment/alignment.cpp:3795-3830). */
int iqgpu_set_boot_weights(iqgpu_engine *e, const float *weights, int32_t nreps);
/* RELL scores of ntrees trees: out[t*nreps + r] = sum_ptn pattern_lh[t*nptn + ptn]
 * * weight[r][ptn] (saveCurrentTree, tree/iqtree.cpp:3551-3630); FP32 products
 * like the reference's float dot product, FP64 accumulation every 256 patterns. */
int iqgpu_rell(iqgpu_engine *e, const double *pattern_lh, int32_t ntrees, double *out);
/* RELL scores of the tree whose lnL was computed last, read from its pattern
 * lnL on the device (no host copy): out[r] for every replicate r. */
int iqgpu_rell_current(iqgpu_engine *e, double *out);

/* ---- serving: continuous batching of jobs ------------------------------ */
/* A job is one likelihood + branch-optimisation request on its own tree and
 * alignment (computeLikelihood, then optimizeAllBranches with opt_iterations
 * rounds; 0 = lnL only). The server copies every input at submission. */
typedef struct {
    int32_t ntaxa, nptn, nstates, ncat, state_unknown, opt_iterations;
    const double *eval, *evec, *inv_evec, *rates, *props, *state_freq, *tip_lh;
    const double *ptn_freq;
    const uint8_t *tip_states;  /* ntaxa x nptn */
    const int32_t *edges;       /* 2 x (2*ntaxa-3) */
    const double *lengths;      /* 2*ntaxa-3 */
    double tolerance;           /* optimizeAllBranches tolerance (0 = 1e-3) */
} iqgpu_job;

typedef struct {
    int64_t id;
    int32_t status;             /* IQGPU_OK, IQGPU_ERR_OOM if refused, ... */
    int32_t slots;              /* partial slots of the job's engine; fewer than the tree's
                                   3*(ntaxa-2) directed partials means they were recycled */
    double lnl_initial, lnl;    /* before and after branch optimisation */
    double t_submit, t_start, t_end;  /* seconds since the server started */
    int64_t bytes;              /* HBM the job's engine held */
    char error[128];
} iqgpu_job_result;

typedef struct {
    int32_t device, precision_unused, max_active, pad;
    uint64_t memory_budget;     /* arena bytes; 0 = 90% of free HBM */
} iqgpu_server_config;

typedef struct {
    int64_t submitted, admitted, refused, completed, peak_active;
    uint64_t peak_bytes, arena_bytes;
} iqgpu_server_stats;

typedef struct iqgpu_server iqgpu_server;

/* Reserve the arena and start the scheduler. Jobs are admitted in arrival
 * order when a worker slot (max_active) is free and their engine fits in the
 * arena's free space. A job whose partials do not fit in half the arena gets
 * an engine with fewer partial slots than its tree has directed partials,
 * recycled least-recently-used first and recomputed when needed (the
 * reference's LM_MEM_SAVE, tree/memslot.h:44-74, tree/phylotree.cpp:967-1027);
 * a job that does not fit even then is refused (IQGPU_ERR_OOM). Admitted
 * jobs run concurrently, each on its own stream. */
int iqgpu_server_create(const iqgpu_server_config *cfg, iqgpu_server **out);
/* Queue a job (precision IQGPU_F64 or IQGPU_F32); returns its id at once. */
int iqgpu_server_submit(iqgpu_server *s, const iqgpu_job *job, int32_t precision, int64_t *id);
/* Block until the job finishes; lengths (optional, 2*ntaxa-3) get the optimised branch lengths. */
int iqgpu_server_wait(iqgpu_server *s, int64_t id, iqgpu_job_result *out, double *lengths);
int iqgpu_server_get_stats(iqgpu_server *s, iqgpu_server_stats *out);
/* Finish queued and running jobs, then release the arena. */
int iqgpu_server_destroy(iqgpu_server *s);

/* Seeded sequence simulation on the device (benchmark inputs; no counterpart
 * on the reference's likelihood path). Edges in preorder: edge_parent[0] is
 * the root and every parent appears as a child (or the root) before its own
 * edges; cum_trans[edge][cat][x][y] are cumulative rows of P(r_cat t_edge),
 * cum_freq the cumulative root frequencies. Writes ntaxa x nsites states. */
int iqgpu_simulate(int32_t ntaxa, int64_t nsites, int32_t nstates, int32_t ncat, const int32_t *edge_parent,
                   const int32_t *edge_child, const float *cum_trans, const float *cum_freq, uint64_t seed,
                   int32_t device, uint8_t *states_out);

/* ---- derivative sums without device allocation ------------------------- */
/* No counterpart in the reference. For callers that may not allocate device
 * memory when they need a derivative (GPU memory owned by a pool they must
 * not bypass, a pipeline that cannot afford the device synchronisation of
 * cudaMalloc/cudaFree, or only borrowed device buffers at hand): the FP64
 * derivative sums of iqgpu_likelihood_derv for reversible single-class
 * models (one eigen system; no mixture classes, no +ASC terms, and the exact
 * sum rather than IQGPU_FLAG_REF_TRIPLE_TAIL's), from a theta buffer the
 * caller owns. All pointers ending in _dev are device memory:
 * theta_dev[B][ldp] (B = nstates*ncat, eigen space, row c*nstates+x),
 * buffer_scale_dev/freq_dev/invar_dev[nptn]; eval/rates/props are host
 * arrays. out_dev receives {df, ddf, lnl}: the sums of lnL's first and
 * second derivatives in the branch length and lnL itself at len. The kernel
 * runs on cuda_stream (NULL = legacy default stream); nothing is allocated or
 * freed. Its only scratch is a static device array sized for at most 524,288
 * patterns; larger nptn is rejected with IQGPU_ERR_ARG. Every call on a
 * device shares that array, so calls whose kernels overlap on the GPU race:
 * serialise them (one stream, or events). The first call on each device
 * resolves the array's device address (set-up that must not happen inside a
 * stream capture), so make one call on each device before capturing. The
 * address is kept for the life of the process: after cudaDeviceReset on a
 * device, the next call there would use a stale address, so do not reset a
 * device between calls. */
int iqgpu_derv_noalloc(const double *theta_dev, const double *buffer_scale_dev, const double *freq_dev,
                       const double *invar_dev, int32_t nptn, int64_t ldp, int32_t nstates, int32_t ncat,
                       const double *eval, const double *rates, const double *props, double len,
                       double *out_dev, void *cuda_stream);

/* ---- tree-level drivers (PhyloTree restatement) ------------------------ */
/* edges[2*k], edges[2*k+1]: endpoints of branch k; leaves are 0..ntaxa-1,
 * internal nodes ntaxa..2*ntaxa-3; a node's neighbour order is edge order. */
int iqgpu_tree_create(iqgpu_engine *e, const int32_t *edges, const double *lengths, iqgpu_tree **out);
/* The same for a tree with multifurcating nodes (degree 3 to 32): nedge edges
 * (ntaxa .. 2*ntaxa-3), internal nodes ntaxa..nedge; the engine needs a slot
 * per directed internal partial (multifurcating updates follow the
 * reference's, tree/phylokernelnew.h:1407-1631). */
int iqgpu_tree_create_n(iqgpu_engine *e, int32_t nedge, const int32_t *edges, const double *lengths,
                        iqgpu_tree **out);
int iqgpu_tree_destroy(iqgpu_tree *t);
/* PhyloTree::computeLikelihood (tree/phylotree.cpp:1233-1280). pattern_lh may be NULL. */
int iqgpu_tree_compute_likelihood(iqgpu_tree *t, double *lnl, double *pattern_lh);
/* PhyloTree::optimizeOneBranch (tree/phylotree.cpp:2594-2644) */
int iqgpu_tree_optimize_one_branch(iqgpu_tree *t, int32_t node1, int32_t node2, int32_t max_nr_step);
/* PhyloTree::optimizeAllBranches (tree/phylotree.cpp:2698-2774) */
int iqgpu_tree_optimize_all_branches(iqgpu_tree *t, int32_t iterations, double tolerance,
                                     int32_t max_nr_step, double *lnl);
int iqgpu_tree_get_lengths(iqgpu_tree *t, double *lengths);
int iqgpu_tree_set_lengths(iqgpu_tree *t, const double *lengths);
/* params->min_branch_length / max_branch_length (defaults 1e-6, 10) */
int iqgpu_tree_set_bounds(iqgpu_tree *t, double min_bl, double max_bl);
/* Pattern-node updates executed so far (throughput accounting). */
int iqgpu_tree_num_updates(iqgpu_tree *t, int64_t *updates);
/* Where optimizeOneBranch runs minimizeNewton: on the device through
 * iqgpu_newton_branch (on = 1, the default; engines it does not serve keep the
 * host loop) or on the host, one iqgpu_likelihood_derv per step (on = 0).
 * With on = 1 iqgpu_tree_optimize_all_branches runs each pass over the
 * branches on the device with one host wait per pass, where the engine is not
 * in a caller's region and every directed internal partial has a slot of its
 * own (a pass that meets the 0.95 max_bl comparison or an error is taken again
 * branch by branch); on = 2 keeps one host wait per branch. */
int iqgpu_tree_set_device_newton(iqgpu_tree *t, int32_t on);

/* ---- partitions: one graph launch over several engines ------------------- */
/* Replaces the OpenMP loop of PhyloSuperTree::computeLikelihood
 * (tree/phylosupertree.cpp:701-723) over per-partition PhyloTrees: a group of
 * engines (one per partition, each with its own model, patterns, buffers and
 * stream, all on one device) whose branch-lnL evaluations are captured into
 * one CUDA graph (the partitions' kernels run concurrently on forked streams)
 * and replayed with one launch. */
typedef struct iqgpu_group iqgpu_group;
int iqgpu_group_create(iqgpu_engine *const *engines, int32_t n, iqgpu_group **out);
/* Per member: op list (ops[i], nops[i]) that makes partial a current, and the
 * branch (a[i], b[i], len[i]) to evaluate. Stages the lists, captures and
 * instantiates the graph. */
int iqgpu_group_prepare(iqgpu_group *g, const iqgpu_op *const *ops, const int32_t *nops, const int32_t *a,
                        const int32_t *b, const double *len);
/* New branch lengths for the same traversals (same slots and children). */
int iqgpu_group_set_lengths(iqgpu_group *g, const iqgpu_op *const *ops, const double *len);
/* One replay: lnL of every member (per_part may be NULL) and their sum. */
int iqgpu_group_lnl(iqgpu_group *g, double *per_part, double *total);
int iqgpu_group_destroy(iqgpu_group *g);

#ifdef __cplusplus
}
#endif
#endif
