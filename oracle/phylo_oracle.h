/*
 * CPU FP64 oracle for the Felsenstein-pruning likelihood path.
 *
 * TEST INFRASTRUCTURE ONLY. Tests, the smoke check and the bench's CPU
 * baseline legs use this to check and to time against; nothing in the
 * product links it.
 *
 * It restates IQ-TREE 2's scalar kernel path (tree/phylokernelnew.h with a
 * one-lane vector class, as the reference builds it when INSTRSET < 2,
 * tree/phylotreesse.cpp:186-191) plus the host drivers around it
 * (tree/phylotree.cpp, utils/optimization.cpp). Storage follows the
 * reference: a partial is pattern-major, partial[ptn*B + c*n + x] with
 * B = n*ncat, in eigen space; scale counts are uint8, one per pattern (NORM)
 * or per pattern x category (SAFE).
 *
 * Parity status: pinned to the reference's own compiled kernels. The whole
 * reference does not build here (Eigen3, Boost, cmake-generated headers), but
 * its kernel templates do: oracle/ref/ compiles tree/phylokernelnew.h against
 * a stand-in PhyloTree environment into oracle/_ref/, and the tests require
 * this oracle (one thread) to reproduce those kernels bit for bit. It is also
 * checked against analytic known-answer tests (closed-form two-taxon JC69,
 * zero-length star trees, P(t) row sums) and an independent standard-basis
 * pruning written in numpy.
 */
#ifndef IQ_PHYLO_ORACLE_H
#define IQ_PHYLO_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2^-256 and its log: tree/phylotree.h:74-80 */
#define ORC_SCALING_THRESHOLD_EXP 256
#define ORC_SCALING_THRESHOLD 8.636168555094444625386e-78
#define ORC_LOG_SCALING_THRESHOLD -177.4456782233459932741

typedef struct {
    int nptn, nstates, ncat, ntaxa, state_unknown, safe;
    const double *eval;      /* n */
    const double *evec;      /* n*n, U[x][i] */
    const double *inv_evec;  /* n*n, Uinv[i][j] */
    const double *rates;     /* ncat */
    const double *props;     /* ncat */
    const double *tip_lh;    /* (state_unknown+1)*n, eigen-space tip vectors */
    const double *ptn_freq;  /* nptn */
    const double *ptn_invar; /* nptn */
    const uint8_t *tip_states; /* ntaxa*nptn */
    /* 1: the reference's dotProductTriple, which adds the last block entry a
     * second time when nstates is odd and nstates*ncat even
     * (tree/phylokernelnew.h:699-718); 0: the exact derivative sum. */
    int ref_triple_tail;
    /* +ASC (Lewis): the last asc_n patterns are the unobserved constant
     * patterns appended with weight 0 (alignment/alignment.cpp:4140-4156);
     * lnL, pattern lnL and derivatives are corrected for them with asc_nsite
     * sites (tree/phylokernelnew.h:2506-2546 and 2620-2628 derivatives,
     * 2936-2966 and 3198-3222 branch lnL, 3341-3365 and 3405-3420 lnL from
     * the buffer). 0 = off. */
    int asc_n;
    double asc_nsite;
} orc_model;

/* Largest node degree of a tree (a multifurcating node of degree d has d-1
 * children in a traversal). */
#define ORC_MAX_DEG 32

/* A reference to a directed partial: >= 0 is a slot, < 0 is tip taxon
 * (-1-ref). An op has nchild >= 2 children in the node's neighbour order;
 * nchild > 2 is a multifurcating node (tree/phylokernelnew.h:1407-1631). */
typedef struct {
    int dad_slot;
    int nchild;
    int child[ORC_MAX_DEG - 1];
    double len[ORC_MAX_DEG - 1];
} orc_op;

/* Partial update for a traversal list (computePartialLikelihoodGenericSIMD). */
void orc_compute_partials(const orc_model *m, double *partials, uint8_t *scale,
                          const orc_op *ops, int nops, int nthreads);

/* Branch lnL (computeLikelihoodBranchGenericSIMD). `a` is the dad_branch
 * partial, `b` the node_branch partial; either may be a tip. pattern_lh may
 * be NULL. Returns lnL. */
double orc_branch_lnl(const orc_model *m, const double *partials, const uint8_t *scale,
                      int a, int b, double len, double *pattern_lh, int nthreads);

/* theta = node o dad plus per-pattern scale offset (computeLikelihoodBufferGenericSIMD). */
void orc_compute_theta(const orc_model *m, const double *partials, const uint8_t *scale,
                       int a, int b, double *theta, double *buffer_scale, int nthreads);

/* First and second derivative sums of lnL w.r.t. the branch length
 * (computeLikelihoodDervGenericSIMD). */
void orc_derv(const orc_model *m, const double *theta, const double *buffer_scale, double len,
              double *df, double *ddf, int nthreads);
/* Lewis +ASC correction of a tree lnL and of the observed patterns' lnL. */
double orc_asc_lewis_lnl(const orc_model *m, double tree_lh, double prob_const, double *plh);

/* lnL from the theta buffer (computeLikelihoodFromBufferGenericSIMD). */
double orc_lnl_from_buffer(const orc_model *m, const double *theta, const double *buffer_scale,
                           double len, double *pattern_lh, int nthreads);

/* ---- tree-level drivers (PhyloTree restatement) ---- */
typedef struct orc_tree orc_tree;

/* nedge edges edges[2k], edges[2k+1]; leaves are 0..ntaxa-1, internal nodes
 * any ids above (2*ntaxa-3 edges for a binary tree, fewer with multifurcating
 * nodes); a node's neighbour order is edge order. */
orc_tree *orc_tree_new(const orc_model *m, const int *edges, int nedge, const double *lengths, int nthreads);
void orc_tree_free(orc_tree *t);
double orc_tree_compute_likelihood(orc_tree *t, double *pattern_lh);
/* optimizeOneBranch on the branch between node1 and node2. Returns 0 or -1 on NR failure. */
int orc_tree_optimize_one_branch(orc_tree *t, int node1, int node2, int max_nr_step);
/* optimizeAllBranches; returns the final lnL. status (optional) gets 0 or -1. */
double orc_tree_optimize_all_branches(orc_tree *t, int iterations, double tolerance,
                                      int max_nr_step, int *status);
void orc_tree_get_lengths(const orc_tree *t, double *lengths);
void orc_tree_set_lengths(orc_tree *t, const double *lengths);
void orc_tree_set_bounds(orc_tree *t, double min_bl, double max_bl);
/* Number of partial updates (ops) executed so far, for throughput accounting. */
long long orc_tree_num_updates(const orc_tree *t);
/* Copy the partial of directed branch node->nbr (subtree at nbr seen from node)
 * and its scale counts, computing it if needed. Returns 0, -1 if nbr is a leaf. */
int orc_tree_get_partial(orc_tree *t, int node, int nbr, double *partial, uint8_t *scale);

/* Derivative sums (df, ddf of lnL, not negated) on branch node1-node2 at length len;
 * sets that branch's length and rebuilds theta. Returns 0 or -1 if not a branch. */
int orc_tree_derv(orc_tree *t, int node1, int node2, double len, double *df, double *ddf);
/* lnL on the branch node-dad (computeLikelihoodBranch with dad_branch = dad->node). */
/* computeLikelihoodBranch(dad->node, dad); pattern_lh (nptn) may be NULL */
double orc_tree_lnl_branch(orc_tree *t, int node, int dad, double *pattern_lh);

#ifdef __cplusplus
}
#endif
#endif
