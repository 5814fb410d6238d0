/*
 * CPU FP64 oracle -- see phylo_oracle.h. TEST INFRASTRUCTURE ONLY.
 *
 * Pinned to the reference: tests/test_ref_kernels.py compiles IQ-TREE 2's own
 * kernel templates (tree/phylokernelnew.h, one-lane Vec1d kernels) into
 * oracle/_ref/ and checks that this file reproduces them BIT FOR BIT (every
 * partial and scale count, branch lnL, pattern lnL, derivatives), NORM and
 * SAFE, on seeded fixtures, on a tree that underflows 2^-256 and on the
 * reference's own test alignments; tests/golden/ref_*.npz keep the
 * reference's outputs for machines without a reference checkout.
 *
 * Function-by-function restatement of IQ-TREE 2 (paths relative to the
 * iqtree2 source root):
 *   orc_partial_info        tree/phylokernelnew.h:895-1110  (computePartialInfo)
 *   orc_compute_partials    tree/phylokernelnew.h:1289-2039 (computePartialLikelihoodGenericSIMD)
 *   orc_compute_theta       tree/phylokernelnew.h:2048-2231 (computeLikelihoodBufferGenericSIMD)
 *   orc_derv                tree/phylokernelnew.h:2233-2633 (computeLikelihoodDervGenericSIMD)
 *   orc_branch_lnl          tree/phylokernelnew.h:2641-3223 (computeLikelihoodBranchGenericSIMD)
 *   orc_lnl_from_buffer     tree/phylokernelnew.h:3232-3428 (computeLikelihoodFromBufferGenericSIMD)
 *   traversal               tree/phylotree.cpp:5918-6028, tree/phylokernelnew.h:1145-1200
 *   minimize_newton         utils/optimization.cpp:422-499
 *   optimize_one_branch     tree/phylotree.cpp:2594-2644, computeFuncDerv :2529-2536
 *   optimize_all_branches   tree/phylotree.cpp:2698-2774, computeBestTraversal :2689
 *   farthest leaf, preorder tree/mtree.cpp:3040-3082
 *   clear_reverse           tree/phylonode.cpp:22-33
 * The summation helpers restate the reference's vector helpers as its
 * one-lane build compiles them (JAMES_VERSION dotProductVec :83-126,
 * dotProductDualVec :214-314, productVecMat :449-567, dotProduct3Vec
 * :737-793, dotProductTriple :666-725, sumVec :44-70), with the one-lane
 * mul_add as a separately rounded multiply and add; the file is compiled with
 * -ffp-contract=off. Sums over patterns split across OpenMP threads differ
 * from the reference's packet split by rounding only; with one thread they
 * are the reference's.
 */
#include "phylo_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* summation helpers: the reference's vector helpers on one lane        */
/* ------------------------------------------------------------------ */

/* The one-lane vector class of the reference (vectorclass/vectorf64.h:
 * 339-351) multiplies and adds with two roundings; this file is compiled with
 * -ffp-contract=off so the compiler fuses nothing either. */
static inline double mul_add(double a, double b, double c) { return a * b + c; }
/* the one-lane max (std::max order: the second argument only if larger) */
static inline double fmax_ref(double a, double b) { return a < b ? b : a; }
#define ORC_MAX_BLOCK (64 * 16)
static inline double nmul_add(double a, double b, double c) { return c - a * b; }

/* dotProductVec as compiled (JAMES_VERSION, tree/phylokernelnew.h:83-126):
 * four accumulators over A[0..N-cruft), the N%4 tail added into the first
 * accumulators in turn, then (X+v1)+(v2+v3); N == 4 and N < 4 have their own
 * forms. */
static double dot_vec(const double *A, const double *B, int N) {
    if (N == 4) return (A[0] * B[0] + A[1] * B[1]) + (A[2] * B[2] + A[3] * B[3]);
    const int cruft = N & 3;
    if (N == cruft) {
        double X = 0.0;
        for (int i = 0; i < cruft; i++) X = mul_add(A[i], B[i], X);
        return X;
    }
    double X = A[0] * B[0], v1 = A[1] * B[1], v2 = A[2] * B[2], v3 = A[3] * B[3];
    int i = 4;
    for (; i < N - cruft; i += 4) {
        X = mul_add(A[i], B[i], X);
        v1 = mul_add(A[i + 1], B[i + 1], v1);
        v2 = mul_add(A[i + 2], B[i + 2], v2);
        v3 = mul_add(A[i + 3], B[i + 3], v3);
    }
    if (cruft > 0) {
        X = mul_add(A[i], B[i], X);
        if (cruft > 1) {
            v1 = mul_add(A[i + 1], B[i + 1], v1);
            if (cruft > 2) v2 = mul_add(A[i + 2], B[i + 2], v2);
        }
    }
    return (X + v1) + (v2 + v3);
}

/* X = (A.B) * (C.D), dotProductDualVec (tree/phylokernelnew.h:214-314). The
 * second factor of the N%4 = 0 and 1 forms is summed ((CD0+CD1)+CD2)+CD3. */
static double dot_dual(const double *A, const double *B, const double *C, const double *D, int N) {
    switch (N) {
    case 1: return (A[0] * B[0]) * (C[0] * D[0]);
    case 2: return mul_add(A[1], B[1], A[0] * B[0]) * mul_add(C[1], D[1], C[0] * D[0]);
    case 3:
        return mul_add(A[2], B[2], mul_add(A[1], B[1], A[0] * B[0])) *
               mul_add(C[2], D[2], mul_add(C[1], D[1], C[0] * D[0]));
    case 4:
        return (mul_add(A[1], B[1], A[0] * B[0]) + mul_add(A[3], B[3], A[2] * B[2])) *
               (mul_add(C[1], D[1], C[0] * D[0]) + mul_add(C[3], D[3], C[2] * D[2]));
    default: break;
    }
    double AB[4], CD[4];
    int i, j;
    switch (N % 4) {
    case 0:
        for (j = 0; j < 4; j++) { AB[j] = A[j] * B[j]; CD[j] = C[j] * D[j]; }
        for (i = 4; i < N; i += 4)
            for (j = 0; j < 4; j++) {
                AB[j] = mul_add(A[i + j], B[i + j], AB[j]);
                CD[j] = mul_add(C[i + j], D[i + j], CD[j]);
            }
        return ((AB[0] + AB[1]) + (AB[2] + AB[3])) * (((CD[0] + CD[1]) + CD[2]) + CD[3]);
    case 1:
        for (j = 0; j < 4; j++) { AB[j] = A[j] * B[j]; CD[j] = C[j] * D[j]; }
        for (i = 4; i < N - 1; i += 4)
            for (j = 0; j < 4; j++) {
                AB[j] = mul_add(A[i + j], B[i + j], AB[j]);
                CD[j] = mul_add(C[i + j], D[i + j], CD[j]);
            }
        return mul_add(A[N - 1], B[N - 1], (AB[0] + AB[1]) + (AB[2] + AB[3])) *
               mul_add(C[N - 1], D[N - 1], ((CD[0] + CD[1]) + CD[2]) + CD[3]);
    case 2:
        for (j = 0; j < 2; j++) { AB[j] = A[j] * B[j]; CD[j] = C[j] * D[j]; }
        for (i = 2; i < N; i += 2)
            for (j = 0; j < 2; j++) {
                AB[j] = mul_add(A[i + j], B[i + j], AB[j]);
                CD[j] = mul_add(C[i + j], D[i + j], CD[j]);
            }
        return (AB[0] + AB[1]) * (CD[0] + CD[1]);
    default:
        for (j = 0; j < 2; j++) { AB[j] = A[j] * B[j]; CD[j] = C[j] * D[j]; }
        for (i = 2; i < N - 1; i += 2)
            for (j = 0; j < 2; j++) {
                AB[j] = mul_add(A[i + j], B[i + j], AB[j]);
                CD[j] = mul_add(C[i + j], D[i + j], CD[j]);
            }
        return mul_add(A[N - 1], B[N - 1], AB[0] + AB[1]) * mul_add(C[N - 1], D[N - 1], CD[0] + CD[1]);
    }
}

/* One row of productVecMat (tree/phylokernelnew.h:449-567): sum_j A[j]*M[j]
 * with the reference's per-N unrolling. */
static double vec_mat_row(const double *A, const double *M, int N) {
    switch (N) {
    case 1: return A[0] * M[0];
    case 2: return mul_add(A[1], M[1], A[0] * M[0]);
    case 3: return mul_add(A[2], M[2], mul_add(A[1], M[1], A[0] * M[0]));
    case 4: return mul_add(A[1], M[1], A[0] * M[0]) + mul_add(A[3], M[3], A[2] * M[2]);
    default: break;
    }
    double V[4];
    int x, j;
    switch (N % 4) {
    case 0:
        for (j = 0; j < 4; j++) V[j] = A[j] * M[j];
        for (x = 4; x < N; x += 4)
            for (j = 0; j < 4; j++) V[j] = mul_add(A[x + j], M[x + j], V[j]);
        return (V[0] + V[1]) + (V[2] + V[3]);
    case 1:
        for (j = 0; j < 4; j++) V[j] = A[j] * M[j];
        for (x = 4; x < N - 1; x += 4)
            for (j = 0; j < 4; j++) V[j] = mul_add(A[x + j], M[x + j], V[j]);
        return mul_add(A[N - 1], M[N - 1], (V[0] + V[1]) + (V[2] + V[3]));
    case 2:
        for (j = 0; j < 2; j++) V[j] = A[j] * M[j];
        for (x = 2; x < N; x += 2)
            for (j = 0; j < 2; j++) V[j] = mul_add(A[x + j], M[x + j], V[j]);
        return V[0] + V[1];
    default:
        for (j = 0; j < 2; j++) V[j] = A[j] * M[j];
        for (x = 2; x < N - 1; x += 2)
            for (j = 0; j < 2; j++) V[j] = mul_add(A[x + j], M[x + j], V[j]);
        return mul_add(A[N - 1], M[N - 1], V[0] + V[1]);
    }
}

/* X[i] = sum_j A[j] * M[i*N+j]; returns the updated running max |X|
 * (productVecMat with Xmax, tree/phylokernelnew.h:449-567). */
static double prod_vec_mat(const double *A, const double *M, double *X, int N, double xmax) {
    for (int i = 0; i < N; i++) {
        X[i] = vec_mat_row(A, M + (size_t)i * N, N);
        double a = fabs(X[i]);
        if (a > xmax) xmax = a;
    }
    return xmax;
}

/* X = sum A[i]*B[i]*C[i], dotProduct3Vec (tree/phylokernelnew.h:737-793):
 * no special form for N <= 4. */
static double dot3(const double *A, const double *B, const double *C, int N) {
    double V[4];
    int i, j;
    switch (N % 4) {
    case 0:
        for (j = 0; j < 4; j++) V[j] = A[j] * B[j] * C[j];
        for (i = 4; i < N; i += 4)
            for (j = 0; j < 4; j++) V[j] = mul_add(A[i + j] * B[i + j], C[i + j], V[j]);
        return (V[0] + V[1]) + (V[2] + V[3]);
    case 1:
        for (j = 0; j < 4; j++) V[j] = A[j] * B[j] * C[j];
        for (i = 4; i < N - 1; i += 4)
            for (j = 0; j < 4; j++) V[j] = mul_add(A[i + j] * B[i + j], C[i + j], V[j]);
        return mul_add(A[N - 1] * B[N - 1], C[N - 1], (V[0] + V[1]) + (V[2] + V[3]));
    case 2:
        for (j = 0; j < 2; j++) V[j] = A[j] * B[j] * C[j];
        for (i = 2; i < N; i += 2)
            for (j = 0; j < 2; j++) V[j] = mul_add(A[i + j] * B[i + j], C[i + j], V[j]);
        return V[0] + V[1];
    default:
        for (j = 0; j < 2; j++) V[j] = A[j] * B[j] * C[j];
        for (i = 2; i < N - 1; i += 2)
            for (j = 0; j < 2; j++) V[j] = mul_add(A[i + j] * B[i + j], C[i + j], V[j]);
        return mul_add(A[N - 1] * B[N - 1], C[N - 1], V[0] + V[1]);
    }
}

/* (X,Y,Z) = (A.D, B.D, C.D) over N = block entries, dotProductTriple
 * (tree/phylokernelnew.h:666-725) with ADD = false; the parity of
 * `nstates` picks the two-accumulator form, as in the reference. */
static void dot_triple(const double *A, const double *B, const double *C, const double *D,
                       int N, int nstates, double *X, double *Y, double *Z) {
    double AD[2], BD[2], CD[2];
    int i, j;
    for (j = 0; j < 2; j++) {
        AD[j] = A[j] * D[j];
        BD[j] = B[j] * D[j];
        CD[j] = C[j] * D[j];
    }
    if ((nstates & 1) == 0) {
        for (i = 2; i < N; i += 2)
            for (j = 0; j < 2; j++) {
                AD[j] = mul_add(A[i + j], D[i + j], AD[j]);
                BD[j] = mul_add(B[i + j], D[i + j], BD[j]);
                CD[j] = mul_add(C[i + j], D[i + j], CD[j]);
            }
        *X = AD[0] + AD[1];
        *Y = BD[0] + BD[1];
        *Z = CD[0] + CD[1];
    } else {
        for (i = 2; i < N - 1; i += 2)
            for (j = 0; j < 2; j++) {
                AD[j] = mul_add(A[i + j], D[i + j], AD[j]);
                BD[j] = mul_add(B[i + j], D[i + j], BD[j]);
                CD[j] = mul_add(C[i + j], D[i + j], CD[j]);
            }
        *X = mul_add(A[N - 1], D[N - 1], AD[0] + AD[1]);
        *Y = mul_add(B[N - 1], D[N - 1], BD[0] + BD[1]);
        *Z = mul_add(C[N - 1], D[N - 1], CD[0] + CD[1]);
    }
}

static double sum_vec(const double *A, int N) {
    double X = 0.0;
    int cruft = N & 3, k = 0;
    if (cruft < N) {
        double V[4] = {0, 0, 0, 0};
        for (; k < N - cruft; k += 4) {
            V[0] += A[k];
            V[1] += A[k + 1];
            V[2] += A[k + 2];
            V[3] += A[k + 3];
        }
        V[0] += V[2];
        V[1] += V[3];
        V[0] += V[1];
        X += V[0];
    }
    for (; k < N; k++) X += A[k];
    return X;
}

static int num_threads(int want) {
#ifdef _OPENMP
    return want > 0 ? want : omp_get_max_threads();
#else
    (void)want;
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* per-child precompute: echild and tip lookup table                    */
/* ------------------------------------------------------------------ */

/* echild[c][x][i] = U[x][i] * exp(eval[i]*rate_c*len) */
static void orc_echild(const orc_model *m, double len, double *echild) {
    int n = m->nstates;
    for (int c = 0; c < m->ncat; c++) {
        double lc = m->rates[c] * len;
        for (int x = 0; x < n; x++)
            for (int i = 0; i < n; i++)
                echild[((size_t)c * n + x) * n + i] = m->evec[x * n + i] * exp(m->eval[i] * lc);
    }
}

/* A[0]*B[0] + A[1]*B[1] + ..., left to right (computePartialInfo's one-lane
 * leaf-table sum, tree/phylokernelnew.h:1037-1046) */
static double seq_dot(const double *A, const double *B, int N) {
    double v = A[0] * B[0];
    for (int i = 1; i < N; i++) v = mul_add(A[i], B[i], v);
    return v;
}

/* leaf[s][c][x] = sum_i echild[c][x][i]*tip_lh[s][i]; unknown state row = 1.0 */
static void orc_leaf_table(const orc_model *m, const double *echild, double *leaf) {
    int n = m->nstates, B = n * m->ncat, S = m->state_unknown;
    for (int s = 0; s < S; s++)
        for (int c = 0; c < m->ncat; c++)
            for (int x = 0; x < n; x++)
                leaf[(size_t)s * B + c * n + x] = seq_dot(echild + ((size_t)c * n + x) * n, m->tip_lh + (size_t)s * n, n);
    for (int k = 0; k < B; k++) leaf[(size_t)S * B + k] = 1.0;
}

static inline int tip_state(const orc_model *m, int taxon, int ptn) {
    return m->tip_states[(size_t)taxon * m->nptn + ptn];
}

/* ------------------------------------------------------------------ */
/* partial likelihood update                                            */
/* ------------------------------------------------------------------ */

static void orc_compute_one(const orc_model *m, double *partials, uint8_t *scale, const orc_op *op, int nth) {
    const int n = m->nstates, C = m->ncat, B = n * C, S = m->state_unknown;
    const int safe = m->safe;
    const size_t pstride = (size_t)m->nptn * B;
    const size_t sstride = (size_t)m->nptn * (safe ? C : 1);
    int lref = op->child[0], rref = op->child[1];
    double llen = op->len[0], rlen = op->len[1];
    if (lref >= 0 && rref < 0) { /* left internal, right tip: swap so the tip is left */
        int t = lref; lref = rref; rref = t;
        double tl = llen; llen = rlen; rlen = tl;
    }
    double *eleft = malloc(sizeof(double) * (size_t)C * n * n);
    double *eright = malloc(sizeof(double) * (size_t)C * n * n);
    orc_echild(m, llen, eleft);
    orc_echild(m, rlen, eright);
    double *leafL = NULL, *leafR = NULL;
    if (lref < 0) {
        leafL = malloc(sizeof(double) * (size_t)(S + 1) * B);
        orc_leaf_table(m, eleft, leafL);
    }
    if (rref < 0) {
        leafR = malloc(sizeof(double) * (size_t)(S + 1) * B);
        orc_leaf_table(m, eright, leafR);
    }
    double *dad = partials + (size_t)op->dad_slot * pstride;
    uint8_t *sdad = scale + (size_t)op->dad_slot * sstride;
    const double *R = rref >= 0 ? partials + (size_t)rref * pstride : NULL;
    const double *L = lref >= 0 ? partials + (size_t)lref * pstride : NULL;
    const uint8_t *sR = rref >= 0 ? scale + (size_t)rref * sstride : NULL;
    const uint8_t *sL = lref >= 0 ? scale + (size_t)lref * sstride : NULL;
    const int nptn = m->nptn;

#pragma omp parallel for schedule(static) num_threads(nth)
    for (int ptn = 0; ptn < nptn; ptn++) {
        double tmp[64];
        double *pd = dad + (size_t)ptn * B;
        if (lref < 0 && rref < 0) {
            /* tip-tip: no scaling (tree/phylokernelnew.h:1632-1747) */
            const double *tl = leafL + (size_t)tip_state(m, -1 - lref, ptn) * B;
            const double *tr = leafR + (size_t)tip_state(m, -1 - rref, ptn) * B;
            if (safe) memset(sdad + (size_t)ptn * C, 0, C);
            else sdad[ptn] = 0;
            for (int c = 0; c < C; c++) {
                for (int x = 0; x < n; x++) tmp[x] = tl[c * n + x] * tr[c * n + x];
                prod_vec_mat(tmp, m->inv_evec, pd + c * n, n, 0.0);
            }
        } else if (lref < 0) {
            /* tip-internal (tree/phylokernelnew.h:1748-1906) */
            const double *tl = leafL + (size_t)tip_state(m, -1 - lref, ptn) * B;
            const double *pr = R + (size_t)ptn * B;
            if (safe) memcpy(sdad + (size_t)ptn * C, sR + (size_t)ptn * C, C);
            else sdad[ptn] = sR[ptn];
            double lh_max = 0.0;
            for (int c = 0; c < C; c++) {
                if (safe) lh_max = 0.0;
                for (int x = 0; x < n; x++)
                    tmp[x] = tl[c * n + x] * dot_vec(eright + ((size_t)c * n + x) * n, pr + c * n, n);
                lh_max = prod_vec_mat(tmp, m->inv_evec, pd + c * n, n, lh_max);
                if (safe && lh_max < ORC_SCALING_THRESHOLD && m->ptn_invar[ptn] == 0.0) {
                    for (int i = 0; i < n; i++) pd[c * n + i] = ldexp(pd[c * n + i], ORC_SCALING_THRESHOLD_EXP);
                    sdad[(size_t)ptn * C + c] += 1;
                }
            }
            if (!safe && lh_max < ORC_SCALING_THRESHOLD && m->ptn_invar[ptn] == 0.0) {
                for (int i = 0; i < B; i++) pd[i] = ldexp(pd[i], ORC_SCALING_THRESHOLD_EXP);
                sdad[ptn] += 1;
            }
        } else {
            /* internal-internal (tree/phylokernelnew.h:1907-2032) */
            const double *pl = L + (size_t)ptn * B;
            const double *pr = R + (size_t)ptn * B;
            double lh_max = 0.0;
            if (!safe) sdad[ptn] = (uint8_t)(sL[ptn] + sR[ptn]);
            for (int c = 0; c < C; c++) {
                if (safe) {
                    lh_max = 0.0;
                    sdad[(size_t)ptn * C + c] = (uint8_t)(sL[(size_t)ptn * C + c] + sR[(size_t)ptn * C + c]);
                }
                for (int x = 0; x < n; x++)
                    tmp[x] = dot_dual(eleft + ((size_t)c * n + x) * n, pl + c * n,
                                      eright + ((size_t)c * n + x) * n, pr + c * n, n);
                lh_max = prod_vec_mat(tmp, m->inv_evec, pd + c * n, n, lh_max);
                if (safe && lh_max < ORC_SCALING_THRESHOLD && m->ptn_invar[ptn] == 0.0) {
                    for (int i = 0; i < n; i++) pd[c * n + i] = ldexp(pd[c * n + i], ORC_SCALING_THRESHOLD_EXP);
                    sdad[(size_t)ptn * C + c] += 1;
                }
            }
            if (!safe && lh_max < ORC_SCALING_THRESHOLD && m->ptn_invar[ptn] == 0.0) {
                for (int i = 0; i < B; i++) pd[i] = ldexp(pd[i], ORC_SCALING_THRESHOLD_EXP);
                sdad[ptn] += 1;
            }
        }
    }
    free(eleft);
    free(eright);
    free(leafL);
    free(leafR);
}

/* Multifurcating node, nchild > 2 (tree/phylokernelnew.h:1407-1631, the
 * non-site-model branch): the running product of the children's contributions
 * in neighbour order, each child's internal partial entering as the left-to-
 * right sum echild[c][x][.].child[c][.] and a tip child as its leaf-table row;
 * the 2^-256 check (per category in SAFE, whole block in NORM) after every
 * child on the product; one U^-1 transform at the end with no check after. */
static void orc_compute_multi(const orc_model *m, double *partials, uint8_t *scale, const orc_op *op, int nth) {
    const int n = m->nstates, C = m->ncat, B = n * C, S = m->state_unknown, k = op->nchild;
    const int safe = m->safe;
    const size_t pstride = (size_t)m->nptn * B;
    const size_t sstride = (size_t)m->nptn * (safe ? C : 1);
    double *ech[ORC_MAX_DEG - 1], *leaf[ORC_MAX_DEG - 1];
    for (int ch = 0; ch < k; ch++) {
        ech[ch] = malloc(sizeof(double) * (size_t)C * n * n);
        orc_echild(m, op->len[ch], ech[ch]);
        leaf[ch] = NULL;
        if (op->child[ch] < 0) {
            leaf[ch] = malloc(sizeof(double) * (size_t)(S + 1) * B);
            orc_leaf_table(m, ech[ch], leaf[ch]);
        }
    }
    double *dad = partials + (size_t)op->dad_slot * pstride;
    uint8_t *sdad = scale + (size_t)op->dad_slot * sstride;
    const int nptn = m->nptn;

#pragma omp parallel for schedule(static) num_threads(nth)
    for (int ptn = 0; ptn < nptn; ptn++) {
        double all[ORC_MAX_BLOCK];
        uint8_t *sd = safe ? sdad + (size_t)ptn * C : sdad + ptn;
        for (int i = 0; i < B; i++) all[i] = 1.0;
        memset(sd, 0, safe ? C : 1);
        for (int ch = 0; ch < k; ch++) {
            const int ref = op->child[ch];
            if (ref < 0) {
                const double *tl = leaf[ch] + (size_t)tip_state(m, -1 - ref, ptn) * B;
                for (int i = 0; i < B; i++) all[i] *= tl[i];
            } else {
                const double *pc = partials + (size_t)ref * pstride + (size_t)ptn * B;
                const uint8_t *sc = scale + (size_t)ref * sstride;
                if (!safe) sd[0] = (uint8_t)(sd[0] + sc[ptn]);
                for (int c = 0; c < C; c++) {
                    if (safe) sd[c] = (uint8_t)(sd[c] + sc[(size_t)ptn * C + c]);
                    for (int x = 0; x < n; x++) {
                        const double *e = ech[ch] + ((size_t)c * n + x) * n;
                        all[c * n + x] *= seq_dot(e, pc + c * n, n);
                    }
                }
            }
            if (m->ptn_invar[ptn] != 0.0) continue;
            if (safe) {
                for (int c = 0; c < C; c++) {
                    double lh_max = 0.0;
                    for (int x = 0; x < n; x++) lh_max = fmax_ref(lh_max, fabs(all[c * n + x]));
                    if (lh_max < ORC_SCALING_THRESHOLD) {
                        for (int x = 0; x < n; x++) all[c * n + x] = ldexp(all[c * n + x], ORC_SCALING_THRESHOLD_EXP);
                        sd[c] += 1;
                    }
                }
            } else {
                double lh_max = 0.0;
                for (int i = 0; i < B; i++) lh_max = fmax_ref(lh_max, fabs(all[i]));
                if (lh_max < ORC_SCALING_THRESHOLD) {
                    for (int i = 0; i < B; i++) all[i] = ldexp(all[i], ORC_SCALING_THRESHOLD_EXP);
                    sd[0] += 1;
                }
            }
        }
        double *pd = dad + (size_t)ptn * B;
        for (int c = 0; c < C; c++) prod_vec_mat(all + c * n, m->inv_evec, pd + c * n, n, 0.0);
    }
    for (int ch = 0; ch < k; ch++) {
        free(ech[ch]);
        free(leaf[ch]);
    }
}

void orc_compute_partials(const orc_model *m, double *partials, uint8_t *scale,
                          const orc_op *ops, int nops, int nthreads) {
    int nth = num_threads(nthreads);
    for (int k = 0; k < nops; k++) {
        if (ops[k].nchild > 2) orc_compute_multi(m, partials, scale, &ops[k], nth);
        else orc_compute_one(m, partials, scale, &ops[k], nth);
    }
}

/* ------------------------------------------------------------------ */
/* branch likelihood                                                    */
/* ------------------------------------------------------------------ */

static void make_val(const orc_model *m, double len, double *val) {
    int n = m->nstates;
    for (int c = 0; c < m->ncat; c++) {
        double l = m->rates[c] * len, p = m->props[c];
        for (int i = 0; i < n; i++) val[c * n + i] = exp(m->eval[i] * l) * p;
    }
}

/* Lewis correction of a tree lnL (tree/phylokernelnew.h:3198-3222): the
 * observed patterns' lnL drop by log(1 - P_const), the total by nsite times
 * that. Returns NAN when P_const is outside [0, 1) (the reference asserts). */
double orc_asc_lewis_lnl(const orc_model *m, double tree_lh, double prob_const, double *plh) {
    if (!(prob_const < 1.0 && prob_const >= 0.0)) return NAN;
    const double lc = log(1.0 - prob_const);
    if (plh)
        for (int ptn = 0; ptn < m->nptn - m->asc_n; ptn++) plh[ptn] -= lc;
    return tree_lh - m->asc_nsite * lc;
}

double orc_branch_lnl(const orc_model *m, const double *partials, const uint8_t *scale,
                      int a, int b, double len, double *pattern_lh, int nthreads) {
    const int n = m->nstates, C = m->ncat, B = n * C, S = m->state_unknown, safe = m->safe;
    const size_t pstride = (size_t)m->nptn * B;
    const size_t sstride = (size_t)m->nptn * (safe ? C : 1);
    int nth = num_threads(nthreads);
    if (a < 0) { int t = a; a = b; b = t; } /* node must be internal: dad becomes the leaf */
    double *val = malloc(sizeof(double) * B);
    make_val(m, len, val);
    double *lh_node_tab = NULL;
    if (b < 0) {
        lh_node_tab = malloc(sizeof(double) * (size_t)(S + 1) * B);
        for (int s = 0; s <= S; s++)
            for (int c = 0; c < C; c++)
                for (int i = 0; i < n; i++)
                    lh_node_tab[(size_t)s * B + c * n + i] = val[c * n + i] * m->tip_lh[(size_t)s * n + i];
    }
    const double *pa = partials + (size_t)a * pstride;
    const uint8_t *sa = scale + (size_t)a * sstride;
    const double *pb = b >= 0 ? partials + (size_t)b * pstride : NULL;
    const uint8_t *sb = b >= 0 ? scale + (size_t)b * sstride : NULL;
    double *plh = pattern_lh ? pattern_lh : malloc(sizeof(double) * m->nptn);
    const int nptn = m->nptn, orig = m->nptn - m->asc_n;
    double *thread_sum = calloc(nth, sizeof(double)), *thread_const = calloc(nth, sizeof(double));

#pragma omp parallel num_threads(nth)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double acc = 0.0, pconst = 0.0;
#pragma omp for schedule(static)
        for (int ptn = 0; ptn < nptn; ptn++) {
            double lh_cat[16], lh = 0.0, min_scale = 0.0;
            const double *dadp = pa + (size_t)ptn * B;
            if (b < 0) {
                const double *lhn = lh_node_tab + (size_t)tip_state(m, -1 - b, ptn) * B;
                for (int c = 0; c < C; c++) {
                    lh_cat[c] = dot_vec(lhn + c * n, dadp + c * n, n);
                    if (!safe) lh += lh_cat[c];
                }
                if (safe) {
                    const uint8_t *sd = sa + (size_t)ptn * C;
                    uint8_t mn = sd[0];
                    for (int c = 1; c < C; c++) if (sd[c] < mn) mn = sd[c];
                    min_scale = mn;
                    for (int c = 0; c < C; c++) {
                        if (sd[c] == mn + 1) lh_cat[c] *= ORC_SCALING_THRESHOLD;
                        else if (sd[c] > mn + 1) lh_cat[c] = 0.0;
                    }
                    lh = sum_vec(lh_cat, C);
                } else {
                    min_scale = sa[ptn];
                }
            } else {
                const double *nodep = pb + (size_t)ptn * B;
                for (int c = 0; c < C; c++) {
                    lh_cat[c] = dot3(val + c * n, nodep + c * n, dadp + c * n, n);
                    if (!safe) lh += lh_cat[c];
                }
                if (safe) {
                    uint8_t sum[16], mn;
                    mn = sum[0] = (uint8_t)(sa[(size_t)ptn * C] + sb[(size_t)ptn * C]);
                    for (int c = 1; c < C; c++) {
                        sum[c] = (uint8_t)(sa[(size_t)ptn * C + c] + sb[(size_t)ptn * C + c]);
                        if (sum[c] < mn) mn = sum[c];
                    }
                    min_scale = mn;
                    for (int c = 0; c < C; c++) {
                        if (sum[c] == mn + 1) lh_cat[c] *= ORC_SCALING_THRESHOLD;
                        else if (sum[c] > mn + 1) lh_cat[c] = 0.0;
                    }
                    lh = sum_vec(lh_cat, C);
                } else {
                    min_scale = (double)(sa[ptn] + sb[ptn]);
                }
            }
            double sc = min_scale * ORC_LOG_SCALING_THRESHOLD;
            lh = fabs(lh) + m->ptn_invar[ptn];
            if (ptn >= orig) {  /* unobserved constant pattern: its likelihood, once unscaled */
                if (min_scale != 0.0) lh *= ORC_SCALING_THRESHOLD;
                pconst += lh;
                plh[ptn] = 0.0;
                continue;
            }
            lh = log(lh) + sc;
            plh[ptn] = lh;
            acc = mul_add(lh, m->ptn_freq[ptn], acc);
        }
        thread_sum[tid] = acc;
        thread_const[tid] = pconst;
    }
    double tree_lh = 0.0, prob_const = 0.0;
    for (int t = 0; t < nth; t++) {
        tree_lh += thread_sum[t];
        prob_const += thread_const[t];
    }
    if (!isfinite(tree_lh)) {
        /* arbitrarily fix underflown sites (tree/phylokernelnew.h:3119-3132) */
        tree_lh = 0.0;
        for (int ptn = 0; ptn < orig; ptn++) {
            if (!isfinite(plh[ptn])) plh[ptn] = ORC_LOG_SCALING_THRESHOLD * 4;
            tree_lh += plh[ptn] * m->ptn_freq[ptn];
        }
    }
    if (m->asc_n > 0) tree_lh = orc_asc_lewis_lnl(m, tree_lh, prob_const, plh);
    free(thread_sum);
    free(thread_const);
    free(val);
    free(lh_node_tab);
    if (!pattern_lh) free(plh);
    return tree_lh;
}

/* ------------------------------------------------------------------ */
/* theta buffer, derivatives, lnL from buffer                           */
/* ------------------------------------------------------------------ */

void orc_compute_theta(const orc_model *m, const double *partials, const uint8_t *scale,
                       int a, int b, double *theta, double *buffer_scale, int nthreads) {
    const int n = m->nstates, C = m->ncat, B = n * C, safe = m->safe;
    const size_t pstride = (size_t)m->nptn * B;
    const size_t sstride = (size_t)m->nptn * (safe ? C : 1);
    int nth = num_threads(nthreads);
    if (a < 0) { int t = a; a = b; b = t; }
    const double *pa = partials + (size_t)a * pstride;
    const uint8_t *sa = scale + (size_t)a * sstride;
    const double *pb = b >= 0 ? partials + (size_t)b * pstride : NULL;
    const uint8_t *sb = b >= 0 ? scale + (size_t)b * sstride : NULL;
    const int nptn = m->nptn;
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int ptn = 0; ptn < nptn; ptn++) {
        double *th = theta + (size_t)ptn * B;
        const double *dadp = pa + (size_t)ptn * B;
        if (b < 0) {
            const double *tip = m->tip_lh + (size_t)tip_state(m, -1 - b, ptn) * n;
            for (int c = 0; c < C; c++)
                for (int i = 0; i < n; i++) th[c * n + i] = tip[i] * dadp[c * n + i];
            if (safe) {
                const uint8_t *sd = sa + (size_t)ptn * C;
                uint8_t mn = sd[0];
                for (int c = 1; c < C; c++) if (sd[c] < mn) mn = sd[c];
                buffer_scale[ptn] = mn;
                for (int c = 0; c < C; c++) {
                    if (sd[c] == mn + 1)
                        for (int x = 0; x < n; x++) th[c * n + x] *= ORC_SCALING_THRESHOLD;
                    else if (sd[c] > mn + 1)
                        for (int x = 0; x < n; x++) th[c * n + x] = 0.0;
                }
            } else {
                buffer_scale[ptn] = sa[ptn];
            }
        } else {
            const double *nodep = pb + (size_t)ptn * B;
            for (int k = 0; k < B; k++) th[k] = nodep[k] * dadp[k];
            if (safe) {
                uint8_t sum[16], mn;
                mn = sum[0] = (uint8_t)(sa[(size_t)ptn * C] + sb[(size_t)ptn * C]);
                for (int c = 1; c < C; c++) {
                    sum[c] = (uint8_t)(sa[(size_t)ptn * C + c] + sb[(size_t)ptn * C + c]);
                    if (sum[c] < mn) mn = sum[c];
                }
                buffer_scale[ptn] = mn;
                for (int c = 0; c < C; c++) {
                    if (sum[c] == mn + 1)
                        for (int x = 0; x < n; x++) th[c * n + x] *= ORC_SCALING_THRESHOLD;
                    else if (sum[c] > mn + 1)
                        for (int x = 0; x < n; x++) th[c * n + x] = 0.0;
                }
            } else {
                buffer_scale[ptn] = (double)(sa[ptn] + sb[ptn]);
            }
        }
        buffer_scale[ptn] *= ORC_LOG_SCALING_THRESHOLD;
    }
}

void orc_derv(const orc_model *m, const double *theta, const double *buffer_scale, double len, double *df,
              double *ddf, int nthreads) {
    const int n = m->nstates, C = m->ncat, B = n * C;
    int nth = num_threads(nthreads);
    double *val0 = malloc(sizeof(double) * B), *val1 = malloc(sizeof(double) * B), *val2 = malloc(sizeof(double) * B);
    for (int c = 0; c < C; c++) {
        double prop = m->props[c], rate = m->rates[c];
        for (int i = 0; i < n; i++) {
            double cof = m->eval[i] * rate;
            double v = exp(cof * len) * prop;
            double v1 = cof * v;
            val0[c * n + i] = v;
            val1[c * n + i] = v1;
            val2[c * n + i] = cof * v1;
        }
    }
    const int nptn = m->nptn, orig = m->nptn - m->asc_n;
    double *tdf = calloc(nth, sizeof(double)), *tddf = calloc(nth, sizeof(double));
    double *tc = calloc(3 * (size_t)nth, sizeof(double));
#pragma omp parallel num_threads(nth)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double my_df = 0.0, my_ddf = 0.0, c_lh = 0.0, c_df = 0.0, c_ddf = 0.0;
#pragma omp for schedule(static)
        for (int ptn = 0; ptn < nptn; ptn++) {
            double lh, d1, d2;
            /* the split follows nstates parity in the reference; following the
             * parity of B itself gives the exact sum */
            dot_triple(val0, val1, val2, theta + (size_t)ptn * B, B, m->ref_triple_tail ? n : B, &lh, &d1, &d2);
            lh = fabs(lh) + m->ptn_invar[ptn];
            if (ptn >= orig) {  /* unobserved constant pattern (tree/phylokernelnew.h:2506-2546) */
                if (buffer_scale[ptn] != 0.0) {
                    lh *= ORC_SCALING_THRESHOLD;
                    d1 *= ORC_SCALING_THRESHOLD;
                    d2 *= ORC_SCALING_THRESHOLD;
                }
                c_lh += lh;
                c_df += d1;
                c_ddf += d2;
                continue;
            }
            lh = 1.0 / lh;
            double df_frac = d1 * lh, ddf_frac = d2 * lh;
            double freq = m->ptn_freq[ptn];
            double tmp1 = df_frac * freq, tmp2 = ddf_frac * freq;
            my_df += tmp1;
            my_ddf += nmul_add(tmp1, df_frac, tmp2);
        }
        tdf[tid] = my_df;
        tddf[tid] = my_ddf;
        tc[3 * tid] = c_lh;
        tc[3 * tid + 1] = c_df;
        tc[3 * tid + 2] = c_ddf;
    }
    double sdf = 0.0, sddf = 0.0, clh = 0.0, cdf = 0.0, cddf = 0.0;
    for (int t = 0; t < nth; t++) {
        sdf += tdf[t];
        sddf += tddf[t];
        clh += tc[3 * t];
        cdf += tc[3 * t + 1];
        cddf += tc[3 * t + 2];
    }
    if (m->asc_n > 0) {  /* Lewis correction (tree/phylokernelnew.h:2620-2628) */
        const double pv = 1.0 - clh, df_frac = cdf / pv, ddf_frac = cddf / pv;
        sdf += m->asc_nsite * df_frac;
        sddf += m->asc_nsite * (ddf_frac + df_frac * df_frac);
    }
    if (!isfinite(sdf)) sdf = sddf = 0.0; /* tree/phylokernelnew.h:2629-2632 */
    *df = sdf;
    *ddf = sddf;
    free(tdf); free(tddf); free(tc); free(val0); free(val1); free(val2);
}

double orc_lnl_from_buffer(const orc_model *m, const double *theta, const double *buffer_scale,
                           double len, double *pattern_lh, int nthreads) {
    const int n = m->nstates, C = m->ncat, B = n * C;
    int nth = num_threads(nthreads);
    double *val0 = malloc(sizeof(double) * B);
    make_val(m, len, val0);
    const int nptn = m->nptn, orig = m->nptn - m->asc_n;
    double *plh = pattern_lh ? pattern_lh : malloc(sizeof(double) * nptn);
    double *tsum = calloc(nth, sizeof(double)), *tconst = calloc(nth, sizeof(double));
#pragma omp parallel num_threads(nth)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double acc = 0.0, pconst = 0.0;
#pragma omp for schedule(static)
        for (int ptn = 0; ptn < nptn; ptn++) {
            double lh = dot_vec(val0, theta + (size_t)ptn * B, B);
            lh = fabs(lh) + m->ptn_invar[ptn];
            if (ptn >= orig) {  /* unobserved constant pattern (tree/phylokernelnew.h:3341-3365) */
                if (buffer_scale[ptn] != 0.0) lh *= ORC_SCALING_THRESHOLD;
                pconst += lh;
                plh[ptn] = 0.0;
                continue;
            }
            lh = log(fabs(lh)) + buffer_scale[ptn];
            plh[ptn] = lh;
            /* the reference adds each pattern's term on its own
             * (tree/phylokernelnew.h:3376-3392) */
            acc += mul_add(lh, m->ptn_freq[ptn], 0.0);
        }
        tsum[tid] = acc;
        tconst[tid] = pconst;
    }
    double tree_lh = 0.0, prob_const = 0.0;
    for (int t = 0; t < nth; t++) {
        tree_lh += tsum[t];
        prob_const += tconst[t];
    }
    if (!isfinite(tree_lh)) {
        tree_lh = 0.0;
        for (int ptn = 0; ptn < orig; ptn++) {
            if (!isfinite(plh[ptn])) plh[ptn] = ORC_LOG_SCALING_THRESHOLD * 4;
            tree_lh += plh[ptn] * m->ptn_freq[ptn];
        }
    }
    if (m->asc_n > 0) tree_lh = orc_asc_lewis_lnl(m, tree_lh, prob_const, plh);
    free(tsum);
    free(tconst);
    free(val0);
    if (!pattern_lh) free(plh);
    return tree_lh;
}

/* ------------------------------------------------------------------ */
/* tree-level drivers                                                   */
/* ------------------------------------------------------------------ */

struct orc_tree {
    orc_model m;
    int ntaxa, nnode, nedge, nth;
    int *deg;          /* [nnode] */
    int (*nbr)[ORC_MAX_DEG];     /* neighbour node */
    int (*edge)[ORC_MAX_DEG];    /* edge id of that neighbour */
    int (*slot)[ORC_MAX_DEG];    /* slot of directed partial node->nbr (nbr internal), else -1 */
    uint8_t (*computed)[ORC_MAX_DEG];
    double *lengths;   /* [nedge] */
    double *partials;
    uint8_t *scale;
    double *theta, *buffer_scale;
    int *height;       /* topological height from the current traversal root */
    orc_op *ops;
    int nops;
    long long nupdates;
    double min_bl, max_bl;
    /* current branch (current_it / current_it_back) */
    int cur_node1, cur_node2;
    int theta_computed;
};

static int nbr_index(const orc_tree *t, int node, int nb) {
    for (int j = 0; j < t->deg[node]; j++)
        if (t->nbr[node][j] == nb) return j;
    return -1;
}

static int is_leaf(const orc_tree *t, int node) { return node < t->ntaxa; }

orc_tree *orc_tree_new(const orc_model *m, const int *edges, int nedge, const double *lengths, int nthreads) {
    orc_tree *t = calloc(1, sizeof(orc_tree));
    t->m = *m;
    t->ntaxa = m->ntaxa;
    t->nedge = nedge;
    t->nnode = 0;
    for (int k = 0; k < 2 * nedge; k++)
        if (edges[k] + 1 > t->nnode) t->nnode = edges[k] + 1;
    t->nth = num_threads(nthreads);
    t->deg = calloc(t->nnode, sizeof(int));
    t->nbr = calloc(t->nnode, sizeof(*t->nbr));
    t->edge = calloc(t->nnode, sizeof(*t->edge));
    t->slot = calloc(t->nnode, sizeof(*t->slot));
    t->computed = calloc(t->nnode, sizeof(*t->computed));
    t->lengths = malloc(sizeof(double) * t->nedge);
    memcpy(t->lengths, lengths, sizeof(double) * t->nedge);
    for (int k = 0; k < t->nedge; k++) {
        int u = edges[2 * k], v = edges[2 * k + 1];
        if (t->deg[u] >= ORC_MAX_DEG || t->deg[v] >= ORC_MAX_DEG) { orc_tree_free(t); return NULL; }
        t->nbr[u][t->deg[u]] = v; t->edge[u][t->deg[u]++] = k;
        t->nbr[v][t->deg[v]] = u; t->edge[v][t->deg[v]++] = k;
    }
    int ns = 0;
    for (int u = 0; u < t->nnode; u++)
        for (int j = 0; j < ORC_MAX_DEG; j++)
            t->slot[u][j] = (j < t->deg[u] && !is_leaf(t, t->nbr[u][j])) ? ns++ : -1;
    const int B = m->nstates * m->ncat;
    t->partials = malloc(sizeof(double) * (size_t)ns * m->nptn * B);
    t->scale = malloc((size_t)ns * m->nptn * (m->safe ? m->ncat : 1));
    t->theta = malloc(sizeof(double) * (size_t)m->nptn * B);
    t->buffer_scale = malloc(sizeof(double) * m->nptn);
    t->height = calloc(t->nnode, sizeof(int));
    t->ops = malloc(sizeof(orc_op) * (size_t)(ns + 1));
    t->min_bl = 1e-6;
    t->max_bl = 10.0;
    t->cur_node1 = t->cur_node2 = -1;
    return t;
}

void orc_tree_free(orc_tree *t) {
    if (!t) return;
    free(t->deg); free(t->nbr); free(t->edge); free(t->slot); free(t->computed);
    free(t->lengths); free(t->partials); free(t->scale); free(t->theta);
    free(t->buffer_scale); free(t->height); free(t->ops);
    free(t);
}

void orc_tree_get_lengths(const orc_tree *t, double *lengths) { memcpy(lengths, t->lengths, sizeof(double) * t->nedge); }
void orc_tree_set_bounds(orc_tree *t, double min_bl, double max_bl) { t->min_bl = min_bl; t->max_bl = max_bl; }
long long orc_tree_num_updates(const orc_tree *t) { return t->nupdates; }

void orc_tree_set_lengths(orc_tree *t, const double *lengths) {
    memcpy(t->lengths, lengths, sizeof(double) * t->nedge);
    memset(t->computed, 0, sizeof(*t->computed) * t->nnode); /* clearAllPartialLH */
    t->theta_computed = 0;
}

/* reference of directed partial dad->node: slot if node internal, tip otherwise */
static int dref(const orc_tree *t, int dad, int node) {
    if (is_leaf(t, node)) return -1 - node;
    return t->slot[dad][nbr_index(t, dad, node)];
}

/* post-order list of stale directed partials (tree/phylotree.cpp:5918-6028) */
static void traverse(orc_tree *t, int dad, int node) {
    int j = nbr_index(t, dad, node);
    if (is_leaf(t, node) || t->computed[dad][j]) return;
    orc_op op;
    int k = 0;
    for (int q = 0; q < t->deg[node]; q++) {
        int ch = t->nbr[node][q];
        if (ch == dad) continue;
        traverse(t, node, ch);
        op.child[k] = dref(t, node, ch);
        op.len[k] = t->lengths[t->edge[node][q]];
        k++;
    }
    op.nchild = k;
    op.dad_slot = t->slot[dad][j];
    t->computed[dad][j] = 1;
    t->ops[t->nops++] = op;
}

static void run_traversal(orc_tree *t, int node, int dad) {
    t->nops = 0;
    traverse(t, dad, node); /* dad_branch: dad -> node */
    traverse(t, node, dad); /* node_branch: node -> dad */
    if (t->nops) {
        orc_compute_partials(&t->m, t->partials, t->scale, t->ops, t->nops, t->nth);
        t->nupdates += (long long)t->nops * t->m.nptn;
    }
}

static double branch_len(const orc_tree *t, int u, int v) { return t->lengths[t->edge[u][nbr_index(t, u, v)]]; }

/* computeLikelihoodBranch(dad_branch = dad->node, dad) */
static double lnl_branch(orc_tree *t, int node, int dad, double *pattern_lh) {
    if (is_leaf(t, node)) { int x = node; node = dad; dad = x; }
    run_traversal(t, node, dad);
    return orc_branch_lnl(&t->m, t->partials, t->scale, dref(t, dad, node), dref(t, node, dad),
                          branch_len(t, node, dad), pattern_lh, t->nth);
}

/* MTree::findFarthestLeaf: sets height[] and returns the deepest leaf */
static int farthest_leaf(orc_tree *t, int node, int dad) {
    if (dad >= 0 && is_leaf(t, node)) { t->height[node] = 0; return node; }
    int res = -1;
    t->height[node] = 0;
    for (int q = 0; q < t->deg[node]; q++) {
        int ch = t->nbr[node][q];
        if (ch == dad) continue;
        int leaf = farthest_leaf(t, ch, node);
        if (t->height[node] < t->height[ch] + 1) {
            t->height[node] = t->height[ch] + 1;
            res = leaf;
        }
    }
    return res;
}

double orc_tree_compute_likelihood(orc_tree *t, double *pattern_lh) {
    if (t->cur_node1 < 0) {
        int leaf = farthest_leaf(t, 0, -1); /* root is taxon 0, a leaf */
        t->cur_node1 = leaf;
        t->cur_node2 = t->nbr[leaf][0];
    }
    /* computeLikelihoodBranch(current_it = node1->node2, node1) */
    return lnl_branch(t, t->cur_node2, t->cur_node1, pattern_lh);
}

static void clear_reverse(orc_tree *t, int node, int dad) {
    for (int q = 0; q < t->deg[node]; q++) {
        int x = t->nbr[node][q];
        if (x == dad) continue;
        t->computed[x][nbr_index(t, x, node)] = 0;
        clear_reverse(t, x, node);
    }
}

/* computeFuncDerv on the current branch: node1 = current_it_back->node */
static void func_derv(orc_tree *t, double value, double *f, double *df) {
    int n1 = t->cur_node1, n2 = t->cur_node2;
    t->lengths[t->edge[n1][nbr_index(t, n1, n2)]] = value;
    int node = n2, dad = n1;
    if (is_leaf(t, node)) { node = n1; dad = n2; }
    run_traversal(t, node, dad);
    if (!t->theta_computed) {
        orc_compute_theta(&t->m, t->partials, t->scale, dref(t, dad, node), dref(t, node, dad),
                          t->theta, t->buffer_scale, t->nth);
        t->theta_computed = 1;
    }
    double d1, d2;
    orc_derv(&t->m, t->theta, t->buffer_scale, value, &d1, &d2, t->nth);
    *f = -d1;
    *df = -d2;
}

static double lnl_from_buffer(orc_tree *t) {
    int n1 = t->cur_node1, n2 = t->cur_node2;
    return orc_lnl_from_buffer(&t->m, t->theta, t->buffer_scale, branch_len(t, n1, n2), NULL, t->nth);
}

/* Optimization::minimizeNewton (utils/optimization.cpp:422-499); *status=-1 on failure */
static double minimize_newton(orc_tree *t, double x1, double xguess, double x2, double xacc,
                              int max_nr_step, int *status) {
    double f, df, dx, dxold, temp, xh, xl, rts, rts_old;
    rts = xguess;
    if (rts < x1) rts = x1;
    if (rts > x2) rts = x2;
    func_derv(t, rts, &f, &df);
    if (!isfinite(f) || !isfinite(df)) { *status = -1; return rts; }
    if (df >= 0.0 && fabs(f) < xacc) return rts;
    if (f < 0.0) { xl = rts; xh = x2; } else { xh = rts; xl = x1; }
    dx = dxold = fabs(xh - xl);
    for (int j = 1; j <= max_nr_step; j++) {
        rts_old = rts;
        if ((df <= 0.0) || (((rts - xh) * df - f) * ((rts - xl) * df - f) >= 0.0)) {
            dxold = dx;
            dx = 0.5 * (xh - xl);
            rts = xl + dx;
            if (xl == rts) return rts;
        } else {
            dxold = dx;
            dx = f / df;
            temp = rts;
            rts -= dx;
            if (temp == rts) return rts;
        }
        (void)dxold;
        if (fabs(dx) < xacc || (j == max_nr_step)) return rts_old;
        func_derv(t, rts, &f, &df);
        if (!isfinite(f) || !isfinite(df)) { *status = -1; return rts; }
        if (df > 0.0 && fabs(f) < xacc) return rts;
        if (f < 0.0) xl = rts;
        else if (f > 0.0) xh = rts;
    }
    *status = -1;
    return 0.0;
}

int orc_tree_optimize_one_branch(orc_tree *t, int node1, int node2, int max_nr_step) {
    int e = t->edge[node1][nbr_index(t, node1, node2)];
    /* current_it = node1->node2; computeFuncDerv then calls
     * computeLikelihoodDerv(current_it, node1), i.e. dad = node1, node = node2 */
    t->cur_node1 = node1;
    t->cur_node2 = node2;
    double current_len = t->lengths[e];
    t->theta_computed = 0;
    int status = 0;
    double optx = minimize_newton(t, t->min_bl, current_len, t->max_bl, t->min_bl, max_nr_step, &status);
    if (status) return -1;
    if (optx > t->max_bl * 0.95) {
        /* at the length of the last derivative evaluation, as the reference
           (current_it->length, tree/phylotree.cpp:2619-2621) */
        double opt_lh = lnl_from_buffer(t);
        t->lengths[e] = current_len;
        double orig_lh = lnl_from_buffer(t);
        if (orig_lh > opt_lh) optx = current_len;
    }
    t->lengths[e] = optx;
    if (current_len != optx) {
        clear_reverse(t, node1, node2);
        clear_reverse(t, node2, node1);
    }
    return 0;
}

static void preorder(orc_tree *t, int node, int dad, int *nodes, int *nodes2, int *cnt) {
    if (dad >= 0) { nodes[*cnt] = node; nodes2[*cnt] = dad; (*cnt)++; }
    int order[ORC_MAX_DEG], d = t->deg[node];
    for (int q = 0; q < d; q++) order[q] = t->nbr[node][q];
    for (int i = 0; i < d; i++)
        for (int k = i + 1; k < d; k++)
            if (t->height[order[i]] > t->height[order[k]]) { int x = order[i]; order[i] = order[k]; order[k] = x; }
    for (int q = 0; q < d; q++)
        if (order[q] != dad) preorder(t, order[q], node, nodes, nodes2, cnt);
}

double orc_tree_optimize_all_branches(orc_tree *t, int iterations, double tolerance,
                                      int max_nr_step, int *status) {
    int *nodes = malloc(sizeof(int) * t->nedge), *nodes2 = malloc(sizeof(int) * t->nedge), cnt = 0;
    int farleaf = farthest_leaf(t, 0, -1);
    farthest_leaf(t, farleaf, -1);
    preorder(t, farleaf, -1, nodes, nodes2, &cnt);
    if (status) *status = 0;
    double tree_lh = lnl_branch(t, nodes2[0], nodes[0], NULL);
    double *saved = malloc(sizeof(double) * t->nedge);
    for (int it = 0; it < iterations; it++) {
        memcpy(saved, t->lengths, sizeof(double) * t->nedge);
        for (int j = 0; j < cnt; j++) {
            if (orc_tree_optimize_one_branch(t, nodes[j], nodes2[j], max_nr_step)) {
                if (status) *status = -1;
                free(nodes); free(nodes2); free(saved);
                return tree_lh;
            }
        }
        double new_tree_lh = lnl_from_buffer(t);
        if (new_tree_lh < tree_lh - tolerance * 0.1) {
            orc_tree_set_lengths(t, saved);
            new_tree_lh = orc_tree_compute_likelihood(t, NULL);
            free(nodes); free(nodes2); free(saved);
            return new_tree_lh;
        }
        if (tree_lh <= new_tree_lh && new_tree_lh <= tree_lh + tolerance) {
            free(nodes); free(nodes2); free(saved);
            return new_tree_lh;
        }
        tree_lh = new_tree_lh;
    }
    free(nodes); free(nodes2); free(saved);
    return tree_lh;
}

int orc_tree_get_partial(orc_tree *t, int node, int nbr, double *partial, uint8_t *scale) {
    if (is_leaf(t, nbr)) return -1;
    t->nops = 0;
    traverse(t, node, nbr);
    if (t->nops) {
        orc_compute_partials(&t->m, t->partials, t->scale, t->ops, t->nops, t->nth);
        t->nupdates += (long long)t->nops * t->m.nptn;
    }
    int s = dref(t, node, nbr);
    const int B = t->m.nstates * t->m.ncat;
    const size_t ss = (size_t)t->m.nptn * (t->m.safe ? t->m.ncat : 1);
    memcpy(partial, t->partials + (size_t)s * t->m.nptn * B, sizeof(double) * (size_t)t->m.nptn * B);
    memcpy(scale, t->scale + (size_t)s * ss, ss);
    return 0;
}

int orc_tree_derv(orc_tree *t, int node1, int node2, double len, double *df, double *ddf) {
    if (nbr_index(t, node1, node2) < 0) return -1;
    t->cur_node1 = node1;
    t->cur_node2 = node2;
    t->theta_computed = 0;
    double f, d;
    func_derv(t, len, &f, &d);
    *df = -f;
    *ddf = -d;
    return 0;
}

double orc_tree_lnl_branch(orc_tree *t, int node, int dad, double *pattern_lh) {
    return lnl_branch(t, node, dad, pattern_lh);
}
