// Mixed-precision path, part 1: per-op transition matrices and leaf tables,
// derivative and from-buffer kernels, parameter plumbing. The traversal
// kernel is in traverse_mixed.cu.
//
// Standard basis keeps every partial non-negative (no eigen-space
// cancellation in FP32): dad[c][x] = (P_L,c L_c)[x] * (P_R,c R_c)[x]; a
// pattern is rescaled by an exact power of two when its largest entry falls
// below 2^-40 and the exponent is carried per pattern. FP64 stays in
// exp(lambda r t), the products forming P(t), the per-pattern log, the
// weighted lnL sum, the exponent correction and the derivative sums.
#include <cuda_runtime.h>

#include "mixed.cuh"
#include "nonrev.cuh"

namespace iqg {

// ---------------------------------------------------------------------------
// per-op transition matrices and leaf tables (FP64 exp and products, stored FP32)
// (computePartialInfo, tree/phylokernelnew.h:895-1110, in the standard basis)
// ---------------------------------------------------------------------------
__global__ void k_partial_info_mixed(const OpDev *__restrict__ ops, float *__restrict__ opmats, long long op_stride,
                                     const double *__restrict__ evec, const double *__restrict__ inv,
                                     const double *__restrict__ eval, const double *__restrict__ rates,
                                     const double *__restrict__ tip_lh, int n, int npad, int C, int S, int nmix,
                                     int cpc) {
    const int k = blockIdx.x, ch = blockIdx.y, z = blockIdx.z, Z = gridDim.z;
    const OpDev op = ops[k];
    const double len = op.len[ch];
    const long long nn = (long long)n * n;
    __shared__ double sexp[kMaxCat * kMaxStates];
    for (int t = threadIdx.x; t < C * n; t += blockDim.x) {
        const int c = t / n, i = t % n;
        sexp[t] = exp(eval[(c / cpc) * n + i] * (rates[c] * len));
    }
    __syncthreads();
    float *base = opmats + (long long)k * op_stride;
    const long long PM = (long long)C * n * npad;
    float *Pm = base + ch * PM;
    const long long TB = (long long)(S + 1) * C * npad;
    float *tab = base + 2 * PM + ch * TB;
    const long long nP = PM, nT = (op.child[ch] < 0) ? TB : 0;
    const long long total = nP + nT;
    for (long long t = (long long)z * blockDim.x + threadIdx.x; t < total; t += (long long)Z * blockDim.x) {
        if (t < nP) {
            // P_c[x][y] = sum_i U[x][i] exp(lambda_i r_c t) U^-1[i][y]
            const int c = (int)(t / ((long long)n * npad)), r = (int)(t % ((long long)n * npad));
            const int x = r / npad, y = r % npad;
            const double *U = evec + (c / cpc) * nn, *Ui = inv + (c / cpc) * nn;
            double acc = 0.0;
            if (y < n)
                for (int i = 0; i < n; i++) acc = fma(U[x * n + i] * sexp[c * n + i], Ui[i * n + y], acc);
            Pm[t] = (float)acc;
        } else {
            // leaf table[s][c][x] = (P_c . tipvec_s)[x] = sum_i U[x][i] exp(.) tip_lh[s][i]
            const long long u = t - nP;
            const int s = (int)(u / ((long long)C * npad)), r = (int)(u % ((long long)C * npad));
            const int c = r / npad, x = r % npad, m = c / cpc;
            const double *U = evec + m * nn, *tv = tip_lh + ((long long)s * nmix + m) * n;
            double acc = 0.0;
            if (x < n) {
                if (s == S) {
                    acc = 1.0;  // unknown state: P . 1 = 1
                } else {
                    for (int i = 0; i < n; i++) acc = fma(U[x * n + i] * sexp[c * n + i], tv[i], acc);
                }
            }
            tab[u] = (float)acc;
        }
    }
}

// Double-float product a * b accumulated into (sh, sl): the product's rounding
// error from FMAs, the addition's from TwoSum (Knuth), explicitly rounded
// operations so no contraction changes the error terms. About 44 bits.
__device__ __forceinline__ void df_mac(float ah, float al, float bh, float bl, float &sh, float &sl) {
    const float p = __fmul_rn(ah, bh);
    float pe = fmaf(ah, bh, -p);
    pe = fmaf(ah, bl, pe);
    pe = fmaf(al, bh, pe);
    const float sum = __fadd_rn(sh, p);
    const float bp = __fsub_rn(sum, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(sum, bp)), __fsub_rn(p, bp));
    sh = sum;
    sl = __fadd_rn(sl, __fadd_rn(err, pe));
}

__device__ __forceinline__ void df_split(double v, float &h, float &l) {
    h = (float)v;
    l = (float)(v - (double)h);
}

// Same outputs as k_partial_info_mixed for 16..64 states. One CTA per (op,
// child, category, block of 16 rows): U diag(exp(lambda r_c t)) for its rows
// is split into FP32 pairs in shared memory; U^-1 and the eigen-space tip
// vectors were split once per model (d_ivhl, d_tiphl) and are read through
// L1. Each output is a double-float dot product of length n, rounded once to
// FP32 at the end. GB300 runs FP64 FMAs ~60x slower than FP32; the result is
// stored in FP32, so the 44-bit double-float sums lose nothing that is kept.
constexpr int kPiRows = 8;
__global__ void __launch_bounds__(256) k_partial_info_df(const OpDev *__restrict__ ops, float *__restrict__ opmats,
                                                         long long op_stride, const double *__restrict__ evec,
                                                         const double *__restrict__ eval,
                                                         const double *__restrict__ rates,
                                                         const float *__restrict__ ivhl,
                                                         const float *__restrict__ tiphl, int n, int npad, int C,
                                                         int S, int unit_tips, int nmix, int cpc) {
    __shared__ float ue_h[kPiRows * kMaxStates], ue_l[kPiRows * kMaxStates];
    __shared__ float s_p[kPiRows * kMaxStates];  // this block's rows of P(t), for unit tip vectors
    __shared__ double s_exp[kMaxStates];
    const int rb = (npad + kPiRows - 1) / kPiRows;
    const int k = blockIdx.x, ch = blockIdx.y, c = blockIdx.z / rb, x0 = (blockIdx.z % rb) * kPiRows;
    const int child = ch ? ops[k].child[1] : ops[k].child[0];
    const double len = ch ? ops[k].len[1] : ops[k].len[0];
    const bool tip = child < 0;
    const int nn = n * n, m = c / cpc;  // mixture class of category c
    const double rl = rates[c] * len;
    ivhl += (long long)m * 2 * nn;  // this class's U^-1 split: [hi nn][lo nn]
    // n FP64 exponentials per CTA, then this block's rows of U diag(exp)
    for (int i = threadIdx.x; i < n; i += blockDim.x) s_exp[i] = exp(eval[m * n + i] * rl);
    __syncthreads();
    for (int t = threadIdx.x; t < kPiRows * n; t += blockDim.x) {
        const int xr = t / n, i = t % n, x = x0 + xr;
        if (x < n) df_split(evec[(long long)m * nn + x * n + i] * s_exp[i], ue_h[xr * n + i], ue_l[xr * n + i]);
    }
    __syncthreads();
    float *base = opmats + (long long)k * op_stride;
    const long long PM = (long long)C * n * npad;
    float *Pm = base + ch * PM + (long long)c * n * npad;
    for (int e = threadIdx.x; e < kPiRows * npad; e += blockDim.x) {
        const int xr = e / npad, y = e % npad, x = x0 + xr;
        if (x >= n) continue;
        float sh = 0.f, sl = 0.f;
        if (y < n)
            for (int i = 0; i < n; i++)
                df_mac(ue_h[xr * n + i], ue_l[xr * n + i], __ldg(ivhl + i * n + y), __ldg(ivhl + nn + i * n + y), sh,
                       sl);
        const float pv = __fadd_rn(sh, sl);
        Pm[x * npad + y] = pv;
        s_p[xr * npad + y] = pv;
    }
    if (!tip) return;
    __syncthreads();  // s_p complete
    // leaf table[s][c][x] = sum_i (U e)[x][i] tip_lh[s][i]; the unknown state gives 1
    const long long TB = (long long)(S + 1) * C * npad;
    const int ts = (S + 1) * nmix * n;  // floats of one half of tiphl ([state][class][i])
    float *tab = base + 2 * PM + ch * TB;
    for (int u = threadIdx.x; u < (S + 1) * kPiRows; u += blockDim.x) {
        const int st = u / kPiRows, xr = u % kPiRows, x = x0 + xr;
        if (x >= npad) continue;
        float v = 0.f;
        if (x < n) {
            if (st == S) {
                v = 1.f;
            } else if (unit_tips && st < n) {  // tip vector = column st of U^-1: the same sums as P[x][st]
                v = s_p[xr * npad + st];
            } else {
                float sh = 0.f, sl = 0.f;
                const int tb = (st * nmix + m) * n;
                for (int i = 0; i < n; i++)
                    df_mac(ue_h[xr * n + i], ue_l[xr * n + i], __ldg(tiphl + tb + i), __ldg(tiphl + ts + tb + i), sh,
                           sl);
                v = __fadd_rn(sh, sl);
            }
        }
        tab[(long long)st * C * npad + (long long)c * npad + x] = v;
    }
}

// ---------------------------------------------------------------------------
// derivatives and lnL from the FP32 theta buffer, FP64 sums
// (tree/phylokernelnew.h:2233-2633 and :3232-3428)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTPB) k_derv_mixed(const MixBufParams P) {
    __shared__ double v0[kMaxCat * kMaxStates], v1[kMaxCat * kMaxStates], v2[kMaxCat * kMaxStates];
    const int n = P.n, C = P.ncat, B = n * C;
    for (int t = threadIdx.x; t < B; t += blockDim.x) {
        const int c = t / n, i = t % n;
        const double cof = P.eval[(c / P.cpc) * n + i] * P.rates[c];
        const double val = exp(cof * P.len) * P.props[c];
        const double val1 = cof * val;
        v0[t] = val;
        v1[t] = val1;
        v2[t] = cof * val1;
    }
    __syncthreads();
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double r[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
    if (p < P.nptn) {
        const float *th = P.theta + p;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        for (int k = 0; k < B; k++) {
            const double t0 = (double)th[(long long)k * P.ldp];
            a0 = fma(v0[k], t0, a0);
            a1 = fma(v1[k], t0, a1);
            a2 = fma(v2[k], t0, a2);
        }
        // the +I term is in true scale: bring it to the stored scale
        const double lh = fabs(a0) + P.invar[p] * exp(-P.buffer_scale[p]);
        if (p >= P.asc_first) {  // +ASC constant pattern, in true scale (weight 0 below)
            const double u = exp(P.buffer_scale[p]);
            double *o = P.asc_out + 3 * (p - P.asc_first);
            o[0] = lh * u;
            o[1] = a1 * u;
            o[2] = a2 * u;
        }
        const double inv = 1.0 / lh;
        const double df_frac = a1 * inv, ddf_frac = a2 * inv;
        const double f = P.freq[p];
        const double tmp1 = df_frac * f, tmp2 = ddf_frac * f;
        r[0] = tmp1;
        r[1] = fma(-tmp1, df_frac, tmp2);
        r[2] = (log(lh) + P.buffer_scale[p]) * f;
    }
    mix_grid_reduce(r, P.red);
}

__global__ void __launch_bounds__(kTPB) k_from_buffer_mixed(const MixBufParams P) {
    __shared__ double v0[kMaxCat * kMaxStates];
    const int n = P.n, C = P.ncat, B = n * C;
    for (int t = threadIdx.x; t < B; t += blockDim.x) {
        const int c = t / n, i = t % n;
        v0[t] = exp(P.eval[(c / P.cpc) * n + i] * (P.rates[c] * P.len)) * P.props[c];
    }
    __syncthreads();
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double r[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
    if (p < P.nptn) {
        const float *th = P.theta + p;
        double a0 = 0.0;
        for (int k = 0; k < B; k++) a0 = fma(v0[k], (double)th[(long long)k * P.ldp], a0);
        const double lh = fabs(a0) + P.invar[p] * exp(-P.buffer_scale[p]);
        const double plh = log(lh) + P.buffer_scale[p];
        P.pattern_lh[p] = plh;
        const double f = P.freq[p];
        r[0] = plh * f;
        r[1] = (isfinite(plh) ? plh : 4.0 * kLogScaleThreshold) * f;
        r[2] = isfinite(plh) ? 0.0 : 1.0;
    }
    mix_grid_reduce(r, P.red);
}

// ---------------------------------------------------------------------------
// non-reversible models (tree/phylokernelnonrev.h; P(t) from the complex eigen
// system as ModelMarkov::computeTransMatrixNonrev, model/modelmarkov.cpp:480-490)
// ---------------------------------------------------------------------------
// Per-op P(t) blocks and leaf tables for a non-reversible model, in the layout
// of k_partial_info_mixed: one CTA per (op, child, category). A child reached
// against the edge direction takes P^T; the root leaf's rows are P . root
// frequencies for every state (tree/phylokernelnew.h:932-963).
__global__ void __launch_bounds__(256) k_partial_info_nonrev(const OpDev *__restrict__ ops, float *__restrict__ opmats,
                                                             long long op_stride, const double *__restrict__ nr,
                                                             const double *__restrict__ rates, int n, int npad, int C,
                                                             int S) {
    extern __shared__ double nv_smem[];  // [n*n] P, [2n] exp scratch
    const int k = blockIdx.x, ch = blockIdx.y, c = blockIdx.z;
    const OpDev op = ops[k];
    const NonrevModel m = nonrev_model(nr, n, S);
    double *Pd = nv_smem, *ex = nv_smem + n * n;
    nonrev_matrix(m, n, rates[c], op.len[ch], 0, ex, Pd);
    const bool tr = (op.flags >> ch) & 1, root = (op.flags >> (2 + ch)) & 1;
    float *base = opmats + (long long)k * op_stride;
    const long long PM = (long long)C * n * npad, TB = (long long)(S + 1) * C * npad;
    float *Pm = base + ch * PM + (long long)c * n * npad;
    for (int t = threadIdx.x; t < n * npad; t += blockDim.x) {
        const int x = t / npad, y = t % npad;
        Pm[t] = y < n ? (float)(tr ? Pd[y * n + x] : Pd[x * n + y]) : 0.f;
    }
    if (op.child[ch] >= 0) return;
    float *tab = base + 2 * PM + ch * TB;
    for (int t = threadIdx.x; t < (S + 1) * npad; t += blockDim.x) {
        const int st = t / npad, x = t % npad;
        double acc = 0.0;
        if (x < n) {
            const double *v = root ? m.root : m.tipv + (long long)st * n;
            for (int y = 0; y < n; y++) acc = fma(tr ? Pd[y * n + x] : Pd[x * n + y], v[y], acc);
        }
        tab[(long long)st * C * npad + (long long)c * npad + x] = (float)acc;
    }
}

// prop_c * (r_c lambda)^k-weighted P(r_c t) for k = 0, 1, 2 (P, dP/dt, d2P/dt2):
// one CTA per (category, k), FP32 [3][C][n][npad]
__global__ void __launch_bounds__(256) k_nonrev_branch_mats(float *__restrict__ out, const double *__restrict__ nr,
                                                            const double *__restrict__ rates,
                                                            const double *__restrict__ props, double len, int n,
                                                            int npad, int C, int S) {
    extern __shared__ double nv_smem[];
    const int c = blockIdx.x, k = blockIdx.y;
    double *Pd = nv_smem, *ex = nv_smem + n * n;
    nonrev_matrix(nonrev_model(nr, n, S), n, rates[c], len, k, ex, Pd);
    float *o = out + ((long long)k * C + c) * n * npad;
    for (int t = threadIdx.x; t < n * npad; t += blockDim.x) {
        const int x = t / npad, y = t % npad;
        o[t] = y < n ? (float)(props[c] * Pd[x * n + y]) : 0.f;
    }
}

// Branch lnL (and, with DERV, the Newton-Raphson sums) of a non-reversible
// model straight from the two ends' partials: per pattern and category
// lh_k = sum_x pi_x a[x] (M_k b)[x], M_k the branch matrices above
// (tree/phylokernelnonrev.h:586-1056, 1062-1528); a is the dad side. FP32
// products per category, FP64 sums over categories and patterns; the same
// reductions as k_derv_mixed / k_from_buffer_mixed.
template <bool DERV>
__global__ void __launch_bounds__(kTPB) k_branch_nonrev(const MixParams P, const float *__restrict__ mats,
                                                        const double *__restrict__ tipv) {
    const int n = P.n, npad = P.npad, C = P.ncat;
    const long long ld = P.ldp;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double r[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
    if (p < P.nptn) {
        const long long pb = (p >> 3) * (8LL * C * npad) + (p & 7) * 4;
        const float *pa = P.part + (long long)P.a * P.slot_floats + pb;
        const bool btip = P.b < 0;
        const float *pbp = btip ? nullptr : P.part + (long long)P.b * P.slot_floats + pb;
        const int sb = btip ? P.states[(long long)(-1 - P.b) * ld + p] : 0;
        const int ea = P.expo[(long long)P.a * ld + p], eb = btip ? 0 : P.expo[(long long)P.b * ld + p];
        double h0 = 0.0, h1 = 0.0, h2 = 0.0;
        for (int c = 0; c < C; c++) {
            float bv[kMaxStates];
            for (int y = 0; y < n; y++)
                bv[y] = btip ? (float)tipv[(long long)sb * n + y] : pbp[(c * npad + (y & ~3)) * 8 + (y & 3)];
            float l0 = 0.f, l1 = 0.f, l2 = 0.f;
            for (int x = 0; x < n; x++) {
                const float *m0 = mats + ((long long)c * n + x) * npad;
                float w0 = 0.f, w1 = 0.f, w2 = 0.f;
                for (int y = 0; y < n; y++) {
                    w0 = fmaf(__ldg(m0 + y), bv[y], w0);
                    if (DERV) {
                        w1 = fmaf(__ldg(m0 + (long long)C * n * npad + y), bv[y], w1);
                        w2 = fmaf(__ldg(m0 + 2LL * C * n * npad + y), bv[y], w2);
                    }
                }
                const float av = (float)__ldg(P.pi + x) * pa[(c * npad + (x & ~3)) * 8 + (x & 3)];
                l0 = fmaf(av, w0, l0);
                if (DERV) {
                    l1 = fmaf(av, w1, l1);
                    l2 = fmaf(av, w2, l2);
                }
            }
            h0 += l0;
            h1 += l1;
            h2 += l2;
        }
        // the +I term is in true scale: bring it to the stored scale 2^-(ea+eb)
        const double lh = fabs(h0) + ldexp(P.invar[p], -(ea + eb));
        const double plh = log(lh) + (double)(ea + eb) * kLn2;
        const double f = P.freq[p];
        if (DERV) {
            const double df_frac = h1 / lh, ddf_frac = h2 / lh;
            const double tmp1 = df_frac * f, tmp2 = ddf_frac * f;
            r[0] = tmp1;
            r[1] = fma(-tmp1, df_frac, tmp2);
            r[2] = plh * f;
        } else {
            P.pattern_lh[p] = plh;
            r[0] = plh * f;
            r[1] = (isfinite(plh) ? plh : 4.0 * kLogScaleThreshold) * f;
            r[2] = isfinite(plh) ? 0.0 : 1.0;
        }
    }
    mix_grid_reduce(r, P.red);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
MixParams mix_params(iqgpu_engine *e, int nops) {
    MixParams P;
    P.n = e->n;
    P.npad = e->npad;
    P.ncat = e->C;
    P.state_unknown = e->S;
    P.nops = nops;
    P.op_base = 0;
    P.nptn = (int)e->P;
    P.ldp = e->Ppad;
    P.slot_floats = e->Ppad * e->bp;
    P.op_stride = e->op_stride32;
    P.ops = e->d_ops;
    P.opmats = e->d_opmats32;
    // the FP32 copy of U^-1 ([n][npad]) lives after max_ops+1 op matrix blocks
    P.inv32 = e->d_opmats32 + (long long)(e->cfg.max_ops + 1) * e->op_stride32;
    P.pi = e->d_pi;
    P.tip_lh = e->d_tip;
    P.nmix = e->nmix;
    P.cpc = e->cpc;
    P.freq = e->d_freq;
    P.invar = e->d_invar;
    P.eval = e->d_eval;
    P.rates = e->d_rates;
    P.props = e->d_props;
    P.states = e->d_states;
    P.part = e->d_part32;
    P.expo = e->d_exp;
    P.a = P.b = 0;
    P.len = 0.0;
    P.pattern_lh = e->d_plh;
    P.theta = e->d_theta32;
    P.buffer_scale = e->d_bscale;
    P.red.partials = e->d_red_partials;
    P.red.ticket = e->d_ticket;
    P.red.out = e->d_red_out;
    P.status = e->d_status;
    P.wait_polls = e->wait_polls ? e->wait_polls : kWaitPolls;
    P.branch_op = nops;
    return P;
}

int launch_partial_info_mixed(iqgpu_engine *e, int nops_with_branch) {
    if (nops_with_branch <= 0) return IQGPU_OK;
    if (e->nonrev) {
        const size_t smem = ((size_t)e->n * e->n + 2 * e->n) * 8;
        k_partial_info_nonrev<<<dim3(nops_with_branch, 2, e->C), 256, smem, e->st>>>(
            e->d_ops, e->d_opmats32, e->op_stride32, e->d_nr, e->d_rates, e->n, e->npad, e->C, e->S);
        e->launches++;
        return cuda_fail(cudaGetLastError(), "partial_info_nonrev");
    }
    if (e->n >= 16 && e->d_ivhl) {  // double-float products, one CTA per (op, child, category, 16 rows)
        const int rb = (e->npad + kPiRows - 1) / kPiRows;
        k_partial_info_df<<<dim3(nops_with_branch, 2, e->C * rb), 256, 0, e->st>>>(
            e->d_ops, e->d_opmats32, e->op_stride32, e->d_evec, e->d_eval, e->d_rates, e->d_ivhl, e->d_tiphl, e->n,
            e->npad, e->C, e->S, e->unit_tips ? 1 : 0, e->nmix, e->cpc);
        e->launches++;
        return cuda_fail(cudaGetLastError(), "partial_info_df");
    }
    const int Z = e->n > 20 ? 32 : 4;
    dim3 grid(nops_with_branch, 2, Z);
    k_partial_info_mixed<<<grid, 256, 0, e->st>>>(e->d_ops, e->d_opmats32, e->op_stride32, e->d_evec, e->d_inv,
                                                   e->d_eval, e->d_rates, e->d_tip, e->n, e->npad, e->C, e->S,
                                                   e->nmix, e->cpc);
    e->launches++;
    return cuda_fail(cudaGetLastError(), "partial_info_mixed");
}

static MixBufParams mixbuf_params(iqgpu_engine *e, double len) {
    MixBufParams P;
    P.n = e->n;
    P.ncat = e->C;
    P.cpc = e->cpc;
    P.nptn = (int)e->P;
    P.ldp = e->Ppad;
    P.theta = e->d_theta32;
    P.buffer_scale = e->d_bscale;
    P.freq = e->d_freq;
    P.invar = e->d_invar;
    P.eval = e->d_eval;
    P.rates = e->d_rates;
    P.props = e->d_props;
    P.len = len;
    P.pattern_lh = e->d_plh;
    P.red.partials = e->d_red_partials;
    P.red.ticket = e->d_ticket;
    P.red.out = e->d_red_out;
    P.asc_first = (int)(e->P - e->asc_n);
    P.asc_out = e->d_asc_holder ? e->d_asc_holder : e->d_asc;
    return P;
}

int launch_derv_mixed(iqgpu_engine *e, double len) {
    k_derv_mixed<<<e->nblk, kTPB, 0, e->st>>>(mixbuf_params(e, len));
    e->launches++;
    return cuda_fail(cudaGetLastError(), "derv_mixed");
}

int launch_branch_nonrev(iqgpu_engine *e, double len, bool derv) {
    const size_t smem = ((size_t)e->n * e->n + 2 * e->n) * 8;
    k_nonrev_branch_mats<<<dim3(e->C, derv ? 3 : 1), 256, smem, e->st>>>(e->d_nrmats, e->d_nr, e->d_rates, e->d_props,
                                                                        len, e->n, e->npad, e->C, e->S);
    e->launches++;
    int rc = cuda_fail(cudaGetLastError(), "nonrev_branch_mats");
    if (rc) return rc;
    MixParams P = mix_params(e, 0);
    P.a = e->theta_a;
    P.b = e->theta_b;
    const NonrevModel m = nonrev_model(e->d_nr, e->n, e->S);
    if (derv)
        k_branch_nonrev<true><<<e->nblk, kTPB, 0, e->st>>>(P, e->d_nrmats, m.tipv);
    else
        k_branch_nonrev<false><<<e->nblk, kTPB, 0, e->st>>>(P, e->d_nrmats, m.tipv);
    e->launches++;
    return cuda_fail(cudaGetLastError(), "branch_nonrev");
}

int launch_from_buffer_mixed(iqgpu_engine *e, double len) {
    k_from_buffer_mixed<<<e->nblk, kTPB, 0, e->st>>>(mixbuf_params(e, len));
    e->launches++;
    return cuda_fail(cudaGetLastError(), "from_buffer_mixed");
}

}  // namespace iqg
