// FP64 drop-in path: eigen-space partials with the reference's 2^-256
// scaling, one CUDA thread per pattern, the whole traversal in one launch.
//
// Layout in HBM: a partial slot is [B rows][ldp patterns] doubles with
// row r = c*n + x (category-major, then state) and patterns contiguous, so a
// warp reads 32 consecutive patterns of one row: 256-byte coalesced lines.
// Scale counts are uint8 [ldp] (NORM) or [ncat][ldp] (SAFE).
//
// Every pattern is independent along the whole traversal, so a CTA walks the
// full op list for its 128 patterns and no grid-wide synchronisation is
// needed between ops (the reference does the same per OpenMP packet,
// tree/phylokernelnew.h:2808-2823).
#include <cuda_runtime.h>

#include "engine.cuh"
#include "nonrev.cuh"

namespace iqg {

// ---------------------------------------------------------------------------
// per-op precompute: echild = U diag(exp(lambda r_c t)) and leaf lookup tables
// (computePartialInfo, tree/phylokernelnew.h:895-1110)
// ---------------------------------------------------------------------------
// Mixtures: category c takes its class's eigen system (m = c / cpc) and the
// class's eigen-space tip vectors tip_lh[s][m] (tree/phylokernelnew.h:908-918).
// With `pass` set, record k comes from pass.src with its lengths read from
// pass.len (by pass.edge), and is written to ops for the traversal after it.
struct PassStage {
    const OpDev *src;
    const int32_t *edge;
    const double *len;
};
__global__ void k_partial_info_f64(OpDev *__restrict__ ops, double *__restrict__ opmats,
                                   const double *__restrict__ evec, const double *__restrict__ eval,
                                   const double *__restrict__ rates, const double *__restrict__ tip_lh,
                                   int n, int C, int S, int nmix, int cpc, const PassStage pass) {
    pdl_wait();  // a pass's lengths come from the solve before
    pdl_trigger();
    const int k = blockIdx.x, ch = blockIdx.y, z = blockIdx.z, Z = gridDim.z;
    OpDev op;
    if (pass.src) {
        op = pass.src[k];
        op.len[0] = pass.edge[2 * k] >= 0 ? pass.len[pass.edge[2 * k]] : 0.0;
        op.len[1] = pass.edge[2 * k + 1] >= 0 ? pass.len[pass.edge[2 * k + 1]] : 0.0;
        if (ch == 0 && z == 0 && threadIdx.x == 0) ops[k] = op;
    } else {
        op = ops[k];
    }
    const int ref = op.child[ch];
    if (ref == IQGPU_NO_CHILD) return;  // odd child count of a multifurcating node
    const double len = op.len[ch];
    const long long CNN = (long long)C * n * n;
    const int B = n * C;
    double *base = opmats + op.mat_off;
    double *echild = base + ch * CNN;
    __shared__ double sexp[kMaxCat * kMaxStates];
    for (int t = threadIdx.x; t < C * n; t += blockDim.x) {
        const int c = t / n, i = t % n;
        sexp[t] = exp(eval[(c / cpc) * n + i] * (rates[c] * len));
    }
    __syncthreads();
    const long long nn = (long long)n * n;
    if (z == 0) {
        for (long long t = threadIdx.x; t < CNN; t += blockDim.x) {
            const int c = (int)(t / (n * n)), x = (int)((t / n) % n), i = (int)(t % n);
            echild[t] = evec[(c / cpc) * nn + x * n + i] * sexp[c * n + i];
        }
    }
    if (ref >= 0) return;
    double *tab = base + 2 * CNN + (long long)ch * (S + 1) * B;
    const long long rows = (long long)S * B;
    for (long long t = (long long)z * blockDim.x + threadIdx.x; t < rows; t += (long long)Z * blockDim.x) {
        const int s = (int)(t / B), r = (int)(t % B), c = r / n, x = r % n, m = c / cpc;
        const double *T = tip_lh + ((long long)s * nmix + m) * n, *U = evec + m * nn;
        double acc = (U[x * n] * sexp[c * n]) * T[0];
        for (int i = 1; i < n; i++) acc = fma(U[x * n + i] * sexp[c * n + i], T[i], acc);
        tab[t] = acc;
    }
    if (z == 0)
        for (int t = threadIdx.x; t < B; t += blockDim.x) tab[rows + t] = 1.0;  // STATE_UNKNOWN row
}

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
template <int NT>
__device__ __forceinline__ double dot_reg(const double *__restrict__ row, const double (&v)[NT]) {
    // 4 independent accumulators (the reference's unrolling, and FP64 FMA latency hiding)
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
#pragma unroll
    for (int i = 0; i + 3 < NT; i += 4) {
        a0 = fma(__ldg(row + i), v[i], a0);
        a1 = fma(__ldg(row + i + 1), v[i + 1], a1);
        a2 = fma(__ldg(row + i + 2), v[i + 2], a2);
        a3 = fma(__ldg(row + i + 3), v[i + 3], a3);
    }
#pragma unroll
    for (int i = NT & ~3; i < NT; i++) a0 = fma(__ldg(row + i), v[i], a0);
    return (a0 + a1) + (a2 + a3);
}

__device__ __forceinline__ void warp_reduce(double (&v)[kRedSlots]) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int k = 0; k < kRedSlots; k++) v[k] += __shfl_xor_sync(0xffffffffu, v[k], off);
}

// Block sums -> partials[blockIdx.x]; the last CTA adds all partials in CTA
// order (deterministic) into red.out and re-arms the ticket.
__device__ void grid_reduce(double (&v)[kRedSlots], const Reduce &red) {
    __shared__ double sw[32][kRedSlots];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    warp_reduce(v);
    if (lane == 0)
        for (int k = 0; k < kRedSlots; k++) sw[wid][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        double s[kRedSlots];
        for (int k = 0; k < kRedSlots; k++) s[k] = 0.0;
        for (int w = 0; w < nw; w++)
            for (int k = 0; k < kRedSlots; k++) s[k] += sw[w][k];
        for (int k = 0; k < kRedSlots; k++) red.partials[(long long)blockIdx.x * kRedSlots + k] = s[k];
        __threadfence();
        const unsigned t = atomicAdd(red.ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s[kRedSlots];
    for (int k = 0; k < kRedSlots; k++) s[k] = 0.0;
    // fixed assignment of CTAs to threads, then a fixed-order tree: deterministic
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
        for (int k = 0; k < kRedSlots; k++) s[k] += __ldcg(red.partials + (long long)b * kRedSlots + k);
    warp_reduce(s);
    __syncthreads();
    if (lane == 0)
        for (int k = 0; k < kRedSlots; k++) sw[wid][k] = s[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < kRedSlots; k++) {
            double acc = 0.0;
            for (int w = 0; w < nw; w++) acc += sw[w][k];
            red.out[k] = acc;
        }
        *red.ticket = 0u;
    }
}

// ---------------------------------------------------------------------------
// multifurcating node (tree/phylokernelnew.h:1407-1631): one record of its
// op group. The dad's column of its own slot holds the running product of the
// children's contributions (this thread's pattern only); the first record
// sets it to one and the scale counts to zero, every child multiplies in
// (a tip as its leaf-table row, an internal child as the left-to-right sums
// echild[c][x][.].child[c][.] and its scale counts added), the 2^-256 check
// follows every child (per category in SAFE, over the block in NORM), and the
// last record transforms the product with U^-1, with no check after.
// ---------------------------------------------------------------------------
template <int NT, bool SAFE>
__device__ __forceinline__ void multi_record(const TravParams &P, const OpDev &op, bool first, bool last,
                                             long long p, double invar, double *stmp) {
    constexpr bool REG = (NT != 0 && NT <= 20);
    constexpr int NR = REG ? NT : 1;
    const int n = NT ? NT : P.n;
    const int C = P.ncat, B = n * C, S = P.state_unknown, tid = threadIdx.x;
    const long long ld = P.ldp;
    const long long CNN = (long long)C * n * n, SB = (long long)(S + 1) * B;
    double *acc = P.partials + (long long)op.dad_slot * P.slot_stride + p;
    uint8_t *sd = P.scale + (long long)op.dad_slot * P.scale_stride + p;
    if (first) {
        for (int r = 0; r < B; r++) acc[(long long)r * ld] = 1.0;
        if (SAFE) {
            for (int c = 0; c < C; c++) sd[c * ld] = 0;
        } else {
            sd[0] = 0;
        }
    }
    for (int ch = 0; ch < 2; ch++) {
        const int ref = op.child[ch];
        if (ref == IQGPU_NO_CHILD) continue;
        const double *E = P.opmats + op.mat_off + ch * CNN;
        if (ref < 0) {
            const double *T = P.opmats + op.mat_off + 2 * CNN + ch * SB +
                              (long long)P.states[(long long)(-1 - ref) * ld + p] * B;
            for (int r = 0; r < B; r++) acc[(long long)r * ld] *= __ldg(T + r);
        } else {
            const double *Cp = P.partials + (long long)ref * P.slot_stride + p;
            const uint8_t *sc = P.scale + (long long)ref * P.scale_stride + p;
            if (!SAFE) sd[0] = (uint8_t)(sd[0] + sc[0]);
            for (int c = 0; c < C; c++) {
                if (SAFE) sd[c * ld] = (uint8_t)(sd[c * ld] + sc[c * ld]);
                if constexpr (REG) {
                    double v[NR];
#pragma unroll
                    for (int i = 0; i < NR; i++) v[i] = Cp[(long long)(c * NR + i) * ld];
#pragma unroll
                    for (int x = 0; x < NR; x++) {
                        const double *e = E + (long long)(c * NR + x) * NR;
                        double y = __ldg(e) * v[0];
#pragma unroll
                        for (int i = 1; i < NR; i++) y = fma(__ldg(e + i), v[i], y);
                        acc[(long long)(c * NR + x) * ld] *= y;
                    }
                } else {
                    for (int i = 0; i < n; i++) stmp[i * blockDim.x + tid] = Cp[(long long)(c * n + i) * ld];
                    for (int x = 0; x < n; x++) {
                        const double *e = E + (long long)(c * n + x) * n;
                        double y = __ldg(e) * stmp[tid];
                        for (int i = 1; i < n; i++) y = fma(__ldg(e + i), stmp[i * blockDim.x + tid], y);
                        acc[(long long)(c * n + x) * ld] *= y;
                    }
                }
            }
        }
        if (invar != 0.0) continue;
        if (SAFE) {
            for (int c = 0; c < C; c++) {
                double m = 0.0;
                for (int x = 0; x < n; x++) m = fmax(m, fabs(acc[(long long)(c * n + x) * ld]));
                if (m < kScaleThreshold) {
                    for (int x = 0; x < n; x++) acc[(long long)(c * n + x) * ld] *= kTwoPow256;
                    sd[c * ld] += 1;
                }
            }
        } else {
            double m = 0.0;
            for (int r = 0; r < B; r++) m = fmax(m, fabs(acc[(long long)r * ld]));
            if (m < kScaleThreshold) {
                for (int r = 0; r < B; r++) acc[(long long)r * ld] *= kTwoPow256;
                sd[0] += 1;
            }
        }
    }
    if (!last) return;
    const double *__restrict__ Ui = P.inv_evec;
    for (int c = 0; c < C; c++) {
        const double *U = Ui + (long long)(c / P.cpc) * n * n;
        if constexpr (REG) {
            double t[NR];
#pragma unroll
            for (int x = 0; x < NR; x++) t[x] = acc[(long long)(c * NR + x) * ld];
#pragma unroll
            for (int x = 0; x < NR; x++) acc[(long long)(c * NR + x) * ld] = dot_reg<NR>(U + x * NR, t);
        } else {
            for (int j = 0; j < n; j++) stmp[j * blockDim.x + tid] = acc[(long long)(c * n + j) * ld];
            for (int x = 0; x < n; x++) {
                double a = 0.0;
                for (int j = 0; j < n; j++) a = fma(__ldg(U + (long long)x * n + j), stmp[j * blockDim.x + tid], a);
                acc[(long long)(c * n + x) * ld] = a;
            }
        }
    }
}

// Branch epilogue of a traversal for pattern p (theta, or the branch lnL and
// its grid sums). Every thread of the CTA calls it (the lnL form has a CTA
// barrier and the grid reduction); threads with on = false hold no pattern.
template <int NT, bool SAFE, int EPI>
__device__ __forceinline__ void f64_epilogue(const TravParams &P, long long p, double invar, double *sval, bool on) {
    const int n = NT ? NT : P.n;
    const int C = P.ncat, B = n * C;
    const int tid = threadIdx.x;
    const long long ld = P.ldp;
    // ---- epilogue on the branch (a, b): a is internal (dad_branch), b is node_branch or a tip
    const double *pa = P.partials + (long long)P.a * P.slot_stride + p;
    const uint8_t *sa = P.scale + (long long)P.a * P.scale_stride + p;
    const bool btip = P.b < 0;
    const double *pb = btip ? nullptr : P.partials + (long long)P.b * P.slot_stride + p;
    const uint8_t *sb = btip ? nullptr : P.scale + (long long)P.b * P.scale_stride + p;
    // a tip b: its state's eigen-space tip vector, per mixture class (tipv + class * n)
    const double *tipv = btip ? P.tip_lh + (long long)P.states[(long long)(-1 - P.b) * ld + p] * P.nmix * n : nullptr;
    const bool valid = on && p < P.nptn;

    if constexpr (EPI == EPI_THETA) {
        if (!on) return;
        // theta = node o dad and per-pattern scale offset (tree/phylokernelnew.h:2048-2231)
        double *th = P.theta + p;
        for (int c = 0; c < C; c++)
            for (int x = 0; x < n; x++) {
                const long long r = (long long)(c * n + x) * ld;
                th[r] = (btip ? __ldg(tipv + (c / P.cpc) * n + x) : pb[r]) * pa[r];
            }
        double bs;
        if (SAFE) {
            unsigned sum[kMaxCat], mn = 1u << 30;
            for (int c = 0; c < C; c++) {
                sum[c] = (unsigned)sa[c * ld] + (btip ? 0u : (unsigned)sb[c * ld]);
                sum[c] &= 0xffu;  // UBYTE arithmetic
                mn = min(mn, sum[c]);
            }
            for (int c = 0; c < C; c++) {
                if (sum[c] == mn + 1) {
                    for (int x = 0; x < n; x++) th[(long long)(c * n + x) * ld] *= kScaleThreshold;
                } else if (sum[c] > mn + 1) {
                    for (int x = 0; x < n; x++) th[(long long)(c * n + x) * ld] = 0.0;
                }
            }
            bs = (double)mn;
        } else {
            bs = (double)((unsigned)sa[0] + (btip ? 0u : (unsigned)sb[0]));  // NORM sums do not wrap
        }
        P.buffer_scale[p] = bs * kLogScaleThreshold;
        return;
    } else {
        // branch lnL (tree/phylokernelnew.h:2641-3223)
        for (int t = tid; t < B; t += blockDim.x) {
            const int c = t / n, i = t % n;
            sval[t] = exp(P.eval[(c / P.cpc) * n + i] * (P.rates[c] * P.len)) * P.props[c];
        }
        __syncthreads();
        // threads without a pattern add zeros; every thread reaches the one
        // grid_reduce below (its warp shuffles and barriers need the whole CTA)
        double v[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
        if (on) {
            double lh_cat[kMaxCat];
            double lh = 0.0;
            for (int c = 0; c < C; c++) {
                double acc = 0.0;
                for (int i = 0; i < n; i++) {
                    const long long r = (long long)(c * n + i) * ld;
                    const double w = btip ? sval[c * n + i] * __ldg(tipv + (c / P.cpc) * n + i) : sval[c * n + i] * pb[r];
                    acc = fma(w, pa[r], acc);
                }
                lh_cat[c] = acc;
                if (!SAFE) lh += acc;
            }
            double scale_count;
            if (SAFE) {
                unsigned sum[kMaxCat], mn = 1u << 30;
                for (int c = 0; c < C; c++) {
                    sum[c] = ((unsigned)sa[c * ld] + (btip ? 0u : (unsigned)sb[c * ld])) & 0xffu;
                    mn = min(mn, sum[c]);
                }
                for (int c = 0; c < C; c++) {
                    if (sum[c] == mn + 1) lh_cat[c] *= kScaleThreshold;
                    else if (sum[c] > mn + 1) lh_cat[c] = 0.0;
                    lh += lh_cat[c];
                }
                scale_count = (double)mn;
            } else {
                scale_count = (double)((unsigned)sa[0] + (btip ? 0u : (unsigned)sb[0]));  // NORM sums do not wrap
            }
            lh = fabs(lh) + invar;
            const double plh = log(lh) + scale_count * kLogScaleThreshold;
            P.pattern_lh[p] = plh;
            if (valid) {
                const double f = P.freq[p];
                v[0] = plh * f;
                v[1] = (isfinite(plh) ? plh : 4.0 * kLogScaleThreshold) * f;  // underflow fix-up sum
                v[2] = isfinite(plh) ? 0.0 : 1.0;
            }
        }
        grid_reduce(v, P.red);
    }
}

// ---------------------------------------------------------------------------
// traversal kernel
// ---------------------------------------------------------------------------
template <int NT, bool SAFE, int EPI>
__global__ void __launch_bounds__(kTPB) k_traverse_f64(const TravParams P) {
    constexpr bool REG = (NT != 0 && NT <= 20);
    constexpr int NR = REG ? NT : 1;  // register-array extent
    constexpr int XC = 8;             // output chunk in the shared-memory path
    const int n = NT ? NT : P.n;
    const int C = P.ncat, B = n * C, S = P.state_unknown;
    const int tid = threadIdx.x;
    const long long p = (long long)blockIdx.x * blockDim.x + tid;
    const long long ld = P.ldp;
    extern __shared__ double smem[];
    double *stmp = smem;                                          // !REG: [n][blockDim.x]
    double *sval = smem + (REG ? 0 : (long long)kMaxStates * blockDim.x);  // EPI_LNL: [B]
    const double invar = P.invar[p];
    const long long CNN = (long long)C * n * n;
    const long long SB = (long long)(S + 1) * B;
    const double *__restrict__ Ui = P.inv_evec;
    // SAFE walks with few pattern tiles: one category per CTA (its scale counts
    // and checks involve no other category); otherwise every category
    const int c_lo = P.cat_split ? (int)blockIdx.y : 0, c_hi = P.cat_split ? (int)blockIdx.y + 1 : C;

    bool in_group = false;  // inside the records of a multifurcating node
    for (int k = 0; k < P.nops; ++k) {
        const OpDev op = P.ops[k];
        const bool more = (op.flags & IQGPU_OP_MORE) != 0;
        if (more || in_group) {
            multi_record<NT, SAFE>(P, op, !in_group, !more, p, invar, stmp);
            in_group = more;
            continue;
        }
        int lref = op.child[0], rref = op.child[1];
        const double *eL = P.opmats + op.mat_off, *eR = eL + CNN;
        const double *tL = eL + 2 * CNN, *tR = tL + SB;
        if (lref >= 0 && rref < 0) {  // put the tip on the left (tree/phylokernelnew.h:1390-1400)
            int t = lref; lref = rref; rref = t;
            const double *q = eL; eL = eR; eR = q;
            q = tL; tL = tR; tR = q;
        }
        const bool lint = lref >= 0, rint = rref >= 0;
        double *dad = P.partials + (long long)op.dad_slot * P.slot_stride + p;
        uint8_t *sdad = P.scale + (long long)op.dad_slot * P.scale_stride + p;
        const double *Lp = lint ? P.partials + (long long)lref * P.slot_stride + p : nullptr;
        const double *Rp = rint ? P.partials + (long long)rref * P.slot_stride + p : nullptr;
        const double *tl = lint ? nullptr : tL + (long long)P.states[(long long)(-1 - lref) * ld + p] * B;
        const double *tr = rint ? nullptr : tR + (long long)P.states[(long long)(-1 - rref) * ld + p] * B;
        // scale counts of the dad: 0 (tip-tip), copy (tip-internal), sum (internal-internal)
        if (SAFE) {
            for (int c = c_lo; c < c_hi; c++) {
                unsigned s = 0;
                if (lint) s += P.scale[(long long)lref * P.scale_stride + c * ld + p];
                if (rint) s += P.scale[(long long)rref * P.scale_stride + c * ld + p];
                sdad[c * ld] = (uint8_t)s;
            }
        } else {
            unsigned s = 0;
            if (lint) s += P.scale[(long long)lref * P.scale_stride + p];
            if (rint) s += P.scale[(long long)rref * P.scale_stride + p];
            sdad[0] = (uint8_t)s;
        }
        const bool check = (lint || rint) && invar == 0.0;  // tip-tip never scales
        double lh_max = 0.0;
        for (int c = c_lo; c < c_hi; c++) {
            double cmax = 0.0;
            if constexpr (REG) {
                double lv[NR], rv[NR], tmp[NR];
                if (lint) {
#pragma unroll
                    for (int i = 0; i < NR; i++) lv[i] = Lp[(long long)(c * NR + i) * ld];
                }
                if (rint) {
#pragma unroll
                    for (int i = 0; i < NR; i++) rv[i] = Rp[(long long)(c * NR + i) * ld];
                }
#pragma unroll
                for (int x = 0; x < NR; x++) {
                    const double yl = lint ? dot_reg<NR>(eL + (long long)(c * NR + x) * NR, lv) : __ldg(tl + c * NR + x);
                    const double yr = rint ? dot_reg<NR>(eR + (long long)(c * NR + x) * NR, rv) : __ldg(tr + c * NR + x);
                    tmp[x] = yl * yr;
                }
                double out[NR];
#pragma unroll
                for (int x = 0; x < NR; x++) {
                    out[x] = dot_reg<NR>(Ui + (c / P.cpc) * NR * NR + x * NR, tmp);
                    cmax = fmax(cmax, fabs(out[x]));
                }
                if (SAFE && check && cmax < kScaleThreshold) {
#pragma unroll
                    for (int x = 0; x < NR; x++) out[x] *= kTwoPow256;
                    sdad[c * ld] += 1;
                }
#pragma unroll
                for (int x = 0; x < NR; x++) dad[(long long)(c * NR + x) * ld] = out[x];
            } else {
                // chunked matvecs with tmp staged in shared memory (large n)
                for (int x0 = 0; x0 < n; x0 += XC) {
                    double al[XC], ar[XC];
#pragma unroll
                    for (int xx = 0; xx < XC; xx++) { al[xx] = 0.0; ar[xx] = 0.0; }
                    if (lint || rint) {
                        for (int i = 0; i < n; i++) {
                            const double l = lint ? Lp[(long long)(c * n + i) * ld] : 0.0;
                            const double r = rint ? Rp[(long long)(c * n + i) * ld] : 0.0;
#pragma unroll
                            for (int xx = 0; xx < XC; xx++) {
                                if (x0 + xx < n) {
                                    if (lint) al[xx] = fma(__ldg(eL + (long long)(c * n + x0 + xx) * n + i), l, al[xx]);
                                    if (rint) ar[xx] = fma(__ldg(eR + (long long)(c * n + x0 + xx) * n + i), r, ar[xx]);
                                }
                            }
                        }
                    }
#pragma unroll
                    for (int xx = 0; xx < XC; xx++) {
                        if (x0 + xx < n) {
                            const double yl = lint ? al[xx] : __ldg(tl + c * n + x0 + xx);
                            const double yr = rint ? ar[xx] : __ldg(tr + c * n + x0 + xx);
                            stmp[(x0 + xx) * blockDim.x + tid] = yl * yr;
                        }
                    }
                }
                for (int x0 = 0; x0 < n; x0 += XC) {
                    double acc[XC];
#pragma unroll
                    for (int xx = 0; xx < XC; xx++) acc[xx] = 0.0;
                    for (int j = 0; j < n; j++) {
                        const double t = stmp[j * blockDim.x + tid];
#pragma unroll
                        for (int xx = 0; xx < XC; xx++)
                            if (x0 + xx < n)
                                acc[xx] = fma(__ldg(Ui + ((long long)(c / P.cpc) * n + x0 + xx) * n + j), t, acc[xx]);
                    }
#pragma unroll
                    for (int xx = 0; xx < XC; xx++) {
                        if (x0 + xx < n) {
                            dad[(long long)(c * n + x0 + xx) * ld] = acc[xx];
                            cmax = fmax(cmax, fabs(acc[xx]));
                        }
                    }
                }
                if (SAFE && check && cmax < kScaleThreshold) {
                    for (int x = 0; x < n; x++) dad[(long long)(c * n + x) * ld] *= kTwoPow256;
                    sdad[c * ld] += 1;
                }
            }
            lh_max = fmax(lh_max, cmax);
        }
        if (!SAFE && check && lh_max < kScaleThreshold) {
            for (int r = 0; r < B; r++) dad[(long long)r * ld] *= kTwoPow256;
            sdad[0] += 1;
        }
    }

    if constexpr (EPI != EPI_NONE) f64_epilogue<NT, SAFE, EPI>(P, p, invar, sval, true);
}

// ---------------------------------------------------------------------------
// Short alignments on the FP64 path, 4-state models with n * ncat <= 32: G
// lanes per pattern (the power of two >= 4 * ncat), one per (category, state)
// entry. GB300 issues only a few FP64 FMAs per clock per SM, so a pattern per
// thread leaves a DNA alignment of a few hundred patterns on a handful of SMs
// and serialises each thread's whole op chain; here the same work spreads over
// G times the warps. A lane reads its own entry of each child, the category's
// four entries come from the neighbouring lanes by shuffles, and every sum is
// formed in the order of k_traverse_f64's register path (dot_reg<4>), the
// checks and scale counts as there, so partials, scale counts and lnL are
// identical to it. Binary records only (multifurcating traversals and
// category-split walks stay on k_traverse_f64); the epilogue is
// k_traverse_f64's, run by the pattern's first lane.
// ---------------------------------------------------------------------------
template <bool SAFE, int EPI, int G>
__global__ void __launch_bounds__(128) k_traverse_f64_lanes(const TravParams P) {
    pdl_wait();  // P(t) and the children come from the kernels before
    pdl_trigger();
    constexpr int n = 4;
    static_assert(G >= 4 && G <= 32 && (G & (G - 1)) == 0, "lanes per pattern");
    __shared__ double sval[kMaxCat * kMaxStates];
    const int C = P.ncat, B = n * C;
    const int lane = threadIdx.x & 31, r = lane & (G - 1), base = lane & ~(G - 1);
    const long long p = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const bool act = r < B;
    const int c = act ? r / n : 0, x = r % n;
    const long long ld = P.ldp;
    const double invar = P.invar[p];
    const long long CNN = (long long)C * n * n;
    const long long SB = (long long)(P.state_unknown + 1) * B;
    const double *Ui = P.inv_evec + ((long long)(c / P.cpc) * n + x) * n;
    const int src = base + c * n;  // this category's first lane
    for (int k = 0; k < P.nops; ++k) {
        const OpDev op = P.ops[k];
        int lref = op.child[0], rref = op.child[1];
        const double *eL = P.opmats + op.mat_off, *eR = eL + CNN;
        const double *tL = eL + 2 * CNN, *tR = tL + SB;
        if (lref >= 0 && rref < 0) {  // put the tip on the left (tree/phylokernelnew.h:1390-1400)
            int t = lref; lref = rref; rref = t;
            const double *q = eL; eL = eR; eR = q;
            q = tL; tL = tR; tR = q;
        }
        const bool lint = lref >= 0, rint = rref >= 0;
        // scale counts of the dad: 0 (tip-tip), copy (tip-internal), sum (internal-internal)
        const long long so = SAFE ? (long long)c * ld + p : p;
        unsigned sc = 0;
        if (lint) sc += P.scale[(long long)lref * P.scale_stride + so];
        if (rint) sc += P.scale[(long long)rref * P.scale_stride + so];
        const double lv = (lint && act) ? P.partials[(long long)lref * P.slot_stride + (long long)r * ld + p] : 0.0;
        const double rv = (rint && act) ? P.partials[(long long)rref * P.slot_stride + (long long)r * ld + p] : 0.0;
        double l4[n], r4[n];
#pragma unroll
        for (int i = 0; i < n; i++) {
            l4[i] = __shfl_sync(0xffffffffu, lv, src + i);
            r4[i] = __shfl_sync(0xffffffffu, rv, src + i);
        }
        double tmp = 0.0;
        if (act) {
            const long long row = (long long)(c * n + x) * n;
            const double yl = lint ? dot_reg<n>(eL + row, l4)
                                   : __ldg(tL + (long long)P.states[(long long)(-1 - lref) * ld + p] * B + c * n + x);
            const double yr = rint ? dot_reg<n>(eR + row, r4)
                                   : __ldg(tR + (long long)P.states[(long long)(-1 - rref) * ld + p] * B + c * n + x);
            tmp = yl * yr;
        }
        double t4[n];
#pragma unroll
        for (int i = 0; i < n; i++) t4[i] = __shfl_sync(0xffffffffu, tmp, src + i);
        double out = act ? dot_reg<n>(Ui, t4) : 0.0;
        const bool check = (lint || rint) && invar == 0.0;  // tip-tip never scales
        // the category's (SAFE) or the pattern's (NORM) largest |entry|, NaN ignored as fmax does
        double m = fmax(0.0, fabs(out));
#pragma unroll
        for (int off = 1; off < (SAFE ? n : G); off <<= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
        if (check && m < kScaleThreshold) {
            out *= kTwoPow256;
            sc += 1;
        }
        if (act) P.partials[(long long)op.dad_slot * P.slot_stride + (long long)r * ld + p] = out;
        if (SAFE ? (act && x == 0) : r == 0) P.scale[(long long)op.dad_slot * P.scale_stride + so] = (uint8_t)sc;
    }
    if constexpr (EPI != EPI_NONE) {
        __syncwarp();  // the pattern's entries, written by its lanes, are visible to its first lane
        f64_epilogue<n, SAFE, EPI>(P, p, invar, sval, r == 0);
    }
}

// ---------------------------------------------------------------------------
// 20-state models on the FP64 drop-in, wide form: a CTA of 20 warps over 32
// patterns, warp x computing state x of every category (lane = pattern, so
// every global access is coalesced). k_traverse_f64's register form holds all
// of a pattern's entries in one thread (254 registers, 8 warps per SM), and its
// chains of dependent FP64 FMAs leave GB300's FP64 pipe about a third busy.
// Here a CTA stages the children's entries in shared memory once per op and
// each thread forms its entries' sums in dot_reg<20>'s order (four
// accumulators, the same products, maxima and 2^-256 checks), so partials,
// scale counts and lnL are identical to the register form. Binary records
// only; the epilogue is k_traverse_f64's, run by warp 0.
// ---------------------------------------------------------------------------
constexpr int kWideN = 20, kWideP = 32, kWideMaxCat = 4;

// dot_reg<20> with the row and the vector (stride kWideP) in shared memory
__device__ __forceinline__ double dot_wide(const double *row, const double *v) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
#pragma unroll
    for (int i = 0; i < kWideN; i += 4) {
        a0 = fma(row[i], v[i * kWideP], a0);
        a1 = fma(row[i + 1], v[(i + 1) * kWideP], a1);
        a2 = fma(row[i + 2], v[(i + 2) * kWideP], a2);
        a3 = fma(row[i + 3], v[(i + 3) * kWideP], a3);
    }
    return (a0 + a1) + (a2 + a3);
}

template <bool SAFE, int EPI>
__global__ void __launch_bounds__(kWideN * kWideP, 2) k_traverse_f64_wide(const TravParams P) {
    constexpr int n = kWideN;
    // [C][n][32] left entries, then the products; [C][n][32] right entries, then
    // |entries|; [C][n][n] echild left, echild right, U^-1 of each category's class
    extern __shared__ double wsm[];
    __shared__ double sval[kMaxCat * kMaxStates];
    __shared__ double scmax[kWideMaxCat][kWideP];  // per category and pattern: the largest |entry|
    const int C = P.ncat, B = n * C;
    const int lane = threadIdx.x & 31, x = threadIdx.x >> 5;
    const long long p = (long long)blockIdx.x * kWideP + lane;
    const long long ld = P.ldp;
    const int CN32 = C * n * kWideP, CNN = C * n * n;
    double *sL = wsm, *sR = wsm + CN32, *sM = sR;
    double *sEL = wsm + 2 * CN32, *sER = sEL + CNN, *sU = sER + CNN;
    const double invar = P.invar[p];
    const long long SB = (long long)(P.state_unknown + 1) * B;
    for (int t = threadIdx.x; t < CNN; t += blockDim.x) {  // U^-1 rows per category, once
        const int c = t / (n * n), r = t % (n * n);
        sU[t] = P.inv_evec[(long long)(c / P.cpc) * n * n + r];
    }
    for (int k = 0; k < P.nops; ++k) {
        const OpDev op = P.ops[k];
        int lref = op.child[0], rref = op.child[1];
        const double *eL = P.opmats + op.mat_off, *eR = eL + CNN;
        const double *tL = eL + 2 * CNN, *tR = tL + SB;
        if (lref >= 0 && rref < 0) {  // put the tip on the left (tree/phylokernelnew.h:1390-1400)
            int t = lref; lref = rref; rref = t;
            const double *q = eL; eL = eR; eR = q;
            q = tL; tL = tR; tR = q;
        }
        const bool lint = lref >= 0, rint = rref >= 0;
        __syncthreads();  // the previous op's readers of the shared arrays are done
        for (int c = 0; c < C; c++) {
            const long long r = (long long)(c * n + x) * ld + p;
            if (lint) sL[(c * n + x) * kWideP + lane] = P.partials[(long long)lref * P.slot_stride + r];
            if (rint) sR[(c * n + x) * kWideP + lane] = P.partials[(long long)rref * P.slot_stride + r];
        }
        for (int t = threadIdx.x; t < CNN; t += blockDim.x) {
            if (lint) sEL[t] = __ldg(eL + t);
            if (rint) sER[t] = __ldg(eR + t);
        }
        __syncthreads();
        const double *tl = lint ? nullptr : tL + (long long)P.states[(long long)(-1 - lref) * ld + p] * B;
        const double *tr = rint ? nullptr : tR + (long long)P.states[(long long)(-1 - rref) * ld + p] * B;
        double tmp[kWideMaxCat];
#pragma unroll
        for (int c = 0; c < kWideMaxCat; c++) {
            if (c >= C) break;
            const int row = (c * n + x) * n;
            const double yl = lint ? dot_wide(sEL + row, sL + c * n * kWideP + lane) : __ldg(tl + c * n + x);
            const double yr = rint ? dot_wide(sER + row, sR + c * n * kWideP + lane) : __ldg(tr + c * n + x);
            tmp[c] = yl * yr;
        }
        __syncthreads();  // every read of the children's entries is done: sL takes the products
#pragma unroll
        for (int c = 0; c < kWideMaxCat; c++) {
            if (c >= C) break;
            sL[(c * n + x) * kWideP + lane] = tmp[c];
        }
        __syncthreads();
        double out[kWideMaxCat];
#pragma unroll
        for (int c = 0; c < kWideMaxCat; c++) {
            if (c >= C) break;
            out[c] = dot_wide(sU + (c * n + x) * n, sL + c * n * kWideP + lane);
            sM[(c * n + x) * kWideP + lane] = fabs(out[c]);
        }
        __syncthreads();
        if (x < C) {  // warp c: category c's largest |entry| per pattern, in state order as the register form
            double cmax = 0.0;
            for (int xx = 0; xx < n; xx++) cmax = fmax(cmax, sM[(x * n + xx) * kWideP + lane]);
            scmax[x][lane] = cmax;
        }
        __syncthreads();
        // the category maxima (SAFE), their maximum (NORM)
        const bool check = (lint || rint) && invar == 0.0;  // tip-tip never scales
        double lh_max = 0.0;
        bool scaled[kWideMaxCat];
#pragma unroll
        for (int c = 0; c < kWideMaxCat; c++) {
            scaled[c] = false;
            if (c >= C) break;
            const double cmax = scmax[c][lane];
            if (SAFE && check && cmax < kScaleThreshold) {
                out[c] *= kTwoPow256;
                scaled[c] = true;
            }
            lh_max = fmax(lh_max, cmax);
        }
        const bool scale_all = !SAFE && check && lh_max < kScaleThreshold;
        double *dad = P.partials + (long long)op.dad_slot * P.slot_stride + p;
#pragma unroll
        for (int c = 0; c < kWideMaxCat; c++) {
            if (c >= C) break;
            dad[(long long)(c * n + x) * ld] = scale_all ? out[c] * kTwoPow256 : out[c];
        }
        if (x == 0) {  // scale counts: 0 (tip-tip), copy (tip-internal), sum (internal-internal), + this op's
            uint8_t *sdad = P.scale + (long long)op.dad_slot * P.scale_stride + p;
            if (SAFE) {
                for (int c = 0; c < C; c++) {
                    unsigned sc = 0;
                    if (lint) sc += P.scale[(long long)lref * P.scale_stride + (long long)c * ld + p];
                    if (rint) sc += P.scale[(long long)rref * P.scale_stride + (long long)c * ld + p];
                    sdad[(long long)c * ld] = (uint8_t)(sc + (scaled[c] ? 1u : 0u));
                }
            } else {
                unsigned sc = 0;
                if (lint) sc += P.scale[(long long)lref * P.scale_stride + p];
                if (rint) sc += P.scale[(long long)rref * P.scale_stride + p];
                sdad[0] = (uint8_t)(sc + (scale_all ? 1u : 0u));
            }
        }
    }
    if constexpr (EPI != EPI_NONE) {
        __syncthreads();  // the last op's entries, written by every warp, are visible to warp 0
        f64_epilogue<kWideN, SAFE, EPI>(P, p, invar, sval, x == 0);
    }
}

// ---------------------------------------------------------------------------
// SAFE walks for large state counts (codon: 21..64 states), one category per
// CTA: SAFE checks the 2^-256 threshold per category, so a category's update
// needs nothing from the others. A CTA of 16 warps over 32 patterns (lane =
// pattern); warp w computes states w, w + 16, w + 32, w + 48 of category
// blockIdx.y. Per op the CTA stages the category's child entries and both
// echild blocks in shared memory (U^-1 of the category's class once per
// launch), and each entry's sums run in the generic register-free path's
// order (one accumulator, i = 0 .. n-1), with its maximum, check and scale
// counts, so partials and scale counts are identical to it. The generic path
// kept a pattern's whole category in one thread (6 warps per SM on codon 40 x
// 10,000); here each of those sums has a thread of its own. Binary records
// only; the epilogue runs as its own launch afterwards.
// ---------------------------------------------------------------------------
constexpr int kCatWarps = 16, kCatP = 32, kCatMaxN = 64, kCatPer = kCatMaxN / kCatWarps;

__device__ __forceinline__ double dot_seq(const double *row, const double *v, int n) {
    double a = 0.0;
    for (int i = 0; i < n; i++) a = fma(row[i], v[i * kCatP], a);
    return a;
}

__global__ void __launch_bounds__(kCatWarps * kCatP, 1) k_traverse_f64_cat(const TravParams P) {
    // [n][32] left entries, then the products; [n][32] right entries; [n][n]
    // echild left, echild right, U^-1 of the category's class
    extern __shared__ double csm[];
    __shared__ double scm[kCatWarps][kCatP];
    const int n = P.n, C = P.ncat, B = n * C, c = blockIdx.y;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long p = (long long)blockIdx.x * kCatP + lane;
    const long long ld = P.ldp;
    const int N32 = n * kCatP, NN = n * n;
    double *sL = csm, *sR = csm + N32, *sEL = csm + 2 * N32, *sER = sEL + NN, *sU = sER + NN;
    const double invar = P.invar[p];
    const long long CNN = (long long)C * n * n;
    const long long SB = (long long)(P.state_unknown + 1) * B;
    for (int t = threadIdx.x; t < NN; t += blockDim.x) sU[t] = P.inv_evec[(long long)(c / P.cpc) * NN + t];
    for (int k = 0; k < P.nops; ++k) {
        const OpDev op = P.ops[k];
        int lref = op.child[0], rref = op.child[1];
        const double *eL = P.opmats + op.mat_off, *eR = eL + CNN;
        const double *tL = eL + 2 * CNN, *tR = tL + SB;
        if (lref >= 0 && rref < 0) {  // put the tip on the left (tree/phylokernelnew.h:1390-1400)
            int t = lref; lref = rref; rref = t;
            const double *q = eL; eL = eR; eR = q;
            q = tL; tL = tR; tR = q;
        }
        const bool lint = lref >= 0, rint = rref >= 0;
        __syncthreads();  // the previous op's readers of the shared arrays are done
        for (int j = 0; j < kCatPer; j++) {
            const int x = w + j * kCatWarps;
            if (x >= n) break;
            const long long r = (long long)(c * n + x) * ld + p;
            if (lint) sL[x * kCatP + lane] = P.partials[(long long)lref * P.slot_stride + r];
            if (rint) sR[x * kCatP + lane] = P.partials[(long long)rref * P.slot_stride + r];
        }
        for (int t = threadIdx.x; t < NN; t += blockDim.x) {
            if (lint) sEL[t] = __ldg(eL + (long long)c * NN + t);
            if (rint) sER[t] = __ldg(eR + (long long)c * NN + t);
        }
        __syncthreads();
        const double *tl = lint ? nullptr : tL + (long long)P.states[(long long)(-1 - lref) * ld + p] * B + c * n;
        const double *tr = rint ? nullptr : tR + (long long)P.states[(long long)(-1 - rref) * ld + p] * B + c * n;
        double v[kCatPer];
#pragma unroll
        for (int j = 0; j < kCatPer; j++) {
            const int x = w + j * kCatWarps;
            v[j] = 0.0;
            if (x >= n) continue;
            const double yl = lint ? dot_seq(sEL + x * n, sL + lane, n) : __ldg(tl + x);
            const double yr = rint ? dot_seq(sER + x * n, sR + lane, n) : __ldg(tr + x);
            v[j] = yl * yr;
        }
        __syncthreads();  // every read of the children's entries is done: sL takes the products
#pragma unroll
        for (int j = 0; j < kCatPer; j++) {
            const int x = w + j * kCatWarps;
            if (x < n) sL[x * kCatP + lane] = v[j];
        }
        __syncthreads();
        double m = 0.0;
#pragma unroll
        for (int j = 0; j < kCatPer; j++) {
            const int x = w + j * kCatWarps;
            if (x >= n) continue;
            v[j] = dot_seq(sU + x * n, sL + lane, n);
            m = fmax(m, fabs(v[j]));
        }
        scm[w][lane] = m;
        __syncthreads();
        double cmax = 0.0;  // the category's largest |entry| for this pattern
        for (int ww = 0; ww < kCatWarps; ww++) cmax = fmax(cmax, scm[ww][lane]);
        const bool check = (lint || rint) && invar == 0.0;  // tip-tip never scales
        const bool scaled = check && cmax < kScaleThreshold;
        double *dad = P.partials + (long long)op.dad_slot * P.slot_stride + p;
#pragma unroll
        for (int j = 0; j < kCatPer; j++) {
            const int x = w + j * kCatWarps;
            if (x < n) dad[(long long)(c * n + x) * ld] = scaled ? v[j] * kTwoPow256 : v[j];
        }
        if (w == 0) {  // this category's scale count: the children's (uint8 sum) plus this op's
            unsigned sc = 0;
            if (lint) sc += P.scale[(long long)lref * P.scale_stride + (long long)c * ld + p];
            if (rint) sc += P.scale[(long long)rref * P.scale_stride + (long long)c * ld + p];
            P.scale[(long long)op.dad_slot * P.scale_stride + (long long)c * ld + p] = (uint8_t)(sc + (scaled ? 1u : 0u));
        }
    }
}

// ---------------------------------------------------------------------------
// non-reversible models on the FP64 path (tree/phylokernelnonrev.h): the
// partials stay in the standard basis. echild is P(r_c t) itself (P^T for a
// child reached against the edge direction) and the traversal runs with
// U^-1 = I, so k_traverse_f64 computes the reference's nonrev update,
// dad[x] = (P_L L)[x] (P_R R)[x], with its 2^-256 scaling rule unchanged.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_partial_info_nonrev64(const OpDev *__restrict__ ops,
                                                               double *__restrict__ opmats,
                                                               const double *__restrict__ nr,
                                                               const double *__restrict__ rates, int n, int C, int S) {
    extern __shared__ double nv64[];  // [n*n] P, [2n] exp scratch
    const int k = blockIdx.x, ch = blockIdx.y, c = blockIdx.z;
    const OpDev op = ops[k];
    const NonrevModel m = nonrev_model(nr, n, S);
    double *Pd = nv64, *ex = nv64 + n * n;
    nonrev_matrix(m, n, rates[c], op.len[ch], 0, ex, Pd);
    const bool tr = (op.flags >> ch) & 1, root = (op.flags >> (2 + ch)) & 1;
    const long long CNN = (long long)C * n * n, B = (long long)n * C;
    double *base = opmats + op.mat_off;
    double *echild = base + ch * CNN + (long long)c * n * n;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int x = t / n, i = t % n;
        echild[t] = tr ? Pd[i * n + x] : Pd[x * n + i];
    }
    if (op.child[ch] >= 0) return;
    double *tab = base + 2 * CNN + (long long)ch * (S + 1) * B;
    for (int t = threadIdx.x; t < (S + 1) * n; t += blockDim.x) {
        const int st = t / n, x = t % n;
        const double *v = root ? m.root : m.tipv + (long long)st * n;
        double acc = 0.0;
        for (int y = 0; y < n; y++) acc = fma(tr ? Pd[y * n + x] : Pd[x * n + y], v[y], acc);
        tab[(long long)st * B + (long long)c * n + x] = acc;
    }
}

// prop_c * (r_c lambda)^k-weighted P(r_c t), k = 0, 1, 2: FP64 [3][C][n][n]
__global__ void __launch_bounds__(256) k_nonrev_branch_mats64(double *__restrict__ out, const double *__restrict__ nr,
                                                              const double *__restrict__ rates,
                                                              const double *__restrict__ props, double len, int n,
                                                              int C, int S) {
    extern __shared__ double nv64[];
    const int c = blockIdx.x, k = blockIdx.y;
    double *Pd = nv64, *ex = nv64 + n * n;
    nonrev_matrix(nonrev_model(nr, n, S), n, rates[c], len, k, ex, Pd);
    double *o = out + ((long long)k * C + c) * n * n;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) o[t] = props[c] * Pd[t];
}

// Branch lnL (and with DERV the Newton-Raphson sums) of a non-reversible model
// from the two ends' FP64 partials: lh_k = sum_c sum_x w_x a[c][x] (M_k,c b_c)[x]
// (tree/phylokernelnonrev.h:586-1056, 1062-1528), a the dad side, w the state
// frequencies (unrooted) or ones (rooted); the scale counts as the reversible
// branch lnL treats them (SAFE: categories one count above the minimum scaled
// by 2^-256, more than one zeroed; NORM: the two ends' counts add).
template <bool SAFE, bool DERV>
__global__ void __launch_bounds__(kTPB) k_branch_nonrev64(const TravParams P, const double *__restrict__ mats,
                                                          const double *__restrict__ tipv,
                                                          const double *__restrict__ w) {
    const int n = P.n, C = P.ncat;
    const long long ld = P.ldp, CNN = (long long)C * n * n;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double v[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
    if (p < P.nptn) {
        const double *pa = P.partials + (long long)P.a * P.slot_stride + p;
        const uint8_t *sa = P.scale + (long long)P.a * P.scale_stride + p;
        const bool btip = P.b < 0;
        const double *pb = btip ? nullptr : P.partials + (long long)P.b * P.slot_stride + p;
        const uint8_t *sb = btip ? nullptr : P.scale + (long long)P.b * P.scale_stride + p;
        const int sbst = btip ? P.states[(long long)(-1 - P.b) * ld + p] : 0;
        double l0[kMaxCat], l1[kMaxCat], l2[kMaxCat];
        for (int c = 0; c < C; c++) {
            double bv[kMaxStates];
            for (int y = 0; y < n; y++) bv[y] = btip ? tipv[(long long)sbst * n + y] : pb[(long long)(c * n + y) * ld];
            double h0 = 0.0, h1 = 0.0, h2 = 0.0;
            for (int x = 0; x < n; x++) {
                const double *m0 = mats + ((long long)c * n + x) * n;
                double w0 = 0.0, w1 = 0.0, w2 = 0.0;
                for (int y = 0; y < n; y++) {
                    w0 = fma(__ldg(m0 + y), bv[y], w0);
                    if (DERV) {
                        w1 = fma(__ldg(m0 + CNN + y), bv[y], w1);
                        w2 = fma(__ldg(m0 + 2 * CNN + y), bv[y], w2);
                    }
                }
                const double av = __ldg(w + x) * pa[(long long)(c * n + x) * ld];
                h0 = fma(av, w0, h0);
                if (DERV) {
                    h1 = fma(av, w1, h1);
                    h2 = fma(av, w2, h2);
                }
            }
            l0[c] = h0;
            l1[c] = h1;
            l2[c] = h2;
        }
        double scale_count, lh = 0.0, d1 = 0.0, d2 = 0.0;
        if (SAFE) {
            unsigned sum[kMaxCat], mn = 1u << 30;
            for (int c = 0; c < C; c++) {
                sum[c] = ((unsigned)sa[c * ld] + (btip ? 0u : (unsigned)sb[c * ld])) & 0xffu;
                mn = min(mn, sum[c]);
            }
            for (int c = 0; c < C; c++) {
                const double f = sum[c] == mn ? 1.0 : sum[c] == mn + 1 ? kScaleThreshold : 0.0;
                lh += l0[c] * f;
                d1 += l1[c] * f;
                d2 += l2[c] * f;
            }
            scale_count = (double)mn;
        } else {
            for (int c = 0; c < C; c++) {
                lh += l0[c];
                d1 += l1[c];
                d2 += l2[c];
            }
            scale_count = (double)((unsigned)sa[0] + (btip ? 0u : (unsigned)sb[0]));
        }
        lh = fabs(lh) + P.invar[p];
        const double plh = log(lh) + scale_count * kLogScaleThreshold;
        const double f = P.freq[p];
        if (DERV) {
            const double df_frac = d1 / lh, ddf_frac = d2 / lh;
            const double tmp1 = df_frac * f, tmp2 = ddf_frac * f;
            v[0] = tmp1;
            v[1] = fma(-tmp1, df_frac, tmp2);
            v[2] = plh * f;
        } else {
            P.pattern_lh[p] = plh;
            v[0] = plh * f;
            v[1] = (isfinite(plh) ? plh : 4.0 * kLogScaleThreshold) * f;
            v[2] = isfinite(plh) ? 0.0 : 1.0;
        }
    }
    grid_reduce(v, P.red);
}

// ---------------------------------------------------------------------------
// derivatives and lnL from the theta buffer
// ---------------------------------------------------------------------------
struct BufParams {
    int n, ncat, nptn;
    int tail_dup;  // IQGPU_FLAG_REF_TRIPLE_TAIL with odd n and even n*ncat
    long long ldp;
    const double *theta, *buffer_scale, *freq, *invar;
    const double *eval, *rates, *props;
    int cpc;  // categories per mixture class (eval is [class][n])
    double len;
    double *pattern_lh;
    Reduce red;
    int asc_first;    // +ASC: patterns from here on are the unobserved constant ones (nptn: none)
    double *asc_out;  // their (lh, df, ddf), unscaled once as the reference does
};

// (tree/phylokernelnew.h:2233-2633): df = sum freq*d1/lh, ddf = sum freq*(d2/lh - (d1/lh)^2)
__global__ void __launch_bounds__(kTPB) k_derv_f64(const BufParams P) {
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
        const double *th = P.theta + p;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, b0 = 0.0, b1 = 0.0, b2 = 0.0;
        int k = 0;
        for (; k + 1 < B; k += 2) {
            const double t0 = th[(long long)k * P.ldp], t1 = th[(long long)(k + 1) * P.ldp];
            a0 = fma(v0[k], t0, a0); a1 = fma(v1[k], t0, a1); a2 = fma(v2[k], t0, a2);
            b0 = fma(v0[k + 1], t1, b0); b1 = fma(v1[k + 1], t1, b1); b2 = fma(v2[k + 1], t1, b2);
        }
        if (k < B) {
            const double t0 = th[(long long)k * P.ldp];
            a0 = fma(v0[k], t0, a0); a1 = fma(v1[k], t0, a1); a2 = fma(v2[k], t0, a2);
        }
        if (P.tail_dup) {  // the reference's odd-state tail, added a second time
            const double t0 = th[(long long)(B - 1) * P.ldp];
            a0 = fma(v0[B - 1], t0, a0); a1 = fma(v1[B - 1], t0, a1); a2 = fma(v2[B - 1], t0, a2);
        }
        double lh = a0 + b0, d1 = a1 + b1, d2 = a2 + b2;
        lh = fabs(lh) + P.invar[p];
        if (p >= P.asc_first) {  // +ASC constant pattern (tree/phylokernelnew.h:2506-2546); weight 0 below
            const double u = P.buffer_scale[p] != 0.0 ? kScaleThreshold : 1.0;
            double *o = P.asc_out + 3 * (p - P.asc_first);
            o[0] = lh * u;
            o[1] = d1 * u;
            o[2] = d2 * u;
        }
        const double inv = 1.0 / lh;
        const double df_frac = d1 * inv, ddf_frac = d2 * inv;
        const double f = P.freq[p];
        const double tmp1 = df_frac * f, tmp2 = ddf_frac * f;
        r[0] = tmp1;
        r[1] = fma(-tmp1, df_frac, tmp2);
        r[2] = (log(lh) + P.buffer_scale[p]) * f;  // lnL at this length, for free
    }
    grid_reduce(r, P.red);
}

// ---------------------------------------------------------------------------
// Optimization::minimizeNewton (utils/optimization.cpp:422-499) over
// computeFuncDerv (tree/phylotree.cpp:2529-2536) on the device, for pattern
// counts a few SMs cover: one thread-block cluster of up to 8 CTAs. Every
// step, each CTA sums the per-pattern derivative terms of k_derv_f64 over its
// interleaved share of the resident theta buffer and reduces them in a fixed
// order; a cluster barrier publishes the CTA sums (double-buffered by step
// parity in shared memory), and every thread adds them from distributed
// shared memory in rank order. All threads of all CTAs then hold the same f
// and df and take the same safeguarded step, so a branch costs one launch and
// one host wait instead of one of each per step. (GB300 issues a few FP64
// FMAs per clock per SM, so the CTAs take contiguous chunks of the patterns:
// one CTA alone would take ~10 us per step on 600 DNA patterns.)
// out: {optx, status + 16 * steps, d2l, last evaluated length}; status 0 ok,
// 1 non-finite NORM derivative, 2 the reference's "Wrong computeFuncDerv",
// 3 too many iterations.
// ---------------------------------------------------------------------------
constexpr int kNewtonThreads = 256;    // largest CTA (sizes the warp-sum array)
constexpr int kNewtonMaxCluster = 16;  // a non-portable cluster size; 8 where 16 cannot be placed
constexpr int kNewtonBlock = 128;       // threads per CTA
constexpr size_t kNewtonCacheBytes = 160 * 1024;  // dynamic shared memory for a CTA's theta rows

__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ double2 ld_dsmem_f64x2(const double2 *local, unsigned rank) {
    unsigned addr = (unsigned)__cvta_generic_to_shared(local), raddr;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(raddr) : "r"(addr), "r"(rank));
    double2 v;
    asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(raddr) : "memory");
    return v;
}

// cache (optional): this CTA's theta rows [B][chunk], then its patterns'
// frequencies and invariant-site terms [chunk] each, loaded once per solve
// scof, sprop: lambda_i r_c and the category weights, read once per solve
__device__ void newton_derv(const BufParams &P, double len, double *v0, double *v1, double *v2, double *red,
                            double2 *part, int step, unsigned rank, unsigned nrank, bool safe, double *f, double *df,
                            const double *cache, const double *scof, const double *sprop, long long chunk) {
    const int n = P.n, C = P.ncat, B = n * C, tid = threadIdx.x;
    __syncthreads();  // this CTA's readers of v0..v2 and red for the previous step are done
    for (int t = tid; t < B; t += blockDim.x) {
        const double cof = scof[t];
        const double val = exp(cof * len) * sprop[t / n];
        const double val1 = cof * val;
        v0[t] = val;
        v1[t] = val1;
        v2[t] = cof * val1;
    }
    __syncthreads();
    double s1 = 0.0, s2 = 0.0;
    // CTA `rank` takes the contiguous patterns [rank * chunk, (rank + 1) * chunk)
    const long long p_end = min((long long)P.nptn, (long long)(rank + 1) * chunk);
    const long long p0 = rank * chunk;
    const long long ldt = cache ? chunk : P.ldp;
    for (long long p = p0 + tid; p < p_end; p += blockDim.x) {
        const double *th = cache ? cache + (p - p0) : P.theta + p;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, b0 = 0.0, b1 = 0.0, b2 = 0.0;
        int k = 0;
        for (; k + 1 < B; k += 2) {
            const double t0 = th[(long long)k * ldt], t1 = th[(long long)(k + 1) * ldt];
            a0 = fma(v0[k], t0, a0); a1 = fma(v1[k], t0, a1); a2 = fma(v2[k], t0, a2);
            b0 = fma(v0[k + 1], t1, b0); b1 = fma(v1[k + 1], t1, b1); b2 = fma(v2[k + 1], t1, b2);
        }
        if (k < B) {
            const double t0 = th[(long long)k * ldt];
            a0 = fma(v0[k], t0, a0); a1 = fma(v1[k], t0, a1); a2 = fma(v2[k], t0, a2);
        }
        if (P.tail_dup) {
            const double t0 = th[(long long)(B - 1) * ldt];
            a0 = fma(v0[B - 1], t0, a0); a1 = fma(v1[B - 1], t0, a1); a2 = fma(v2[B - 1], t0, a2);
        }
        const double lh = fabs(a0 + b0) + (cache ? cache[(B + 1) * chunk + (p - p0)] : P.invar[p]);
        const double inv = 1.0 / lh;
        const double df_frac = (a1 + b1) * inv, ddf_frac = (a2 + b2) * inv;
        const double fq = cache ? cache[B * chunk + (p - p0)] : P.freq[p];
        const double tmp1 = df_frac * fq, tmp2 = ddf_frac * fq;
        s1 += tmp1;
        s2 += fma(-tmp1, df_frac, tmp2);
    }
    // fixed-order reduction: warps by shuffles, warp sums in order, CTA sums in rank order
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, off);
        s2 += __shfl_xor_sync(0xffffffffu, s2, off);
    }
    if ((tid & 31) == 0) {
        red[2 * (tid >> 5)] = s1;
        red[2 * (tid >> 5) + 1] = s2;
    }
    __syncthreads();
    if (tid == 0) {
        double t1 = 0.0, t2 = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            t1 += red[2 * w];
            t2 += red[2 * w + 1];
        }
        part[step & 1] = make_double2(t1, t2);
    }
    // publishes part[step & 1] of every CTA; part[(step + 1) & 1] is rewritten
    // only after the next barrier, which every CTA reaches after reading this one
    cluster_sync_all();
    double2 v[kNewtonMaxCluster];  // every CTA's sums requested at once, then added in rank order
#pragma unroll
    for (unsigned q = 0; q < kNewtonMaxCluster; q++)
        if (q < nrank) v[q] = ld_dsmem_f64x2(part + (step & 1), q);
    double t1 = 0.0, t2 = 0.0;
#pragma unroll
    for (unsigned q = 0; q < kNewtonMaxCluster; q++)
        if (q < nrank) {
            t1 += v[q].x;
            t2 += v[q].y;
        }
    if (!isfinite(t1) && safe) t1 = t2 = 0.0;  // tree/phylokernelnew.h:2629-2632
    *f = -t1;  // computeFuncDerv returns the negated sums
    *df = -t2;
}

// xg_dev (optional) holds the start length in device memory; len_out
// (optional) takes the optimum when the solve succeeded (status 0)
__global__ void __launch_bounds__(kNewtonThreads, 1) k_newton_f64(const BufParams P, double x1, double xguess,
                                                                double x2, double xacc, int max_steps, int safe,
                                                                double *out, const double *xg_dev,
                                                                double *len_out, int cached, long long chunk) {
    pdl_wait();  // theta and the start length come from the kernels before
    pdl_trigger();
    extern __shared__ double newton_cache[];
    __shared__ double scof[kMaxCat * kMaxStates], sprop[kMaxCat];
    __shared__ double v0[kMaxCat * kMaxStates], v1[kMaxCat * kMaxStates], v2[kMaxCat * kMaxStates];
    __shared__ double red[2 * (kNewtonThreads / 32)];
    __shared__ double2 part[2];
    unsigned rank, nrank;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(nrank));
    double f, df, dx, temp, xh, xl, rts, rts_old, xlast;
    int status = 0, steps = 0, step = 0;
    for (int t = threadIdx.x; t < P.n * P.ncat; t += blockDim.x) {
        const int c = t / P.n, i = t % P.n;
        scof[t] = P.eval[(c / P.cpc) * P.n + i] * P.rates[c];
        if (i == 0) sprop[c] = P.props[c];
    }
    const double *cache = nullptr;
    if (cached) {  // this CTA's patterns, as newton_derv splits them, read once for every step
        const int B = P.n * P.ncat;
        const long long p0 = rank * chunk;
        for (long long i = threadIdx.x; i < (B + 2) * chunk; i += blockDim.x) {
            const long long k = i / chunk, p = p0 + i % chunk;
            double v = 0.0;
            if (p < P.nptn) v = k < B ? P.theta[k * P.ldp + p] : (k == B ? P.freq[p] : P.invar[p]);
            newton_cache[i] = v;
        }
        cache = newton_cache;  // newton_derv's first barrier orders these stores before the reads
    }
    rts = xg_dev ? *xg_dev : xguess;
    if (rts < x1) rts = x1;
    if (rts > x2) rts = x2;
    xlast = rts;
    newton_derv(P, rts, v0, v1, v2, red, part, step++, rank, nrank, safe != 0, &f, &df, cache, scof, sprop, chunk);
    if (!isfinite(f)) status = safe ? 2 : 1;
    else if (!isfinite(df)) status = 2;
    else if (!(df >= 0.0 && fabs(f) < xacc)) {
        if (f < 0.0) { xl = rts; xh = x2; } else { xh = rts; xl = x1; }
        dx = fabs(xh - xl);
        status = 3;
        for (int j = 1; j <= max_steps; j++) {
            steps = j;
            rts_old = rts;
            if ((df <= 0.0) || (((rts - xh) * df - f) * ((rts - xl) * df - f) >= 0.0)) {
                dx = 0.5 * (xh - xl);
                rts = xl + dx;
                if (xl == rts) { status = 0; break; }
            } else {
                dx = f / df;
                temp = rts;
                rts -= dx;
                if (temp == rts) { status = 0; break; }
            }
            if (fabs(dx) < xacc || (j == max_steps)) { rts = rts_old; status = 0; break; }
            xlast = rts;
            newton_derv(P, rts, v0, v1, v2, red, part, step++, rank, nrank, safe != 0, &f, &df, cache, scof, sprop, chunk);
            if (!isfinite(f)) { status = safe ? 2 : 1; break; }
            if (!isfinite(df)) { status = 2; break; }
            if (df > 0.0 && fabs(f) < xacc) { status = 0; break; }
            if (f < 0.0) xl = rts;
            else if (f > 0.0) xh = rts;
        }
    }
    if (rank == 0 && threadIdx.x == 0) {
        out[0] = rts;
        out[1] = (double)(status + 16 * steps);
        out[2] = df;  // d2l: minimizeNewton leaves it at the latest df
        out[3] = xlast;
        // every CTA read *xg_dev before its first cluster barrier, which this one passed
        if (len_out && status == 0) *len_out = rts;
    }
    cluster_sync_all();  // no CTA leaves while another may still read its shared memory
}

// (tree/phylokernelnew.h:3232-3428)
__global__ void __launch_bounds__(kTPB) k_from_buffer_f64(const BufParams P) {
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
        const double *th = P.theta + p;
        double a0 = 0.0, a1 = 0.0;
        int k = 0;
        for (; k + 1 < B; k += 2) {
            a0 = fma(v0[k], th[(long long)k * P.ldp], a0);
            a1 = fma(v0[k + 1], th[(long long)(k + 1) * P.ldp], a1);
        }
        if (k < B) a0 = fma(v0[k], th[(long long)k * P.ldp], a0);
        double lh = fabs(a0 + a1) + P.invar[p];
        const double plh = log(fabs(lh)) + P.buffer_scale[p];
        P.pattern_lh[p] = plh;
        const double f = P.freq[p];
        r[0] = plh * f;
        r[1] = (isfinite(plh) ? plh : 4.0 * kLogScaleThreshold) * f;
        r[2] = isfinite(plh) ? 0.0 : 1.0;
    }
    grid_reduce(r, P.red);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static TravParams trav_params(iqgpu_engine *e, int nops) {
    TravParams P;
    P.n = e->n;
    P.ncat = e->C;
    P.state_unknown = e->S;
    P.nops = nops;
    P.nptn = (int)e->P;
    P.ldp = e->Ppad;
    P.slot_stride = (long long)e->B * e->Ppad;
    P.scale_stride = (long long)(e->cfg.safe ? e->C : 1) * e->Ppad;
    P.op_stride = e->op_stride;
    P.ops = e->d_ops;
    P.opmats = e->d_opmats;
    P.inv_evec = e->d_inv;
    P.eval = e->d_eval;
    P.rates = e->d_rates;
    P.props = e->d_props;
    P.tip_lh = e->d_tip;
    P.nmix = e->nmix;
    P.cpc = e->cpc;
    P.freq = e->d_freq;
    P.invar = e->d_invar;
    P.states = e->d_states;
    P.partials = e->d_part;
    P.scale = e->d_scale;
    P.a = P.b = 0;
    P.len = 0.0;
    P.cat_split = 0;
    P.pattern_lh = e->d_plh;
    P.theta = e->d_theta;
    P.buffer_scale = e->d_bscale;
    P.red.partials = e->d_red_partials;
    P.red.ticket = e->d_ticket;
    P.red.out = e->d_red_out;
    return P;
}

int launch_partial_info_f64(iqgpu_engine *e, int nops, const OpDev *src, const int32_t *edge, const double *len) {
    if (nops <= 0) return IQGPU_OK;
    if (e->nonrev) {
        const size_t smem = ((size_t)e->n * e->n + 2 * e->n) * 8;
        k_partial_info_nonrev64<<<dim3(nops, 2, e->C), 256, smem, e->st>>>(e->d_ops, e->d_opmats, e->d_nr, e->d_rates,
                                                                          e->n, e->C, e->S);
        e->launches++;
        return cuda_fail(cudaGetLastError(), "partial_info_nonrev64");
    }
    dim3 grid(nops, 2, e->n > 20 ? 16 : 2);
    cudaError_t err = pdl_launch(k_partial_info_f64, grid, dim3(256), 0, e->st, e->d_ops, e->d_opmats,
                                 (const double *)e->d_evec, (const double *)e->d_eval, (const double *)e->d_rates,
                                 (const double *)e->d_tip, e->n, e->C, e->S, e->nmix, e->cpc,
                                 PassStage{src, edge, len});
    e->launches++;
    if (err != cudaSuccess) return cuda_fail(err, "partial_info_f64");
    return cuda_fail(cudaGetLastError(), "partial_info_f64");
}

// Patterns per CTA of the FP64 pattern-tile kernels: 128, or one warp's 32
// when 128-pattern tiles would leave most SMs idle (short alignments: GB300
// issues only a few FP64 FMAs per clock per SM, so these kernels run at the
// FP64 rate of the SMs they occupy). Per-pattern arithmetic is the same; the
// grid reduction groups the CTA sums differently.
static int f64_tpb(const iqgpu_engine *e) { return e->nblk < e->sms ? 32 : kTPB; }

template <int NT, bool SAFE, int EPI>
static int launch_trav_t(iqgpu_engine *e, const TravParams &P) {
    const int tpb = f64_tpb(e);
    const dim3 grid((unsigned)(e->Ppad / tpb), P.cat_split ? e->C : 1);
    constexpr bool REG = (NT != 0 && NT <= 20);
    size_t smem = (REG ? 0 : (size_t)kMaxStates * tpb * sizeof(double)) +
                  (EPI == EPI_LNL ? (size_t)kMaxCat * kMaxStates * sizeof(double) : 0);
    auto kern = k_traverse_f64<NT, SAFE, EPI>;
    if (smem > 0) {  // static arrays count against the 48 KB default too
        cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return cuda_fail(err, "traverse_f64 smem attribute");
    }
    kern<<<grid, tpb, smem, e->st>>>(P);
    e->launches++;
    return cuda_fail(cudaGetLastError(), "traverse_f64");
}

// 4-state models on short alignments: the lane kernel (see above)
template <bool SAFE, int EPI, int G>
static int launch_lanes_t(iqgpu_engine *e, const TravParams &P) {
    cudaError_t err =
        pdl_launch(k_traverse_f64_lanes<SAFE, EPI, G>, dim3((unsigned)(e->Ppad * G / 128)), dim3(128), 0, e->st, P);
    e->launches++;
    if (err != cudaSuccess) return cuda_fail(err, "traverse_f64_lanes");
    return cuda_fail(cudaGetLastError(), "traverse_f64_lanes");
}

// (at full size, 87,306 DNA patterns, the lane kernel measured 16.1 ms per
// evaluation against 13.7 ms for the pattern kernel: it is for short alignments)
static bool use_lanes(const iqgpu_engine *e, const TravParams &P) {
    return e->n == 4 && e->C <= 8 && !e->nonrev && !e->has_multi && !P.cat_split && e->nblk < e->sms;
}

// 20-state models: the wide kernel (see above)
template <bool SAFE, int EPI>
static int launch_wide_t(iqgpu_engine *e, const TravParams &P) {
    const size_t smem = ((size_t)2 * e->C * kWideN * kWideP + (size_t)3 * e->C * kWideN * kWideN) * sizeof(double);
    auto kern = k_traverse_f64_wide<SAFE, EPI>;
    // (always: with its static arrays even 2 categories pass the 48 KB default)
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return cuda_fail(err, "traverse_f64_wide smem attribute");
    kern<<<(unsigned)(e->Ppad / kWideP), kWideN * kWideP, smem, e->st>>>(P);
    e->launches++;
    return cuda_fail(cudaGetLastError(), "traverse_f64_wide");
}

static bool use_wide(const iqgpu_engine *e, const TravParams &P) {
    return e->n == kWideN && e->C <= kWideMaxCat && !e->nonrev && !e->has_multi && !P.cat_split;
}

template <bool SAFE, int EPI>
static int dispatch_n(iqgpu_engine *e, const TravParams &P) {
    if (use_wide(e, P)) return launch_wide_t<SAFE, EPI>(e, P);
    if (use_lanes(e, P)) {
        switch (e->C) {
        case 1: return launch_lanes_t<SAFE, EPI, 4>(e, P);
        case 2: return launch_lanes_t<SAFE, EPI, 8>(e, P);
        case 3: case 4: return launch_lanes_t<SAFE, EPI, 16>(e, P);
        default: return launch_lanes_t<SAFE, EPI, 32>(e, P);
        }
    }
    switch (e->n) {
    case 4: return launch_trav_t<4, SAFE, EPI>(e, P);
    case 20: return launch_trav_t<20, SAFE, EPI>(e, P);
    default: return launch_trav_t<0, SAFE, EPI>(e, P);
    }
}

template <int EPI>
static int dispatch_safe(iqgpu_engine *e, const TravParams &P) {
    return e->cfg.safe ? dispatch_n<true, EPI>(e, P) : dispatch_n<false, EPI>(e, P);
}

int launch_traverse_f64(iqgpu_engine *e, int nops, int epi, int32_t a, int32_t b, double len) {
    TravParams P = trav_params(e, nops);
    P.a = a;
    P.b = b;
    P.len = len;
    if (nops == 0 && epi == EPI_NONE) return IQGPU_OK;
    // SAFE op walks over too few pattern tiles to fill the GPU (codon, short
    // alignments): one CTA per (tile, category), then the epilogue on its own
    // Large state counts in SAFE: the per-category kernel for the walk, any size
    if (e->cfg.safe && !e->nonrev && !e->has_multi && nops > 0 && e->n > 20 && e->n <= kCatMaxN) {
        const size_t smem = ((size_t)2 * e->n * kCatP + (size_t)3 * e->n * e->n) * sizeof(double);
        cudaError_t err = cudaFuncSetAttribute(k_traverse_f64_cat, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem);
        if (err != cudaSuccess) return cuda_fail(err, "traverse_f64_cat smem attribute");
        k_traverse_f64_cat<<<dim3((unsigned)(e->Ppad / kCatP), e->C), kCatWarps * kCatP, smem, e->st>>>(P);
        e->launches++;
        if ((err = cudaGetLastError()) != cudaSuccess) return cuda_fail(err, "traverse_f64_cat");
        if (epi == EPI_NONE) return IQGPU_OK;
        P.nops = 0;
    } else if (e->cfg.safe && !e->nonrev && !e->has_multi && nops > 0 && e->C > 1 && e->nblk < 2 * e->sms) {
        P.cat_split = 1;
        int rc = dispatch_safe<EPI_NONE>(e, P);
        if (rc || epi == EPI_NONE) return rc;
        P.cat_split = 0;
        P.nops = 0;
    }
    switch (epi) {
    case EPI_NONE: return dispatch_safe<EPI_NONE>(e, P);
    case EPI_LNL: return dispatch_safe<EPI_LNL>(e, P);
    default: return dispatch_safe<EPI_THETA>(e, P);
    }
}

static BufParams buf_params(iqgpu_engine *e, double len) {
    BufParams P;
    P.n = e->n;
    P.ncat = e->C;
    P.nptn = (int)e->P;
    P.tail_dup = (e->cfg.flags & IQGPU_FLAG_REF_TRIPLE_TAIL) && (e->n & 1) && ((e->n * e->C) % 2 == 0);
    P.ldp = e->Ppad;
    P.theta = e->d_theta;
    P.buffer_scale = e->d_bscale;
    P.freq = e->d_freq;
    P.invar = e->d_invar;
    P.eval = e->d_eval;
    P.cpc = e->cpc;
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

int launch_newton_f64(iqgpu_engine *e, double x1, double xguess, double x2, double xacc, int max_steps,
                      double *out_dev, const double *xg_dev, double *len_out) {
    // Per SM GB300 issues only a few FP64 FMAs per clock, so the solve spreads
    // the patterns over one cluster of up to 16 CTAs (one per 32 patterns),
    // each a contiguous chunk, with the CTA's theta rows, frequencies and
    // invariant terms in shared memory when they fit.
    static int cluster_max[64] = {};  // per device: 16 or 8, once probed
    const int dv = e->dev >= 0 && e->dev < 64 ? e->dev : 0;
    if (!cluster_max[dv]) {
        cudaError_t err = cudaFuncSetAttribute(k_newton_f64, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)kNewtonCacheBytes);
        if (err != cudaSuccess) return cuda_fail(err, "newton_f64 smem attribute");
        cluster_max[dv] = 8;
        if (cudaFuncSetAttribute(k_newton_f64, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
            cudaLaunchConfig_t probe = {};
            probe.gridDim = dim3(kNewtonMaxCluster);
            probe.blockDim = dim3(kNewtonBlock);
            probe.dynamicSmemBytes = kNewtonCacheBytes;
            cudaLaunchAttribute pa[1];
            pa[0].id = cudaLaunchAttributeClusterDimension;
            pa[0].val.clusterDim.x = kNewtonMaxCluster;
            pa[0].val.clusterDim.y = 1;
            pa[0].val.clusterDim.z = 1;
            probe.attrs = pa;
            probe.numAttrs = 1;
            int nc = 0;
            if (cudaOccupancyMaxActiveClusters(&nc, k_newton_f64, &probe) == cudaSuccess && nc >= 1)
                cluster_max[dv] = kNewtonMaxCluster;
        }
        cudaGetLastError();  // a refused probe leaves no error behind
    }
    const int q = (int)std::min<long long>(cluster_max[dv], std::max<long long>(1, (e->P + 31) / 32));
    const long long chunk = (e->P + q - 1) / q;
    const size_t cache_bytes = (size_t)(e->n * e->C + 2) * chunk * sizeof(double);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)q);
    cfg.blockDim = dim3(kNewtonBlock);
    cfg.dynamicSmemBytes = cache_bytes <= kNewtonCacheBytes ? cache_bytes : 0;
    cfg.stream = e->st;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)q;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;  // a dependent launch (pdl_wait)
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    const BufParams P = buf_params(e, 0.0);
    const int safe = e->cfg.safe ? 1 : 0;
    const int cached = cfg.dynamicSmemBytes > 0 ? 1 : 0;
    cudaError_t err = cudaLaunchKernelEx(&cfg, k_newton_f64, P, x1, xguess, x2, xacc, max_steps, safe, out_dev, xg_dev,
                                         len_out, cached, chunk);
    e->launches++;
    if (err != cudaSuccess) return cuda_fail(err, "newton_f64");
    return cuda_fail(cudaGetLastError(), "newton_f64");
}

int launch_derv_f64(iqgpu_engine *e, double len) {
    k_derv_f64<<<(unsigned)(e->Ppad / f64_tpb(e)), f64_tpb(e), 0, e->st>>>(buf_params(e, len));
    e->launches++;
    return cuda_fail(cudaGetLastError(), "derv_f64");
}

int launch_from_buffer_f64(iqgpu_engine *e, double len) {
    k_from_buffer_f64<<<(unsigned)(e->Ppad / f64_tpb(e)), f64_tpb(e), 0, e->st>>>(buf_params(e, len));
    e->launches++;
    return cuda_fail(cudaGetLastError(), "from_buffer_f64");
}

int launch_branch_nonrev64(iqgpu_engine *e, double len, bool derv) {
    const size_t smem = ((size_t)e->n * e->n + 2 * e->n) * 8;
    double *mats = reinterpret_cast<double *>(e->d_nrmats);
    k_nonrev_branch_mats64<<<dim3(e->C, derv ? 3 : 1), 256, smem, e->st>>>(mats, e->d_nr, e->d_rates, e->d_props, len,
                                                                          e->n, e->C, e->S);
    e->launches++;
    int rc = cuda_fail(cudaGetLastError(), "nonrev_branch_mats64");
    if (rc) return rc;
    TravParams P = trav_params(e, 0);
    P.a = e->theta_a;
    P.b = e->theta_b;
    const double *tipv = nonrev_model(e->d_nr, e->n, e->S).tipv;
    if (e->cfg.safe) {
        if (derv) k_branch_nonrev64<true, true><<<e->nblk, kTPB, 0, e->st>>>(P, mats, tipv, e->d_pi);
        else k_branch_nonrev64<true, false><<<e->nblk, kTPB, 0, e->st>>>(P, mats, tipv, e->d_pi);
    } else {
        if (derv) k_branch_nonrev64<false, true><<<e->nblk, kTPB, 0, e->st>>>(P, mats, tipv, e->d_pi);
        else k_branch_nonrev64<false, false><<<e->nblk, kTPB, 0, e->st>>>(P, mats, tipv, e->d_pi);
    }
    e->launches++;
    return cuda_fail(cudaGetLastError(), "branch_nonrev64");
}

}  // namespace iqg
