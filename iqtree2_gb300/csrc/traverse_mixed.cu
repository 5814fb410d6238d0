// Mixed-precision path, part 2: the traversal kernels on CUDA cores.
//
// Thread mapping (both schedules): a CTA owns TP consecutive patterns and runs
// TP*ncat threads; warp w handles 32 patterns of one rate category, so the
// transition-matrix rows it reads are warp-uniform (shared-memory broadcast)
// and its float4 loads of the children are whole 128-byte lines. Each thread
// keeps its category's outputs in registers until the pattern's largest entry
// over all categories is known (one shared-memory max across the category
// warps), then applies the exact power-of-two rescale and stores once.
//
// Two schedules of the same per-op body:
//  * fused: one CTA walks the whole post-order op list for its patterns (a
//    pattern's partials depend only on the same pattern's children), with
//    each op's P(t) blocks staged in shared memory by a TMA bulk copy that
//    runs one op ahead (double buffer). One launch; children are usually still
//    in L2 when their parent reads them; latency per op is exposed.
//  * level-synchronous: ops are grouped by tree level (all ops of a level are
//    independent); one launch per level runs every (op, pattern tile) pair of
//    the level as its own CTA, so many independent ops are in flight per SM.
// The autotuner picks the schedule and the tile per workload.
#include <cuda_runtime.h>

#include <algorithm>

#include "mixed.cuh"

namespace iqg {

// (a0, a1) = (x0 * y0 + a0, x1 * y1 + a1) in one packed FP32 instruction
// (fma.rn.f32x2, sm_100 and later): two IEEE round-to-nearest FMAs, the same
// results as two fmaf calls at half the issue slots.
__device__ __forceinline__ void fma2(float &a0, float &a1, float x0, float x1, float y0, float y1) {
    unsigned long long x, y, a;
    asm("mov.b64 %0, {%1, %2};" : "=l"(x) : "f"(x0), "f"(x1));
    asm("mov.b64 %0, {%1, %2};" : "=l"(y) : "f"(y0), "f"(y1));
    asm("mov.b64 %0, {%1, %2};" : "=l"(a) : "f"(a0), "f"(a1));
    asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(a) : "l"(x), "l"(y));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a0), "=f"(a1) : "l"(a));
}

// Row of P(t) (shared memory) times the child's states: even and odd states
// accumulate separately and are added at the end.
template <int NQ>
__device__ __forceinline__ float row_dot_s(const float *prow, const float4 (&v)[NQ]) {
    float a0 = 0.f, a1 = 0.f;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        const float4 m = *reinterpret_cast<const float4 *>(prow + 4 * q);
        fma2(a0, a1, m.x, m.y, v[q].x, v[q].y);
        fma2(a0, a1, m.z, m.w, v[q].z, v[q].w);
    }
    return a0 + a1;
}

__device__ __forceinline__ float dot4(const float4 a, const float4 b, float acc) {
    return fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, fmaf(a.w, b.w, acc))));
}

// One op for this thread's (pattern, category): sP holds the op's two P(t)
// blocks; smax is this op's [ncat*TP] scratch for the cross-category maximum.
// Contains one __syncthreads (all threads of the CTA must call it).
template <int NQ>
__device__ __forceinline__ void mixed_op(const MixParams &P, int k, const float *sP, float *smax, int c, int pl,
                                         long long p, long long pbase, int TP) {
    constexpr int XC = 16;
    const int n = P.n, npad = P.npad, C = P.ncat, S = P.state_unknown;
    const int nq = NQ ? NQ : npad >> 2;
    const long long ld = P.ldp;
    const long long PM = (long long)C * n * npad;
    const long long TB = (long long)(S + 1) * C * npad;
    const OpDev op = P.ops[k];
    int lref = op.child[0], rref = op.child[1];
    // Multifurcating node (tree/phylokernelnew.h:1407-1631): consecutive records
    // flagged IQGPU_OP_MORE share the dad; a continuation multiplies its
    // children into the dad's running product, each record rescaling it
    // (exact powers of two, exponents accumulate); an odd child count ends
    // with an absent second child.
    const bool cont = k > 0 && (P.ops[k - 1].flags & IQGPU_OP_MORE);
    const bool rnone = rref == IQGPU_NO_CHILD;
    const float *gbase = P.opmats + (long long)k * P.op_stride;
    const float *PL = sP, *PR = sP + PM, *TL = gbase + 2 * PM, *TR = TL + TB;
    if (lref >= 0 && rref < 0 && !rnone) {  // the tip goes on the left (tree/phylokernelnew.h:1390-1400)
        int t = lref; lref = rref; rref = t;
        const float *q = PL; PL = PR; PR = q;
        q = TL; TL = TR; TR = q;
    }
    const bool lint = lref >= 0, rint = rref >= 0;
    float *dad = P.part + (long long)op.dad_slot * P.slot_floats + pbase;
    const float *Lp = lint ? P.part + (long long)lref * P.slot_floats + pbase : nullptr;
    const float *Rp = rint ? P.part + (long long)rref * P.slot_floats + pbase : nullptr;
    const float *tl = lint ? nullptr : TL + (long long)P.states[(long long)(-1 - lref) * ld + p] * C * npad + c * npad;
    const float *tr = (rint || rnone) ? nullptr
                                      : TR + (long long)P.states[(long long)(-1 - rref) * ld + p] * C * npad + c * npad;
    const float *PLc = PL + (long long)c * n * npad, *PRc = PR + (long long)c * n * npad;
    float cmax = 0.f;
    float4 out[NQ ? NQ : 1];
    if constexpr (NQ > 0) {
        float4 lv[NQ], rv[NQ];
        if (lint) {
#pragma unroll
            for (int q = 0; q < NQ; q++) lv[q] = *reinterpret_cast<const float4 *>(Lp + q * 32);
        }
        if (rint) {
#pragma unroll
            for (int q = 0; q < NQ; q++) rv[q] = *reinterpret_cast<const float4 *>(Rp + q * 32);
        }
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            float o[4];
            const float4 d4 = cont ? *reinterpret_cast<const float4 *>(dad + q * 32) : make_float4(1.f, 1.f, 1.f, 1.f);
            const float dv[4] = {d4.x, d4.y, d4.z, d4.w};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int x = 4 * q + j;
                float v = 0.f;
                if (x < n) {
                    const float yl = lint ? row_dot_s<NQ>(PLc + x * npad, lv) : __ldg(tl + x);
                    const float yr = rint ? row_dot_s<NQ>(PRc + x * npad, rv) : (rnone ? 1.f : __ldg(tr + x));
                    v = yl * yr;
                    if (cont) v *= dv[j];
                }
                o[j] = v;
                cmax = fmaxf(cmax, v);
            }
            out[q] = make_float4(o[0], o[1], o[2], o[3]);
        }
    } else {
        for (int x0 = 0; x0 < npad; x0 += XC) {
            float al[XC], ar[XC];
#pragma unroll
            for (int j = 0; j < XC; j++) { al[j] = 0.f; ar[j] = 0.f; }
            for (int q = 0; q < nq; q++) {
                const float4 l4 = lint ? *reinterpret_cast<const float4 *>(Lp + q * 32) : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 r4 = rint ? *reinterpret_cast<const float4 *>(Rp + q * 32) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int j = 0; j < XC; j++) {
                    const int x = x0 + j;
                    if (x < n) {
                        if (lint) al[j] = dot4(*reinterpret_cast<const float4 *>(PLc + x * npad + 4 * q), l4, al[j]);
                        if (rint) ar[j] = dot4(*reinterpret_cast<const float4 *>(PRc + x * npad + 4 * q), r4, ar[j]);
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < XC; j += 4) {
                float o[4];
                float dv[4] = {1.f, 1.f, 1.f, 1.f};
                if (cont && x0 + j < npad) {
                    const float4 d4 = *reinterpret_cast<const float4 *>(dad + ((x0 + j) >> 2) * 32);
                    dv[0] = d4.x; dv[1] = d4.y; dv[2] = d4.z; dv[3] = d4.w;
                }
#pragma unroll
                for (int jj = 0; jj < 4; jj++) {
                    const int x = x0 + j + jj;
                    float v = 0.f;
                    if (x < n) {
                        const float yl = lint ? al[j + jj] : __ldg(tl + x);
                        const float yr = rint ? ar[j + jj] : (rnone ? 1.f : __ldg(tr + x));
                        v = yl * yr * dv[jj];
                    }
                    o[jj] = v;
                    cmax = fmaxf(cmax, v);
                }
                if (x0 + j < npad)
                    *reinterpret_cast<float4 *>(dad + ((x0 + j) >> 2) * 32) = make_float4(o[0], o[1], o[2], o[3]);
            }
        }
    }
    // pattern maximum over the category warps
    smax[c * TP + pl] = cmax;
    __syncthreads();
    float mx = 0.f;
    for (int cc = 0; cc < C; cc++) mx = fmaxf(mx, smax[cc * TP + pl]);
    int sh = 0;
    float mul = 1.f;
    if (mx < kMixThreshold && mx > 0.f) {  // exact power-of-two rescale
        int ex;
        frexpf(mx, &ex);  // mx = f * 2^ex, f in [0.5, 1)
        sh = 1 - ex;      // mx * 2^sh in [1, 2)
        mul = __int_as_float((127 + sh) << 23);
    }
    if constexpr (NQ > 0) {
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            float4 v = out[q];
            v.x *= mul; v.y *= mul; v.z *= mul; v.w *= mul;
            *reinterpret_cast<float4 *>(dad + q * 32) = v;
        }
    } else if (sh) {
        for (int q = 0; q < nq; q++) {
            float4 v = *reinterpret_cast<float4 *>(dad + q * 32);
            v.x *= mul; v.y *= mul; v.z *= mul; v.w *= mul;
            *reinterpret_cast<float4 *>(dad + q * 32) = v;
        }
    }
    if (c == 0) {
        // exponents are read and written by the category-0 thread of the pattern only
        const int e = (lint ? P.expo[(long long)lref * ld + p] : 0) + (rint ? P.expo[(long long)rref * ld + p] : 0) +
                      (cont ? P.expo[(long long)op.dad_slot * ld + p] : 0);
        P.expo[(long long)op.dad_slot * ld + p] = e - sh;
    }
}

// Branch epilogue (theta or lnL) for this thread's (pattern, category).
template <int NQ, int EPI>
__device__ __forceinline__ void mixed_epilogue(const MixParams &P, int c, int pl, long long p, long long pbase, int TP,
                                               float *s_lc) {
    const int n = P.n, npad = P.npad, C = P.ncat, S = P.state_unknown;
    const int nq = NQ ? NQ : npad >> 2;
    const long long ld = P.ldp;
    const long long PM = (long long)C * n * npad;
    (void)S;
    const float *pa = P.part + (long long)P.a * P.slot_floats + pbase;
    const bool btip = P.b < 0;
    const float *pb = btip ? nullptr : P.part + (long long)P.b * P.slot_floats + pbase;
    const int sb = btip ? P.states[(long long)(-1 - P.b) * ld + p] : 0;
    // this thread's chunks of a and b, read once (NQ > 0: registers)
    constexpr int RQ = NQ ? NQ : 1;
    float4 a4[RQ], b4[RQ];
    if constexpr (NQ > 0) {
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            a4[q] = *reinterpret_cast<const float4 *>(pa + q * 32);
            b4[q] = btip ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4 *>(pb + q * 32);
        }
    }
    auto achunk = [&](int q) -> float4 {
        if constexpr (NQ > 0) return a4[q];
        else return *reinterpret_cast<const float4 *>(pa + q * 32);
    };
    auto bchunk = [&](int q) -> float4 {
        if constexpr (NQ > 0) return b4[q];
        else return *reinterpret_cast<const float4 *>(pb + q * 32);
    };
    if constexpr (EPI == EPI_THETA) {
        // theta[c][i] = (U^-1 a_c)_i (U^-1 b_c)_i in eigen space (tree/phylokernelnew.h:2048-2231)
        float *th = P.theta + p;
        const int m = c / P.cpc;  // mixture class of this category
        if constexpr (NQ > 0) {
            for (int i = 0; i < n; i++) {
                const float *urow = P.inv32 + ((long long)m * n + i) * npad;
                float ua = 0.f, ub = 0.f;
#pragma unroll
                for (int q = 0; q < nq; q++) {
                    const float4 u = ld4(urow + 4 * q);
                    ua = dot4(u, achunk(q), ua);
                    if (!btip) ub = dot4(u, bchunk(q), ub);
                }
                if (btip) ub = (float)__ldg(P.tip_lh + ((long long)sb * P.nmix + m) * n + i);
                th[(long long)(c * n + i) * ld] = ua * ub;
            }
        } else {  // 16 rows at a time: each chunk of a and b read once per block (same order per row)
            for (int i0 = 0; i0 < n; i0 += 16) {
                float ua[16], ub[16];
#pragma unroll
                for (int j = 0; j < 16; j++) ua[j] = ub[j] = 0.f;
                for (int q = 0; q < nq; q++) {
                    const float4 a4 = achunk(q);
                    const float4 b4 = btip ? make_float4(0.f, 0.f, 0.f, 0.f) : bchunk(q);
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        if (i0 + j < n) {
                            const float4 u = ld4(P.inv32 + ((long long)m * n + i0 + j) * npad + 4 * q);
                            ua[j] = dot4(u, a4, ua[j]);
                            if (!btip) ub[j] = dot4(u, b4, ub[j]);
                        }
                    }
                }
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int i = i0 + j;
                    if (i < n) {
                        const float vb = btip ? (float)__ldg(P.tip_lh + ((long long)sb * P.nmix + m) * n + i) : ub[j];
                        th[(long long)(c * n + i) * ld] = ua[j] * vb;
                    }
                }
            }
        }
        if (c == 0) {
            const int ea = P.expo[(long long)P.a * ld + p];
            const int eb = btip ? 0 : P.expo[(long long)P.b * ld + p];
            P.buffer_scale[p] = (double)(ea + eb) * kLn2;
        }
    } else {
        // branch lnL: lh = sum_c p_c sum_x pi_x a[c][x] (P_c b)[x] (tree/phylokernelnew.h:2641-3223)
        const float *base = P.opmats + (long long)P.branch_op * P.op_stride;  // branch matrices, child 0 = b
        float lc = 0.f;
        const double *pic = P.pi + (long long)(c / P.cpc) * n;  // root frequencies of this category's class
        auto term = [&](int x, float av) {
            float w;
            if (btip) {
                w = __ldg(base + 2 * PM + (long long)sb * C * npad + c * npad + x);
            } else {
                const float *prow = base + (long long)(c * n + x) * npad;
                float s0 = 0.f;
#pragma unroll
                for (int q = 0; q < nq; q++) s0 = dot4(ld4(prow + 4 * q), bchunk(q), s0);
                w = s0;
            }
            lc = fmaf((float)__ldg(pic + x) * av, w, lc);
        };
        if constexpr (NQ > 0) {  // x in order, a from the register chunks
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                const float av[4] = {a4[q].x, a4[q].y, a4[q].z, a4[q].w};
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (4 * q + j < n) term(4 * q + j, av[j]);
            }
        } else {  // 16 states at a time: each chunk of b read once per block of x (same order per x)
            for (int x0 = 0; x0 < n; x0 += 16) {
                float w16[16];
#pragma unroll
                for (int j = 0; j < 16; j++) w16[j] = 0.f;
                if (btip) {
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        if (x0 + j < n) w16[j] = __ldg(base + 2 * PM + (long long)sb * C * npad + c * npad + x0 + j);
                } else {
                    for (int q = 0; q < nq; q++) {
                        const float4 b4 = *reinterpret_cast<const float4 *>(pb + q * 32);
#pragma unroll
                        for (int j = 0; j < 16; j++)
                            if (x0 + j < n)
                                w16[j] = dot4(ld4(base + (long long)(c * n + x0 + j) * npad + 4 * q), b4, w16[j]);
                    }
                }
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int x = x0 + j;
                    if (x < n) lc = fmaf((float)__ldg(pic + x) * pa[(x >> 2) * 32 + (x & 3)], w16[j], lc);
                }
            }
        }
        s_lc[threadIdx.x] = lc;
        __syncthreads();
        double v[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
        if (c == 0) {
            double lh = 0.0;
            for (int cc = 0; cc < C; cc++) lh = fma((double)s_lc[cc * TP + pl], P.props[cc], lh);
            const int ea = P.expo[(long long)P.a * ld + p];
            const int eb = btip ? 0 : P.expo[(long long)P.b * ld + p];
            // the +I term is in true scale: bring it to the stored scale 2^-(ea+eb)
            lh = fabs(lh) + ldexp(P.invar[p], -(ea + eb));
            const double plh = log(lh) + (double)(ea + eb) * kLn2;
            P.pattern_lh[p] = plh;
            if (p < P.nptn) {
                const double f = P.freq[p];
                v[0] = plh * f;
                v[1] = (isfinite(plh) ? plh : 4.0 * kLogScaleThreshold) * f;
                v[2] = isfinite(plh) ? 0.0 : 1.0;
            }
        }
        mix_grid_reduce(v, P.red);
    }
}

// Chain form of the fused schedule for up to kChainCat categories: two lanes
// per pattern, lane h of the pair (half-warps h = 0, 1 over the same 16
// patterns) taking categories h and h + 2. A traversal tail of one-op levels,
// whose ops depend on each other one after the other, then runs with every
// pattern of the alignment resident at once instead of in several waves that
// repeat the whole chain, on twice the warps of one thread per pattern. The
// two half-warps read P(t) rows of adjacent categories, 400 floats apart for
// 20 states (opposite bank halves), so the row reads stay one wavefront. Each
// category's children are loaded when it starts (96 registers, no spills:
// the other warps cover the latency); the outputs are stored as
// computed and, in the uncommon case that the pattern needs the rescale,
// re-read and scaled. Same arithmetic as mixed_op / mixed_epilogue
// (row_dot_s, products, maximum, power-of-two rescale; the lnL terms summed
// over the categories in the same order), so the results are bit-identical
// to k_traverse_mixed.
constexpr int kChainCat = 4;
template <int NQ, int EPI>
__global__ void __launch_bounds__(128, 5) k_chain_mixed(const MixParams P) {
    const int C = P.ncat, n = P.n, npad = P.npad, S = P.state_unknown;
    const long long ld = P.ldp;
    const int h = (threadIdx.x >> 4) & 1;  // category parity of this lane
    const long long p = (long long)blockIdx.x * (blockDim.x >> 1) + (threadIdx.x >> 5) * 16 + (threadIdx.x & 15);
    const long long pbase = (p >> 3) * (8LL * C * npad) + (p & 7) * 4;  // + (c * NQ + q) * 32
    const long long PM = (long long)C * n * npad;
    const long long TB = (long long)(S + 1) * C * npad;
    const unsigned pbytes = (unsigned)(2 * PM * 4);
    extern __shared__ __align__(128) float chain_smem[];  // [2][2 * PM] P(t) double buffer
    __shared__ unsigned long long bars[2];
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
        if (P.nops > 0) {
            mbar_expect_tx(&bars[0], pbytes);
            tma_load_1d(chain_smem, P.opmats, pbytes, &bars[0]);
        }
    }
    __syncthreads();
    for (int k = 0; k < P.nops; ++k) {
        const int buf = k & 1;
        const bool lost = !mbar_wait(&bars[buf], (k >> 1) & 1, kWaitPolls);
        if (__syncthreads_or(lost)) {
            if (threadIdx.x == 0) {
                atomicExch(P.status, kStatusTimeout);
                mbar_wait(&bars[buf], (k >> 1) & 1, kWaitPolls);
            }
            return;
        }
        if (threadIdx.x == 0 && k + 1 < P.nops) {
            fence_proxy_async_smem();
            mbar_expect_tx(&bars[buf ^ 1], pbytes);
            tma_load_1d(chain_smem + (buf ^ 1) * 2 * PM, P.opmats + (long long)(k + 1) * P.op_stride, pbytes,
                        &bars[buf ^ 1]);
        }
        const OpDev op = P.ops[k];
        int lref = op.child[0], rref = op.child[1];
        const float *gbase = P.opmats + (long long)k * P.op_stride;
        const float *PL = chain_smem + buf * 2 * PM, *PR = PL + PM, *TL = gbase + 2 * PM, *TR = TL + TB;
        if (lref >= 0 && rref < 0) {  // the tip goes on the left (tree/phylokernelnew.h:1390-1400)
            int t = lref; lref = rref; rref = t;
            const float *q = PL; PL = PR; PR = q;
            q = TL; TL = TR; TR = q;
        }
        const bool lint = lref >= 0, rint = rref >= 0;
        const float *Lp = lint ? P.part + (long long)lref * P.slot_floats + pbase : nullptr;
        const float *Rp = rint ? P.part + (long long)rref * P.slot_floats + pbase : nullptr;
        const float *tl = lint ? nullptr : TL + (long long)P.states[(long long)(-1 - lref) * ld + p] * C * npad;
        const float *tr = rint ? nullptr : TR + (long long)P.states[(long long)(-1 - rref) * ld + p] * C * npad;
        float *dad = P.part + (long long)op.dad_slot * P.slot_floats + pbase;
        float cmax = 0.f;
#pragma unroll
        for (int i = 0; i < kChainCat / 2; i++) {
            const int c = h + 2 * i;
            if (c < C) {
                float4 lv[NQ], rv[NQ];
#pragma unroll
                for (int q = 0; q < NQ; q++) {
                    if (lint) lv[q] = *reinterpret_cast<const float4 *>(Lp + (c * NQ + q) * 32);
                    if (rint) rv[q] = *reinterpret_cast<const float4 *>(Rp + (c * NQ + q) * 32);
                }
                const float *PLc = PL + (long long)c * n * npad, *PRc = PR + (long long)c * n * npad;
#pragma unroll
                for (int q = 0; q < NQ; q++) {
                    float o[4];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int x = 4 * q + j;
                        float v = 0.f;
                        if (x < n) {
                            const float yl = lint ? row_dot_s<NQ>(PLc + x * npad, lv) : __ldg(tl + c * npad + x);
                            const float yr = rint ? row_dot_s<NQ>(PRc + x * npad, rv) : __ldg(tr + c * npad + x);
                            v = yl * yr;
                        }
                        o[j] = v;
                        cmax = fmaxf(cmax, v);
                    }
                    *reinterpret_cast<float4 *>(dad + (c * NQ + q) * 32) = make_float4(o[0], o[1], o[2], o[3]);
                }
            }
        }
        cmax = fmaxf(cmax, __shfl_xor_sync(0xffffffffu, cmax, 16));  // the pair's maximum over all categories
        int sh = 0;
        if (cmax < kMixThreshold && cmax > 0.f) {  // exact power-of-two rescale of this lane's own stores
            int ex;
            frexpf(cmax, &ex);
            sh = 1 - ex;
            const float mul = __int_as_float((127 + sh) << 23);
            for (int c = h; c < C; c += 2)
                for (int q = 0; q < NQ; q++) {
                    float4 v = *reinterpret_cast<float4 *>(dad + (c * NQ + q) * 32);
                    v.x *= mul; v.y *= mul; v.z *= mul; v.w *= mul;
                    *reinterpret_cast<float4 *>(dad + (c * NQ + q) * 32) = v;
                }
        }
        if (h == 0) {
            const int e = (lint ? P.expo[(long long)lref * ld + p] : 0) + (rint ? P.expo[(long long)rref * ld + p] : 0);
            P.expo[(long long)op.dad_slot * ld + p] = e - sh;
        }
    }
    if constexpr (EPI == EPI_NONE) return;

    const float *pa = P.part + (long long)P.a * P.slot_floats + pbase;
    const bool btip = P.b < 0;
    const float *pb = btip ? nullptr : P.part + (long long)P.b * P.slot_floats + pbase;
    const int sb = btip ? P.states[(long long)(-1 - P.b) * ld + p] : 0;
    const int ea = P.expo[(long long)P.a * ld + p];
    const int eb = btip ? 0 : P.expo[(long long)P.b * ld + p];
    if constexpr (EPI == EPI_THETA) {
        // theta[c][i] = (U^-1 a_c)_i (U^-1 b_c)_i (tree/phylokernelnew.h:2048-2231)
        float *th = P.theta + p;
        for (int c = h; c < C; c += 2) {
            float4 a4[NQ], b4[NQ];
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                a4[q] = *reinterpret_cast<const float4 *>(pa + (c * NQ + q) * 32);
                b4[q] = btip ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4 *>(pb + (c * NQ + q) * 32);
            }
            const int m = c / P.cpc;  // mixture class of this category
            for (int i = 0; i < n; i++) {
                const float *urow = P.inv32 + ((long long)m * n + i) * npad;
                float ua = 0.f, ub = 0.f;
#pragma unroll
                for (int q = 0; q < NQ; q++) {
                    const float4 u = ld4(urow + 4 * q);
                    ua = dot4(u, a4[q], ua);
                    if (!btip) ub = dot4(u, b4[q], ub);
                }
                if (btip) ub = (float)__ldg(P.tip_lh + ((long long)sb * P.nmix + m) * n + i);
                th[(long long)(c * n + i) * ld] = ua * ub;
            }
        }
        if (h == 0) P.buffer_scale[p] = (double)(ea + eb) * kLn2;
    } else {
        // branch lnL: lh = sum_c p_c sum_x pi_x a[c][x] (P_c b)[x] (tree/phylokernelnew.h:2641-3223)
        const float *base = P.opmats + (long long)P.branch_op * P.op_stride;  // branch matrices, child 0 = b
        float lcv[kChainCat / 2] = {0.f, 0.f};
#pragma unroll
        for (int i = 0; i < kChainCat / 2; i++) {
            const int c = h + 2 * i;
            if (c >= C) continue;
            float4 a4[NQ], b4[NQ];
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                a4[q] = *reinterpret_cast<const float4 *>(pa + (c * NQ + q) * 32);
                b4[q] = btip ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4 *>(pb + (c * NQ + q) * 32);
            }
            float lc = 0.f;
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                const float av[4] = {a4[q].x, a4[q].y, a4[q].z, a4[q].w};
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int x = 4 * q + j;
                    if (x < n) {
                        float w;
                        if (btip) {
                            w = __ldg(base + 2 * PM + (long long)sb * C * npad + c * npad + x);
                        } else {
                            const float *prow = base + (long long)(c * n + x) * npad;
                            float s0 = 0.f;
#pragma unroll
                            for (int qq = 0; qq < NQ; qq++) s0 = dot4(ld4(prow + 4 * qq), b4[qq], s0);
                            w = s0;
                        }
                        lc = fmaf((float)__ldg(P.pi + (long long)(c / P.cpc) * n + x) * av[j], w, lc);
                    }
                }
            }
            lcv[i] = lc;
        }
        // lane 0 of the pair sums the categories in order 0, 1, 2, 3
        const float o0 = __shfl_xor_sync(0xffffffffu, lcv[0], 16), o1 = __shfl_xor_sync(0xffffffffu, lcv[1], 16);
        double v[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
        if (h == 0) {
            const float lc_all[kChainCat] = {lcv[0], o0, lcv[1], o1};
            double lh = 0.0;
            for (int c = 0; c < C; c++) lh = fma((double)lc_all[c], P.props[c], lh);
            lh = fabs(lh) + ldexp(P.invar[p], -(ea + eb));
            const double plh = log(lh) + (double)(ea + eb) * kLn2;
            P.pattern_lh[p] = plh;
            if (p < P.nptn) {
                const double f = P.freq[p];
                v[0] = plh * f;
                v[1] = (isfinite(plh) ? plh : 4.0 * kLogScaleThreshold) * f;
                v[2] = isfinite(plh) ? 0.0 : 1.0;
            }
        }
        mix_grid_reduce(v, P.red);
    }
}

// fused schedule: NQ = npad/4 float4 chunks per category held in registers
// (1 DNA, 5 protein); NQ = 0 is the chunked path for larger n (codon)
template <int NQ, int EPI>
__global__ void __launch_bounds__(512) k_traverse_mixed(const MixParams P, const int TP, const int nbuf) {
    const int C = P.ncat, npad = P.npad;
    const int nq = NQ ? NQ : npad >> 2;
    const int c = threadIdx.x / TP;   // warp-uniform (TP is a multiple of 32)
    const int pl = threadIdx.x % TP;
    const long long p = (long long)blockIdx.x * TP + pl;
    const long long pbase = (p >> 3) * (8LL * C * npad) + (p & 7) * 4 + (long long)c * nq * 32;
    const long long PM = (long long)C * P.n * npad;
    const unsigned pbytes = (unsigned)(2 * PM * 4);  // both children's P blocks of one op
    extern __shared__ __align__(128) float smem[];   // [nbuf][2*PM] P(t) staging
    __shared__ unsigned long long bars[2];
    __shared__ float s_max[2][512];
    __shared__ float s_lc[512];

    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
        if (P.nops > 0) {
            mbar_expect_tx(&bars[0], pbytes);
            tma_load_1d(smem, P.opmats, pbytes, &bars[0]);
        }
    }
    __syncthreads();

    for (int k = 0; k < P.nops; ++k) {
        const int buf = nbuf == 2 ? (k & 1) : 0;
        const unsigned parity = nbuf == 2 ? ((k >> 1) & 1) : (k & 1);
        // every thread observes the copy's completion itself; the vote makes the
        // give-up decision uniform across the CTA -- barrier (A)
        const bool lost = !mbar_wait(&bars[buf], parity, kWaitPolls);
        if (__syncthreads_or(lost)) {
            if (threadIdx.x == 0) {
                atomicExch(P.status, kStatusTimeout);
                mbar_wait(&bars[buf], parity, kWaitPolls);  // last bounded wait for the copy in flight
            }
            return;
        }
        if (nbuf == 2 && threadIdx.x == 0 && k + 1 < P.nops) {
            // buffer (k+1)&1 was last read in op k-1, before barrier (A)
            fence_proxy_async_smem();
            mbar_expect_tx(&bars[(k + 1) & 1], pbytes);
            tma_load_1d(smem + ((k + 1) & 1) * 2 * PM, P.opmats + (long long)(k + 1) * P.op_stride, pbytes,
                        &bars[(k + 1) & 1]);
        }
        mixed_op<NQ>(P, k, smem + buf * 2 * PM, s_max[k & 1], c, pl, p, pbase, TP);  // contains barrier (B)
        if (nbuf == 1 && threadIdx.x == 0 && k + 1 < P.nops) {
            // every thread passed (B): nobody reads this op's P(t) any more
            fence_proxy_async_smem();
            mbar_expect_tx(&bars[0], pbytes);
            tma_load_1d(smem, P.opmats + (long long)(k + 1) * P.op_stride, pbytes, &bars[0]);
        }
    }
    if constexpr (EPI != EPI_NONE) mixed_epilogue<NQ, EPI>(P, c, pl, p, pbase, TP, s_lc);
}

// level-synchronous schedule: CTA (x, y) computes op op0+y for pattern tile x
template <int NQ>
__global__ void __launch_bounds__(512) k_level_mixed(const MixParams P, const int TP, const int op0) {
    pdl_wait();  // the children come from the levels before
    pdl_trigger();
    const int C = P.ncat, npad = P.npad;
    const int nq = NQ ? NQ : npad >> 2;
    const int c = threadIdx.x / TP;
    const int pl = threadIdx.x % TP;
    const long long p = (long long)blockIdx.x * TP + pl;
    const long long pbase = (p >> 3) * (8LL * C * npad) + (p & 7) * 4 + (long long)c * nq * 32;
    const long long PM = (long long)C * P.n * npad;
    const unsigned pbytes = (unsigned)(2 * PM * 4);
    const int k = op0 + blockIdx.y;
    extern __shared__ __align__(128) float smem[];
    __shared__ unsigned long long bar;
    __shared__ float s_max[512];
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
        mbar_expect_tx(&bar, pbytes);
        tma_load_1d(smem, P.opmats + (long long)k * P.op_stride, pbytes, &bar);
    }
    __syncthreads();
    const bool lost = !mbar_wait(&bar, 0, kWaitPolls);
    if (__syncthreads_or(lost)) {
        if (threadIdx.x == 0) {
            atomicExch(P.status, kStatusTimeout);
            mbar_wait(&bar, 0, kWaitPolls);
        }
        return;
    }
    mixed_op<NQ>(P, k, smem, s_max, c, pl, p, pbase, TP);
}

// Tip-tip ops of one level (both children tips: the first level of every
// traversal). Each output entry is the product of two leaf-table entries
// (P_c(t) times the tip vector, computed per op by the precompute), so the op
// is a pure store stream: a thread takes PPT patterns 128 apart (one for 16+
// states; four for 4-state models, which write only 16 floats per pattern)
// with all their categories, grid (128 PPT-pattern blocks, ops of the level),
// full occupancy. The products, the zero padding, the running maximum and the
// power-of-two rescale are those of the tip-tip case of every other mixed
// kernel, so the partials are bit-identical (tree/phylokernelnew.h:1632-1747
// computes this case from the same lookup tables).
template <int PPT>
__global__ void __launch_bounds__(128) k_tiptip_level(const MixParams P, const int op0) {
    pdl_wait();  // the leaf tables come from the kernels before
    pdl_trigger();
    const int C = P.ncat, n = P.n, npad = P.npad, kq = npad >> 2;
    const long long ld = P.ldp;
    const int k = op0 + blockIdx.y;
    const OpDev op = P.ops[k];
    const long long PM = (long long)C * n * npad;
    const long long TB = (long long)(P.state_unknown + 1) * C * npad;
    const float *T0 = P.opmats + (long long)k * P.op_stride + 2 * PM;
#pragma unroll
    for (int j = 0; j < PPT; j++) {
        const long long p = ((long long)blockIdx.x * PPT + j) * 128 + threadIdx.x;
        if (p >= ld) break;  // whole 128-pattern blocks: uniform per warp
        const float *tl = T0 + (long long)P.states[(long long)(-1 - op.child[0]) * ld + p] * C * npad;
        const float *tr = T0 + TB + (long long)P.states[(long long)(-1 - op.child[1]) * ld + p] * C * npad;
        float *row = P.part + (long long)op.dad_slot * P.slot_floats + (p >> 3) * (8LL * C * npad) + (p & 7) * 4;
        float cmax = 0.f;
        for (int c = 0; c < C; c++) {
            for (int q = 0; q < kq; q++) {
                const float4 a = ld4(tl + c * npad + 4 * q), b = ld4(tr + c * npad + 4 * q);
                const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
                float o[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    o[i] = (4 * q + i < n) ? av[i] * bv[i] : 0.f;
                    cmax = fmaxf(cmax, o[i]);
                }
                *reinterpret_cast<float4 *>(row + (c * kq + q) * 32) = make_float4(o[0], o[1], o[2], o[3]);
            }
        }
        int sh = 0;
        if (cmax < kMixThreshold && cmax > 0.f) {  // exact power-of-two rescale (rare: re-reads its own stores)
            int ex;
            frexpf(cmax, &ex);
            sh = 1 - ex;
            const float mul = __int_as_float((127 + sh) << 23);
            for (int q = 0; q < C * kq; q++) {
                float4 v = *reinterpret_cast<float4 *>(row + q * 32);
                v.x *= mul; v.y *= mul; v.z *= mul; v.w *= mul;
                *reinterpret_cast<float4 *>(row + q * 32) = v;
            }
        }
        P.expo[(long long)op.dad_slot * ld + p] = -sh;
    }
}

bool level_all_tiptip(const iqgpu_engine *e, int op0, int nl) {
    for (int i = op0; i < op0 + nl; i++)
        if (e->h_ops[i].child[0] >= 0 || e->h_ops[i].child[1] >= 0) return false;
    return nl > 0;
}

int launch_tiptip_level(iqgpu_engine *e, const MixParams &P, int op0, int nl) {
    for (int c0 = 0; c0 < nl; c0 += 65535) {
        const int cnt = std::min(65535, nl - c0);
        cudaError_t err =
            e->npad == 4
                ? pdl_launch(k_tiptip_level<4>, dim3((unsigned)((e->Ppad + 511) / 512), cnt), dim3(128), 0, e->st, P,
                             op0 + c0)
                : pdl_launch(k_tiptip_level<1>, dim3((unsigned)(e->Ppad / 128), cnt), dim3(128), 0, e->st, P, op0 + c0);
        e->launches++;
        if (err == cudaSuccess) err = cudaGetLastError();
        if (err != cudaSuccess) return cuda_fail(err, "tiptip_level");
    }
    return IQGPU_OK;
}

// Patterns per CTA: the autotuned value when set (iqgpu_set_tile), else 32.
// TP * ncat <= 512.
static int mix_tile(const iqgpu_engine *e) {
    int tp = e->tile >= 32 ? e->tile : 32;
    while (tp > 32 && tp * e->C > 512) tp >>= 1;
    return tp;
}

template <int NQ, int EPI>
static int launch_mix_t(iqgpu_engine *e, const MixParams &P) {
    const int TP = mix_tile(e);
    const int grid = (int)(e->Ppad / TP);
    const size_t pm_bytes = (size_t)2 * e->C * e->n * e->npad * 4;  // one op's two P(t) blocks
    const int nbuf = pm_bytes * 2 <= 96 * 1024 ? 2 : 1;
    // an epilogue-only launch stages no P(t): no dynamic shared memory, full occupancy
    const size_t smem = P.nops > 0 ? nbuf * pm_bytes : 0;
    auto kern = k_traverse_mixed<NQ, EPI>;
    if (smem > 0) {  // static arrays count against the 48 KB default too
        cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return cuda_fail(err, "traverse_mixed smem attribute");
    }
    kern<<<grid, TP * e->C, smem, e->st>>>(P, TP, nbuf);
    e->launches++;
    return cuda_fail(cudaGetLastError(), "traverse_mixed");
}

// The chain kernel: two lanes per pattern, 64 patterns per 128-thread CTA, or
// 32 per 64-thread CTA when that is what it takes for every pattern tile to be
// resident in one wave.
template <int NQ, int EPI>
static int launch_chain_t(iqgpu_engine *e, const MixParams &P) {
    const size_t smem = P.nops > 0 ? (size_t)2 * 2 * e->C * e->n * e->npad * 4 : 0;  // double-buffered P(t) of one op
    auto kern = k_chain_mixed<NQ, EPI>;
    cudaError_t err = cudaSuccess;
    if (smem > 0)  // static arrays count against the 48 KB default too
        err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return cuda_fail(err, "chain_mixed smem attribute");
    int sms = 1, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->dev) != cudaSuccess || sms < 1) sms = 1;
    int tb = 128;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem) == cudaSuccess &&
        e->Ppad / 64 > (long long)per_sm * sms &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 64, smem) == cudaSuccess &&
        e->Ppad / 32 <= (long long)per_sm * sms)
        tb = 64;
    // an ordinary launch: as a dependent of the last tensor-core level its CTAs
    // would sit beside that level's CTAs until it ends, and measured slower
    kern<<<(unsigned)(e->Ppad / (tb / 2)), tb, smem, e->st>>>(P);
    e->launches++;
    return cuda_fail(cudaGetLastError(), "chain_mixed");
}

// Levels l0 .. of the uploaded list, one launch each.
template <int NQ>
static int launch_levels_t(iqgpu_engine *e, const MixParams &P, int l0 = 0) {
    const int TP = mix_tile(e);
    const int grid = (int)(e->Ppad / TP);
    const size_t smem = (size_t)2 * e->C * e->n * e->npad * 4;
    auto kern = k_level_mixed<NQ>;
    if (smem > 0) {  // static arrays count against the 48 KB default too
        cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return cuda_fail(err, "level_mixed smem attribute");
    }
    for (int l = l0; l < e->nlevels; l++) {
        const int op0 = e->level_off[l], nl = e->level_off[l + 1] - op0;
        if (nl <= 0) continue;
        if (level_all_tiptip(e, op0, nl)) {
            int rc = launch_tiptip_level(e, P, op0, nl);
            if (rc) return rc;
            continue;
        }
        cudaError_t err = pdl_launch(kern, dim3(grid, nl), dim3(TP * e->C), smem, e->st, P, TP, op0);
        e->launches++;
        if (err == cudaSuccess) err = cudaGetLastError();
        if (err != cudaSuccess) return cuda_fail(err, "level_mixed");
    }
    return IQGPU_OK;
}

template <int EPI>
static int dispatch_mix(iqgpu_engine *e, MixParams P) {
    int rc = IQGPU_OK;
    if (e->level_sync && P.nops > 0) {
        switch (e->npad) {
        case 4: rc = launch_levels_t<1>(e, P); break;
        case 20: rc = launch_levels_t<5>(e, P); break;
        default: rc = launch_levels_t<0>(e, P); break;
        }
        if (rc || EPI == EPI_NONE) return rc;
        P.nops = 0;  // the epilogue runs alone; branch matrices stay at P.branch_op
    }
    switch (e->npad) {
    case 4: return launch_mix_t<1, EPI>(e, P);
    case 20: return launch_mix_t<5, EPI>(e, P);
    default: return launch_mix_t<0, EPI>(e, P);
    }
}

int launch_traverse_dna(iqgpu_engine *e, const MixParams &P, int epi);
int launch_levels_dna(iqgpu_engine *e, MixParams P, int epi);
int launch_flow_dna(iqgpu_engine *e, const MixParams &P);
int launch_traverse_tc(iqgpu_engine *e, const MixParams &M, int *rest);

// ops [rest, nops) and the epilogue on the fused CUDA-core kernel, after ops
// [0, rest) ran on the tensor cores: the op list is shifted so the kernel sees
// them as ops 0.. (the branch matrices keep their block)
template <int EPI>
static int fused_rest(iqgpu_engine *e, MixParams P, int rest) {
    P.ops += rest;
    P.op_base += rest;
    P.opmats += (long long)rest * P.op_stride;
    P.nops -= rest;
    P.branch_op -= rest;
    switch (e->npad) {
    case 4: return launch_mix_t<1, EPI>(e, P);
    case 20: return e->C <= kChainCat ? launch_chain_t<5, EPI>(e, P) : launch_mix_t<5, EPI>(e, P);
    default: return launch_mix_t<0, EPI>(e, P);
    }
}

template <int EPI>
static int launch_fused_any(iqgpu_engine *e, const MixParams &P) {
    switch (e->npad) {
    case 4: return launch_mix_t<1, EPI>(e, P);
    case 20: return launch_mix_t<5, EPI>(e, P);
    default: return launch_mix_t<0, EPI>(e, P);
    }
}

int launch_traverse_mixed(iqgpu_engine *e, int nops, int epi, int32_t a, int32_t b, double len) {
    MixParams P = mix_params(e, nops);
    P.a = a;
    P.b = b;
    P.len = len;
    if (nops == 0 && epi == EPI_NONE) return IQGPU_OK;
    if (e->has_multi) {
        // multifurcating records share their dad: the fused CUDA-core kernel walks
        // them in order per pattern (the level and tensor-core schedules would
        // run them side by side)
        switch (epi) {
        case EPI_NONE: return launch_fused_any<EPI_NONE>(e, P);
        case EPI_LNL: return launch_fused_any<EPI_LNL>(e, P);
        default: return launch_fused_any<EPI_THETA>(e, P);
        }
    }
    if (e->tc) {
        int rest = nops;
        int rc = launch_traverse_tc(e, P, &rest);
        if (rc || (rest >= nops && epi == EPI_NONE)) return rc;
        switch (epi) {
        case EPI_NONE: return fused_rest<EPI_NONE>(e, P, rest);
        case EPI_LNL: return fused_rest<EPI_LNL>(e, P, rest);
        default: return fused_rest<EPI_THETA>(e, P, rest);
        }
    }
    // 4-state models: one thread per pattern and all its categories, unless a
    // per-category tile was chosen explicitly
    if (e->n == 4 && e->C <= 4 && (e->tile == 1 || (e->tile == 2 && e->level_sync))) {
        if (!e->level_sync && !e->flow) return launch_traverse_dna(e, P, epi);
        if (e->level_sync) return launch_levels_dna(e, P, epi);
        int rc = launch_flow_dna(e, P);
        if (rc || epi == EPI_NONE) return rc;
        P.nops = 0;  // the epilogue alone
        return launch_traverse_dna(e, P, epi);
    }
    if (e->n == 4 && e->C <= 4 && e->tile == 0 && !e->level_sync) return launch_traverse_dna(e, P, epi);
    switch (epi) {
    case EPI_NONE: return dispatch_mix<EPI_NONE>(e, P);
    case EPI_LNL: return dispatch_mix<EPI_LNL>(e, P);
    default: return dispatch_mix<EPI_THETA>(e, P);
    }
}

}  // namespace iqg
