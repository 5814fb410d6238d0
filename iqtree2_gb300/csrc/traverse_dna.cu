// Mixed-precision traversal specialised for 4-state (DNA) models.
//
// With n = 4 a category's update is 32 multiply-adds, so the kernel is bound
// by memory latency, not arithmetic: one thread owns one pattern and all of
// its rate categories. A thread then issues every child load of an op at once
// (ncat float4 per child, each warp touching whole 128-byte lines), finds the
// pattern's maximum without any cross-thread exchange, and rescales and
// stores its block in registers; the only barrier per op is the one that
// publishes the op's TMA-staged P(t) matrices (double-buffered, so op k+1's
// copy is in flight while op k computes). A level-synchronous form
// (k_level_dna) runs each tree level as one launch, and a dataflow form
// (k_flow_dna) runs the whole list as one persistent launch.
#include <cuda_runtime.h>

#include <algorithm>

#include "mixed.cuh"

namespace iqg {

constexpr int kDnaTile = 128;  // patterns (= threads) per CTA
constexpr int kDnaMaxCat = 4;  // register-resident categories (ncat <= 4 uses this kernel)

// cp.async (LDGSTS): 16-byte and 4-byte global -> shared copies that complete
// per thread, grouped and waited for in order (no registers held meanwhile)
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

constexpr int kDnaAhead = 4;  // ops whose other child is in flight ahead of the one computed

template <int EPI>
__global__ void __launch_bounds__(kDnaTile, 5) k_traverse_dna(const MixParams P) {
    pdl_wait();  // the levels before wrote its first children
    pdl_trigger();
    constexpr int n = 4, npad = 4;
    const int C = P.ncat, S = P.state_unknown;
    const long long p = (long long)blockIdx.x * kDnaTile + threadIdx.x;
    const long long ld = P.ldp;
    const long long pbase = (p >> 3) * (8LL * C * npad) + (p & 7) * 4;  // + c*32
    const long long PM = (long long)C * n * npad;
    const long long TB = (long long)(S + 1) * C * npad;
    const unsigned pbytes = (unsigned)(2 * PM * 4);
    __shared__ __align__(128) float sP[2][2 * kDnaMaxCat * 16];
    __shared__ unsigned long long bars[2];

    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
        if (P.nops > 0) {
            mbar_expect_tx(&bars[0], pbytes);
            tma_load_1d(sP[0], P.opmats, pbytes, &bars[0]);
        }
    }
    __syncthreads();

    // The previous op's output for this pattern stays in registers (as
    // stored), and the other internal child of each of the next kDnaAhead ops
    // is copied ahead into this thread's slots of a shared-memory ring with
    // cp.async: along a chain of ops (each taking the previous op's output as
    // one child, as the one-op levels near the root do) the children of the
    // coming ops are in flight while the current one computes. The request
    // for op j is issued after op j - kDnaAhead has stored its outputs, and
    // names (pick) a child produced before that op, so its values are in
    // memory a whole op before the copy starts; every thread derives the same
    // choice from the op list.
    __shared__ __align__(16) float4 pf[kDnaAhead][kDnaMaxCat][kDnaTile];
    __shared__ int pfe[kDnaAhead][kDnaTile];
    int prev_dad = -1, prev_e = 0;
    float4 prev[kDnaMaxCat];
    auto pick = [&](int j) -> int {
        const OpDev o = P.ops[j];
        const int skip = j > 0 ? P.ops[j - 1].dad_slot : -1;
#pragma unroll
        for (int ch = 0; ch < 2; ch++) {
            const int r = o.child[ch];
            const long long prod = ch ? (long long)o.prod1 : (long long)o.prod0;
            if (r >= 0 && r != skip && (prod < 0 || prod - P.op_base < (long long)j - kDnaAhead)) return r;
        }
        return -1;
    };
    auto request = [&](int j) {  // one commit group per op, empty when nothing is requested
        const int ref = j < P.nops ? pick(j) : -1;
        if (ref >= 0) {
            const int d = j % kDnaAhead;
            const float *src = P.part + (long long)ref * P.slot_floats + pbase;
#pragma unroll
            for (int c = 0; c < kDnaMaxCat; c++)
                if (c < C) cp_async16(&pf[d][c][threadIdx.x], src + c * 32);
            cp_async4(&pfe[d][threadIdx.x], P.expo + (long long)ref * ld + p);
        }
        cp_async_commit();
    };
    for (int j = 0; j < kDnaAhead; j++) request(j);

    for (int k = 0; k < P.nops; ++k) {
        const int buf = k & 1;
        const bool lost = !mbar_wait(&bars[buf], (k >> 1) & 1, kWaitPolls);
        if (__syncthreads_or(lost)) {
            if (threadIdx.x == 0) {
                atomicExch(P.status, kStatusTimeout);
                mbar_wait(&bars[buf], (k >> 1) & 1, kWaitPolls);
            }
            cp_async_wait<0>();  // no copy into this CTA's shared memory outlives it
            return;
        }
        if (threadIdx.x == 0 && k + 1 < P.nops) {
            fence_proxy_async_smem();
            mbar_expect_tx(&bars[buf ^ 1], pbytes);
            tma_load_1d(sP[buf ^ 1], P.opmats + (long long)(k + 1) * P.op_stride, pbytes, &bars[buf ^ 1]);
        }
        const OpDev op = P.ops[k];
        int lref = op.child[0], rref = op.child[1];
        const float *gbase = P.opmats + (long long)k * P.op_stride;
        const float *PL = sP[buf], *PR = sP[buf] + PM, *TL = gbase + 2 * PM, *TR = TL + TB;
        const bool sw = lref >= 0 && rref < 0;  // the tip goes on the left (tree/phylokernelnew.h:1390-1400)
        if (sw) {
            int t = lref; lref = rref; rref = t;
            const float *q = PL; PL = PR; PR = q;
            q = TL; TL = TR; TR = q;
        }
        const bool lint = lref >= 0, rint = rref >= 0;
        const float *tl = lint ? nullptr : TL + (long long)P.states[(long long)(-1 - lref) * ld + p] * C * npad;
        const float *tr = rint ? nullptr : TR + (long long)P.states[(long long)(-1 - rref) * ld + p] * C * npad;
        float4 out[kDnaMaxCat];
        float mx = 0.f;
        // an internal side comes from registers (previous output), from the
        // ring (the child requested for this op), or is loaded here
        cp_async_wait<kDnaAhead - 1>();  // this thread's copies for ops <= k have landed
        const int got = pick(k), d = k % kDnaAhead;
        float4 lv[kDnaMaxCat], rv[kDnaMaxCat];
        int e = 0;
        auto side = [&](int ref, float4 (&v)[kDnaMaxCat]) {
            if (ref == prev_dad) {
#pragma unroll
                for (int c = 0; c < kDnaMaxCat; c++) v[c] = prev[c];
                e += prev_e;
            } else if (ref == got) {
#pragma unroll
                for (int c = 0; c < kDnaMaxCat; c++) v[c] = pf[d][c][threadIdx.x];
                e += pfe[d][threadIdx.x];
            } else {
                const float *src = P.part + (long long)ref * P.slot_floats + pbase;
#pragma unroll
                for (int c = 0; c < kDnaMaxCat; c++)
                    if (c < C) v[c] = *reinterpret_cast<const float4 *>(src + c * 32);
                e += P.expo[(long long)ref * ld + p];
            }
        };
        if (lint) {
            side(lref, lv);
        } else {
#pragma unroll
            for (int c = 0; c < kDnaMaxCat; c++) if (c < C) lv[c] = ld4(tl + c * npad);
        }
        if (rint) {
            side(rref, rv);
        } else {
#pragma unroll
            for (int c = 0; c < kDnaMaxCat; c++) if (c < C) rv[c] = ld4(tr + c * npad);
        }
#pragma unroll
        for (int c = 0; c < kDnaMaxCat; c++) {
            if (c < C) {
                float yl[4], yr[4];
                const float *pl = PL + c * 16, *pr = PR + c * 16;
#pragma unroll
                for (int x = 0; x < 4; x++) {
                    if (lint) {
                        const float4 m = *reinterpret_cast<const float4 *>(pl + x * 4);
                        yl[x] = fmaf(m.x, lv[c].x, fmaf(m.y, lv[c].y, fmaf(m.z, lv[c].z, m.w * lv[c].w)));
                    } else {
                        yl[x] = x == 0 ? lv[c].x : x == 1 ? lv[c].y : x == 2 ? lv[c].z : lv[c].w;
                    }
                    if (rint) {
                        const float4 m = *reinterpret_cast<const float4 *>(pr + x * 4);
                        yr[x] = fmaf(m.x, rv[c].x, fmaf(m.y, rv[c].y, fmaf(m.z, rv[c].z, m.w * rv[c].w)));
                    } else {
                        yr[x] = x == 0 ? rv[c].x : x == 1 ? rv[c].y : x == 2 ? rv[c].z : rv[c].w;
                    }
                }
                out[c] = make_float4(yl[0] * yr[0], yl[1] * yr[1], yl[2] * yr[2], yl[3] * yr[3]);
                mx = fmaxf(mx, fmaxf(fmaxf(out[c].x, out[c].y), fmaxf(out[c].z, out[c].w)));
            }
        }
        int sh = 0;
        float mul = 1.f;
        if (mx < kMixThreshold && mx > 0.f) {  // exact power-of-two rescale
            int ex;
            frexpf(mx, &ex);
            sh = 1 - ex;
            mul = __int_as_float((127 + sh) << 23);
        }
        float *dad = P.part + (long long)op.dad_slot * P.slot_floats + pbase;
#pragma unroll
        for (int c = 0; c < kDnaMaxCat; c++) {
            if (c < C) {
                float4 v = out[c];
                v.x *= mul; v.y *= mul; v.z *= mul; v.w *= mul;
                *reinterpret_cast<float4 *>(dad + c * 32) = v;
                prev[c] = v;
            }
        }
        P.expo[(long long)op.dad_slot * ld + p] = e - sh;
        prev_dad = op.dad_slot;
        prev_e = e - sh;
        // after this op's stores; slot d is free again (its values are in lv / rv)
        request(k + kDnaAhead);
    }

    if constexpr (EPI == EPI_NONE) return;

    const float *pa = P.part + (long long)P.a * P.slot_floats + pbase;
    const bool btip = P.b < 0;
    const float *pb = btip ? nullptr : P.part + (long long)P.b * P.slot_floats + pbase;
    const int sb = btip ? P.states[(long long)(-1 - P.b) * ld + p] : 0;
    const int ea = P.expo[(long long)P.a * ld + p];
    const int eb = btip ? 0 : P.expo[(long long)P.b * ld + p];

    if constexpr (EPI == EPI_THETA) {
        float *th = P.theta + p;
        for (int c = 0; c < C; c++) {
            const float4 av = *reinterpret_cast<const float4 *>(pa + c * 32);
            const float4 bv = btip ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4 *>(pb + c * 32);
            const int m = c / P.cpc;  // mixture class of this category
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float4 u = ld4(P.inv32 + (m * n + i) * npad);
                const float ua = fmaf(u.x, av.x, fmaf(u.y, av.y, fmaf(u.z, av.z, u.w * av.w)));
                const float ub = btip ? (float)__ldg(P.tip_lh + ((long long)sb * P.nmix + m) * n + i)
                                      : fmaf(u.x, bv.x, fmaf(u.y, bv.y, fmaf(u.z, bv.z, u.w * bv.w)));
                th[(long long)(c * n + i) * ld] = ua * ub;
            }
        }
        P.buffer_scale[p] = (double)(ea + eb) * kLn2;
        return;
    } else {
        const float *base = P.opmats + (long long)P.branch_op * P.op_stride;  // branch matrices, child 0 = b
        double lh = 0.0;
        for (int c = 0; c < C; c++) {
            const float4 av = *reinterpret_cast<const float4 *>(pa + c * 32);
            float w[4];
            if (btip) {
                const float4 t = ld4(base + 2 * PM + (long long)sb * C * npad + c * npad);
                w[0] = t.x; w[1] = t.y; w[2] = t.z; w[3] = t.w;
            } else {
                const float4 bv = *reinterpret_cast<const float4 *>(pb + c * 32);
#pragma unroll
                for (int x = 0; x < 4; x++) {
                    const float4 m = ld4(base + (c * n + x) * npad);
                    w[x] = fmaf(m.x, bv.x, fmaf(m.y, bv.y, fmaf(m.z, bv.z, m.w * bv.w)));
                }
            }
            const double *pic = P.pi + (c / P.cpc) * n;  // root frequencies of this category's class
            float lc = (float)__ldg(pic) * av.x * w[0];
            lc = fmaf((float)__ldg(pic + 1) * av.y, w[1], lc);
            lc = fmaf((float)__ldg(pic + 2) * av.z, w[2], lc);
            lc = fmaf((float)__ldg(pic + 3) * av.w, w[3], lc);
            lh = fma((double)lc, P.props[c], lh);
        }
        lh = fabs(lh) + ldexp(P.invar[p], -(ea + eb));
        const double plh = log(lh) + (double)(ea + eb) * kLn2;
        P.pattern_lh[p] = plh;
        double v[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
        if (p < P.nptn) {
            const double f = P.freq[p];
            v[0] = plh * f;
            v[1] = (isfinite(plh) ? plh : 4.0 * kLogScaleThreshold) * f;
            v[2] = isfinite(plh) ? 0.0 : 1.0;
        }
        mix_grid_reduce(v, P.red);
    }
}

// One op k for the 128 patterns of tile `tile`, one thread per pattern and all
// of its categories. Children and exponents are read at L2 (ld.global.cg):
// under the dataflow schedule they were written by other CTAs of the same
// launch. The op's P(t) blocks (2 x ncat x 16 floats) come through the
// read-only cache (warp-uniform addresses).
template <int PPT>
__device__ __forceinline__ void dna_op(const MixParams &P, int k, long long tile, int dad_slot, int lref, int rref) {
    constexpr int n = 4, npad = 4;
    const int C = P.ncat, S = P.state_unknown;
    const long long ld = P.ldp;
    const long long PM = (long long)C * n * npad;
    const long long TB = (long long)(S + 1) * C * npad;
    const float *gbase = P.opmats + (long long)k * P.op_stride;
    const float *PL = gbase, *PR = gbase + PM, *TL = gbase + 2 * PM, *TR = TL + TB;
    if (lref >= 0 && rref < 0) {  // the tip goes on the left (tree/phylokernelnew.h:1390-1400)
        int t = lref; lref = rref; rref = t;
        const float *q = PL; PL = PR; PR = q;
        q = TL; TL = TR; TR = q;
    }
    const bool lint = lref >= 0, rint = rref >= 0;
    // PPT patterns per thread, 128 apart: every load of all of them is issued first
    long long p[PPT], pbase[PPT];
    bool live[PPT];
    int e[PPT];
    float4 lv[PPT][kDnaMaxCat], rv[PPT][kDnaMaxCat];
#pragma unroll
    for (int j = 0; j < PPT; j++) {
        p[j] = (tile * PPT + j) * kDnaTile + threadIdx.x;
        live[j] = p[j] < ld;  // whole 128-pattern blocks: uniform per warp
        pbase[j] = (p[j] >> 3) * (8LL * C * npad) + (p[j] & 7) * 4;
        if (!live[j]) continue;
        const float *Lp = lint ? P.part + (long long)lref * P.slot_floats + pbase[j] : nullptr;
        const float *Rp = rint ? P.part + (long long)rref * P.slot_floats + pbase[j] : nullptr;
        const float *tl = lint ? nullptr : TL + (long long)P.states[(long long)(-1 - lref) * ld + p[j]] * C * npad;
        const float *tr = rint ? nullptr : TR + (long long)P.states[(long long)(-1 - rref) * ld + p[j]] * C * npad;
        e[j] = (lint ? __ldcg(P.expo + (long long)lref * ld + p[j]) : 0) +
               (rint ? __ldcg(P.expo + (long long)rref * ld + p[j]) : 0);
#pragma unroll
        for (int c = 0; c < kDnaMaxCat; c++) {
            if (c < C) {
                lv[j][c] = lint ? __ldcg(reinterpret_cast<const float4 *>(Lp + c * 32)) : ld4(tl + c * npad);
                rv[j][c] = rint ? __ldcg(reinterpret_cast<const float4 *>(Rp + c * 32)) : ld4(tr + c * npad);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < PPT; j++) {
        if (!live[j]) continue;
        float4 out[kDnaMaxCat];
        float mx = 0.f;
#pragma unroll
        for (int c = 0; c < kDnaMaxCat; c++) {
            if (c < C) {
                float yl[4], yr[4];
#pragma unroll
                for (int x = 0; x < 4; x++) {
                    if (lint) {
                        const float4 m = ld4(PL + c * 16 + x * 4);
                        yl[x] = fmaf(m.x, lv[j][c].x, fmaf(m.y, lv[j][c].y, fmaf(m.z, lv[j][c].z, m.w * lv[j][c].w)));
                    } else {
                        yl[x] = x == 0 ? lv[j][c].x : x == 1 ? lv[j][c].y : x == 2 ? lv[j][c].z : lv[j][c].w;
                    }
                    if (rint) {
                        const float4 m = ld4(PR + c * 16 + x * 4);
                        yr[x] = fmaf(m.x, rv[j][c].x, fmaf(m.y, rv[j][c].y, fmaf(m.z, rv[j][c].z, m.w * rv[j][c].w)));
                    } else {
                        yr[x] = x == 0 ? rv[j][c].x : x == 1 ? rv[j][c].y : x == 2 ? rv[j][c].z : rv[j][c].w;
                    }
                }
                out[c] = make_float4(yl[0] * yr[0], yl[1] * yr[1], yl[2] * yr[2], yl[3] * yr[3]);
                mx = fmaxf(mx, fmaxf(fmaxf(out[c].x, out[c].y), fmaxf(out[c].z, out[c].w)));
            }
        }
        int sh = 0;
        float mul = 1.f;
        if (mx < kMixThreshold && mx > 0.f) {  // exact power-of-two rescale
            int ex;
            frexpf(mx, &ex);
            sh = 1 - ex;
            mul = __int_as_float((127 + sh) << 23);
        }
        float *dad = P.part + (long long)dad_slot * P.slot_floats + pbase[j];
#pragma unroll
        for (int c = 0; c < kDnaMaxCat; c++) {
            if (c < C) {
                float4 v = out[c];
                v.x *= mul; v.y *= mul; v.z *= mul; v.w *= mul;
                *reinterpret_cast<float4 *>(dad + c * 32) = v;
            }
        }
        P.expo[(long long)dad_slot * ld + p[j]] = e[j] - sh;
    }
}

// Level-synchronous form: CTA (x, y) computes op op0 + y for tile x. All
// (op, tile) pairs of a level are independent, so every child load of the
// level can be in flight at once.
// The level's op descriptors travel as a kernel parameter (constant bank), so a
// CTA issues its child loads without first reading its op from global memory.
constexpr int kLevelOps = 1024;
struct LevelOps {
    int3 op[kLevelOps];  // dad slot, child 0, child 1 of ops op0 .. op0 + count - 1
};

// PPT patterns per thread: CTA (x, y) covers patterns 128 PPT x .. 128 PPT (x + 1) - 1.
template <int PPT>
__global__ void __launch_bounds__(kDnaTile) k_level_dna(const MixParams P, const int op0, const LevelOps L) {
    pdl_wait();  // the children come from the levels before
    pdl_trigger();
    const int3 o = L.op[blockIdx.y];
    dna_op<PPT>(P, op0 + blockIdx.y, blockIdx.x, o.x, o.y, o.z);
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Dataflow form: one persistent launch. CTAs take items i = k * ntiles + t
// (op k of the level-ordered list, tile t) from an atomic ticket in increasing
// order; before computing, an item waits until the flags of the items that
// produce its children for the same tile read `epoch` (flags are cleared
// before every launch). Every producer has a
// smaller index, so it was taken earlier by a CTA that is running, and the
// waits end; they are bounded all the same (status word, then the CTA stops).
__global__ void __launch_bounds__(kDnaTile) k_flow_dna(const MixParams P, unsigned *done, unsigned *ticket,
                                                        const unsigned epoch, const int ntiles) {
    __shared__ int s_item;
    __shared__ int s_ok;
    const long long total = (long long)P.nops * ntiles;
    for (;;) {
        if (threadIdx.x == 0) {
            s_item = (int)atomicAdd(ticket, 1u);
            int ok = 1;
            const long long i = s_item;
            if (i < total) {
                const int k = (int)(i / ntiles), t = (int)(i % ntiles);
                const OpDev op = P.ops[k];
                const int prod[2] = {op.prod0, (int)op.prod1};
                for (int j = 0; j < 2 && ok; j++) {
                    if (prod[j] < 0) continue;
                    const unsigned *f = done + (long long)prod[j] * ntiles + t;
                    unsigned polls = 0;
                    while (ld_acquire(f) != epoch) {
                        if (++polls >= P.wait_polls || *(volatile int *)P.status != 0) { ok = 0; break; }
                    }
                }
                if (!ok) atomicExch(P.status, kStatusTimeout);
            }
            s_ok = ok;
        }
        __syncthreads();
        const long long i = s_item;
        const int ok = s_ok;
        __syncthreads();  // s_item / s_ok are rewritten by the next iteration
        if (i >= total || !ok) return;
        const int k = (int)(i / ntiles), t = (int)(i % ntiles);
        const OpDev op = P.ops[k];
        dna_op<1>(P, k, t, op.dad_slot, op.child[0], op.child[1]);
        __threadfence();  // this thread's outputs are visible device-wide before the flag
        __syncthreads();
        if (threadIdx.x == 0) atomicExch(done + i, epoch);
    }
}

int launch_traverse_dna(iqgpu_engine *e, const MixParams &P, int epi);

template <int PPT>
static int launch_levels_dna_t(iqgpu_engine *e, MixParams P, int epi) {
    const int grid = (int)((e->Ppad + kDnaTile * PPT - 1) / (kDnaTile * PPT));
    int per_sm = 1, sms = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_level_dna<PPT>, kDnaTile, 0) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->dev) != cudaSuccess || sms < 1) sms = 1;
    const long long wave = (long long)per_sm * sms;
    int l = 0;
    for (; l < e->nlevels; l++) {
        const int op0 = e->level_off[l], nl = e->level_off[l + 1] - op0;
        if (nl <= 0) continue;
        if ((long long)nl * grid < wave) break;
        if (level_all_tiptip(e, op0, nl)) {  // a store stream: several patterns per thread
            const int rc = launch_tiptip_level(e, P, op0, nl);
            if (rc) return rc;
            continue;
        }
        for (int c0 = 0; c0 < nl; c0 += kLevelOps) {  // levels wider than one parameter block: several launches
            const int cnt = std::min(kLevelOps, nl - c0);
            LevelOps L;
            for (int i = 0; i < cnt; i++) {
                const OpDev &d = e->h_ops[op0 + c0 + i];
                L.op[i] = make_int3(d.dad_slot, d.child[0], d.child[1]);
            }
            cudaError_t err = pdl_launch(k_level_dna<PPT>, dim3(grid, cnt), dim3(kDnaTile), 0, e->st, P, op0 + c0, L);
            e->launches++;
            if (err == cudaSuccess) err = cudaGetLastError();
            if (err != cudaSuccess) return cuda_fail(err, "level_dna");
        }
    }
    const int rest = l < e->nlevels ? e->level_off[l] : P.nops;
    if (rest >= P.nops && epi == EPI_NONE) return IQGPU_OK;
    // the tail ops [rest, nops) and the epilogue: shift the op list so the fused
    // kernel sees them as ops 0.. (the branch matrices keep their block)
    P.ops += rest;
    P.op_base += rest;
    P.opmats += (long long)rest * P.op_stride;
    P.nops -= rest;
    P.branch_op -= rest;
    return launch_traverse_dna(e, P, epi);
}

// Level-synchronous schedule with a fused tail: levels whose (op, tile) pairs
// fill the GPU (at least the resident CTAs of one wave) run one launch each;
// the remaining narrow levels (a Yule tree ends in a chain of one-op levels)
// and the branch epilogue run as one fused launch that walks them per tile.
// Tile 2 selects two patterns per thread in the level launches.
int launch_levels_dna(iqgpu_engine *e, MixParams P, int epi) {
    return e->tile == 2 ? launch_levels_dna_t<2>(e, P, epi) : launch_levels_dna_t<1>(e, P, epi);
}

int launch_flow_dna(iqgpu_engine *e, const MixParams &P) {
    if (P.nops <= 0) return IQGPU_OK;
    const int ntiles = (int)(e->Ppad / kDnaTile);
    // every launch starts from cleared flags and ticket (stream-ordered memsets,
    // so the launch sequence can also be captured into a graph and replayed)
    cudaError_t err = cudaMemsetAsync(e->d_flow_done, 0, (size_t)P.nops * ntiles * 4, e->st);
    if (err == cudaSuccess) err = cudaMemsetAsync(e->d_flow_ticket, 0, 4, e->st);
    if (err != cudaSuccess) return cuda_fail(err, "flow flag reset");
    int per_sm = 1, sms = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_flow_dna, kDnaTile, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->dev) != cudaSuccess || sms < 1) sms = 1;
    const long long items = (long long)P.nops * ntiles;
    const int grid = (int)std::min<long long>(items, (long long)per_sm * sms);
    k_flow_dna<<<grid, kDnaTile, 0, e->st>>>(P, e->d_flow_done, e->d_flow_ticket, 1u, ntiles);
    e->launches++;
    return cuda_fail(cudaGetLastError(), "flow_dna");
}

int launch_traverse_dna(iqgpu_engine *e, const MixParams &P, int epi) {
    const int grid = (int)(e->Ppad / kDnaTile);
    e->launches++;
    cudaError_t err = cudaSuccess;
    switch (epi) {
    case EPI_NONE: err = pdl_launch(k_traverse_dna<EPI_NONE>, dim3(grid), dim3(kDnaTile), 0, e->st, P); break;
    case EPI_LNL: err = pdl_launch(k_traverse_dna<EPI_LNL>, dim3(grid), dim3(kDnaTile), 0, e->st, P); break;
    default: err = pdl_launch(k_traverse_dna<EPI_THETA>, dim3(grid), dim3(kDnaTile), 0, e->st, P); break;
    }
    if (err != cudaSuccess) return cuda_fail(err, "traverse_dna");
    return cuda_fail(cudaGetLastError(), "traverse_dna");
}

}  // namespace iqg
