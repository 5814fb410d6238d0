// Shared definitions of the mixed-precision path (FP32 standard-basis
// partials, per-pattern power-of-two exponents, FP64 exp/log/sums).
//
// Layout. A slot stores each pattern's block of C*npad floats (npad = n
// rounded up to 4), interleaved by groups of 8 patterns so that every
// (category, 4-state) chunk of 8 patterns is one contiguous 128-byte core
// matrix: index(p, c, y) = (p/8)*8*C*npad + (c*npad/4 + y/4)*32 + (p%8)*4 + y%4.
// A warp that handles 32 patterns of one category touches four whole
// 128-byte lines per float4 load. The same bytes form K-major 8-row x 16-byte
// core-matrix tiles, the tensor cores' operand layout.
#pragma once

#include <cuda_runtime.h>

#include "engine.cuh"

namespace iqg {

constexpr float kMixThreshold = 9.094947017729282e-13f;  // 2^-40
constexpr double kLn2 = 0.6931471805599453094172321;
constexpr int kMixTile = 128;  // patterns per CTA; the CTA has kMixTile * ncat threads

struct MixParams {
    int n, npad, ncat, state_unknown, nops, nptn;
    long long ldp;          // Ppad
    long long slot_floats;  // Ppad * C * npad
    long long op_stride;    // floats per op
    const OpDev *ops;
    int op_base;            // index of ops[0] in the uploaded list (the producer indices' origin)
    const float *opmats;    // per op: P child0 [C][n][npad], P child1, table child0 [S+1][C][npad], table child1
    const float *inv32;     // [n][npad] FP32 copy of U^-1
    const double *pi;       // [nmix][n]
    const double *tip_lh;   // eigen-space tip vectors [S+1][nmix][n]
    int nmix, cpc;          // mixture classes; category c uses class c / cpc (eval, U, U^-1, pi, tips)
    const double *freq, *invar;
    const double *eval, *rates, *props;
    const uint8_t *states;
    float *part;
    int32_t *expo;
    int32_t a, b;
    double len;
    double *pattern_lh;
    float *theta;           // [B][ldp]
    double *buffer_scale;
    Reduce red;
    int *status;            // set to a nonzero code when a bounded wait gives up
    unsigned wait_polls;    // polls of a wait on another CTA's progress (dataflow producer flags)
    int branch_op;          // op block holding the evaluated branch's matrices (= total ops)
};

// ---- TMA bulk copies and mbarriers (inline PTX, sm_90+ forms used on sm_103a) ----
__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// 1-D bulk copy global -> shared, completion counted on the mbarrier (16-byte aligned, size % 16 == 0)
__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// Wait for the mbarrier phase with the given parity; gives up after `limit`
// polls and returns false (the caller reports a timeout instead of hanging).
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, unsigned limit) {
    const unsigned a = smem_u32(bar);
    for (unsigned i = 0; i < limit; i++) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

constexpr unsigned kWaitPolls = 1u << 26;  // ~ seconds of polling before a wait is declared lost
constexpr int kStatusTimeout = 1;

struct MixBufParams {
    int n, ncat, nptn;
    int cpc;          // categories per mixture class (eval of category c: eval + (c / cpc) * n)
    long long ldp;
    const float *theta;
    const double *buffer_scale, *freq, *invar, *eval, *rates, *props;
    double len;
    double *pattern_lh;
    Reduce red;
    int asc_first;    // +ASC: patterns from here on are the unobserved constant ones (nptn: none)
    double *asc_out;  // their (lh, df, ddf) in true scale
};

__device__ __forceinline__ float4 ld4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }

// Exact power-of-two rescale of a pattern's own stores: n 16-byte chunks at
// base + chunk(i) floats. The loads go out eight at a time before their
// stores, so re-reading the row costs one memory latency per eight chunks
// (one load after another's store paid a full round trip per chunk).
template <class Chunk>
__device__ __forceinline__ void rescale_chunks(float *base, int n, float mul, Chunk chunk) {
    for (int i0 = 0; i0 < n; i0 += 8) {
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (i0 + u < n) v[u] = *reinterpret_cast<const float4 *>(base + chunk(i0 + u));
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (i0 + u < n) {
                v[u].x *= mul; v[u].y *= mul; v[u].z *= mul; v[u].w *= mul;
                *reinterpret_cast<float4 *>(base + chunk(i0 + u)) = v[u];
            }
    }
}

// Per-pattern sums over the B = ncat * n eigen-space entries of theta (FP32 in
// memory, row stride ld): s_j = sum_k w_j[k] theta[k] for NW weight rows held
// as FP32 pairs (w = hi + lo, from the FP64 values). Double-float arithmetic:
// each product's rounding error comes from an FMA and each addition's from
// TwoSum (Knuth), so the sums carry about 44 bits; eigen-space terms cancel,
// and plain FP32 sums lose too much for the derivatives. About 11 FP32
// operations per term instead of one FP64 FMA, which GB300 runs ~60x slower.
template <int NW>
__device__ __forceinline__ void theta_sums_df(const float (*whi)[kMaxCat * kMaxStates],
                                              const float (*wlo)[kMaxCat * kMaxStates], const float *th, long long ld,
                                              int B, double (&s)[NW]) {
    float sh[NW], sl[NW];
#pragma unroll
    for (int j = 0; j < NW; j++) sh[j] = sl[j] = 0.f;
    for (int k = 0; k < B; k++) {
        const float t = th[(long long)k * ld];
#pragma unroll
        for (int j = 0; j < NW; j++) {
            // explicitly rounded operations: no contraction into FMAs may
            // change the error terms
            const float ph = __fmul_rn(whi[j][k], t);
            float pl = fmaf(whi[j][k], t, -ph);  // exact error of the product
            pl = fmaf(wlo[j][k], t, pl);
            const float sum = __fadd_rn(sh[j], ph);  // TwoSum(sh, ph)
            const float bp = __fsub_rn(sum, sh[j]);
            const float err = __fadd_rn(__fsub_rn(sh[j], __fsub_rn(sum, bp)), __fsub_rn(ph, bp));
            sh[j] = sum;
            sl[j] = __fadd_rn(sl[j], __fadd_rn(err, pl));
        }
    }
#pragma unroll
    for (int j = 0; j < NW; j++) s[j] = (double)sh[j] + (double)sl[j];
}

__device__ __forceinline__ void mix_warp_reduce(double (&v)[kRedSlots]) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int k = 0; k < kRedSlots; k++) v[k] += __shfl_xor_sync(0xffffffffu, v[k], off);
}

// Block sums -> partials[blockIdx.x]; the last CTA (by ticket) adds all
// partials in CTA order, deterministically, and re-arms the ticket.
__device__ __forceinline__ void mix_grid_reduce(double (&v)[kRedSlots], const Reduce &red) {
    __shared__ double sw[32][kRedSlots];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    mix_warp_reduce(v);
    if (lane == 0)
        for (int k = 0; k < kRedSlots; k++) sw[wid][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        double s[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
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
    double s[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
        for (int k = 0; k < kRedSlots; k++) s[k] += __ldcg(red.partials + (long long)b * kRedSlots + k);
    mix_warp_reduce(s);
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

MixParams mix_params(iqgpu_engine *e, int nops);
// Ops [op0, op0 + nl) of the uploaded list whose children are both tips: true
// when every one is, so the level can run on k_tiptip_level.
bool level_all_tiptip(const iqgpu_engine *e, int op0, int nl);
// One launch for such a level (traverse_mixed.cu).
int launch_tiptip_level(iqgpu_engine *e, const MixParams &P, int op0, int nl);

}  // namespace iqg
