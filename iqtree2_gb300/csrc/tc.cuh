// Tensor-core (tcgen05) building blocks for sm_103a, written as inline PTX.
//
// Operands are K-major, no swizzle: a "core matrix" is 8 rows x 16 bytes
// stored contiguously (128 B, row r at byte 16 r). An operand tile is a grid
// of core matrices described by two byte strides: LBO between core matrices
// that are neighbours along K, SBO between neighbours along M (or N). The
// mixed-precision partial layout stores every (8 patterns x 4 states) block as
// exactly such a core matrix, so a child's partials are an A operand as they
// lie in memory.
//
// Accumulators live in tensor memory (TMEM): for M = 128 and cta_group::1,
// row i of D is TMEM lane i and column j is TMEM column (base + j); warp w of
// the CTA reads lanes 32 (w % 4) .. 32 (w % 4) + 31.
#pragma once

#include <cstdint>

namespace iqg {

// ---- TMEM allocation (executed by one whole warp) ----
__device__ __forceinline__ void tmem_alloc(unsigned smem_dst, unsigned ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_dst), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- ordering of tcgen05 operations across a thread barrier ----
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- descriptors ----
// Shared-memory matrix descriptor: start address, LBO and SBO in 16-byte
// units (14 bits each), descriptor version 1 at bits 46-48, base offset 0,
// relative LBO mode, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(unsigned addr, unsigned lbo, unsigned sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor, kind::tf32: D = F32 (bits 4-5 = 1), A = B = TF32
// (bits 7-9 and 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// Instruction descriptor, kind::f16 with BF16 inputs (A = B = 1) and F32 D.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---- MMA issue (one thread) ----
__device__ __forceinline__ void mma_tf32(unsigned d_taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_taddr),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"((unsigned)accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_bf16(unsigned d_taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_taddr),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"((unsigned)accumulate)
        : "memory");
}
// A from tensor memory (lanes = rows of A, one TF32 element per 32-bit column,
// K step = 8 columns from a_taddr), B from shared memory.
__device__ __forceinline__ void mma_tf32_ts(unsigned d_taddr, unsigned a_taddr, uint64_t bdesc, uint32_t idesc,
                                            bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_taddr),
        "r"(a_taddr), "l"(bdesc), "r"(idesc), "r"((unsigned)accumulate)
        : "memory");
}
// Arrive once on the mbarrier when every tcgen05 operation this thread has
// issued so far is complete.
__device__ __forceinline__ void mma_commit(unsigned long long *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     (unsigned)__cvta_generic_to_shared(bar))
                 : "memory");
}

// ---- TMEM -> registers ----
// Each helper issues the loads and waits for them inside one asm block, so
// no use of the destination registers can be scheduled before the wait.
// 32x32b shape: this thread's lane, N consecutive 32-bit columns from taddr.
__device__ __forceinline__ void tmem_ld4(unsigned taddr, float (&v)[4]) {
    unsigned r[4];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 4; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld4x2(unsigned ta, unsigned tb, float (&a)[4], float (&b)[4]) {
    unsigned r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%8];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%4, %5, %6, %7}, [%9];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "r"(ta), "r"(tb)
        : "memory");
#pragma unroll
    for (int i = 0; i < 4; i++) {
        a[i] = __uint_as_float(r[i]);
        b[i] = __uint_as_float(r[4 + i]);
    }
}
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float (&v)[16]) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// 20 consecutive columns of this thread's lane (x16 + x4), waited in the same block.
__device__ __forceinline__ void tmem_ld20(unsigned taddr, float (&v)[20]) {
    unsigned r[20];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%20];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%16, %17, %18, %19}, [%21];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19])
        : "r"(taddr), "r"(taddr + 16u)
        : "memory");
#pragma unroll
    for (int i = 0; i < 20; i++) v[i] = __uint_as_float(r[i]);
}

// 12 consecutive columns (x8 + x4) from each of two addresses, one wait.
__device__ __forceinline__ void tmem_ld12x2(unsigned ta, unsigned tb, float (&a)[12], float (&b)[12]) {
    unsigned r[24];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%24];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%8, %9, %10, %11}, [%25];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%12, %13, %14, %15, %16, %17, %18, %19}, [%26];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%20, %21, %22, %23}, [%27];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23])
        : "r"(ta), "r"(ta + 8u), "r"(tb), "r"(tb + 8u)
        : "memory");
#pragma unroll
    for (int i = 0; i < 12; i++) {
        a[i] = __uint_as_float(r[i]);
        b[i] = __uint_as_float(r[12 + i]);
    }
}
// 8 consecutive columns from each of two addresses, one wait.
__device__ __forceinline__ void tmem_ld8x2(unsigned ta, unsigned tb, float (&a)[8], float (&b)[8]) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%16];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8, %9, %10, %11, %12, %13, %14, %15}, [%17];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(ta), "r"(tb)
        : "memory");
#pragma unroll
    for (int i = 0; i < 8; i++) {
        a[i] = __uint_as_float(r[i]);
        b[i] = __uint_as_float(r[8 + i]);
    }
}

// ---- registers -> TMEM (32x32b: this thread's lane, 8 consecutive columns) ----
__device__ __forceinline__ void tmem_st8(unsigned taddr, const float *v) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
        "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
        "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
        : "memory");
}
// every tcgen05.st this thread issued has completed
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// TF32 split: hi = x rounded to the nearest TF32 value (10 explicit mantissa
// bits; ties away from zero), formed on the bit pattern so that hi is exactly
// representable whatever the tensor core does with low bits; lo = x - hi is
// exact in FP32 and |lo| <= 2^-11 |x|. Rounding (not truncation) makes lo
// zero-mean, so the dropped lo*lo term and the tensor core's handling of lo's
// own low bits leave no systematic bias.
__device__ __forceinline__ float tf32_hi(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// Two floats rounded to BF16 (round to nearest even), packed low = a, high = b.
__device__ __forceinline__ unsigned bf16x2(float a, float b) {
    unsigned v;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(v) : "f"(b), "f"(a));
    return v;
}

// ---- warp-specialised pipelines: non-blocking mbarrier test, plain arrive,
// release/acquire counters in shared memory, a barrier over part of the CTA ----
__device__ __forceinline__ bool mbar_test(unsigned long long *bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"((unsigned)__cvta_generic_to_shared(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"((unsigned)__cvta_generic_to_shared(bar))
                 : "memory");
}
__device__ __forceinline__ void st_release_cta(unsigned *p, unsigned v) {
    asm volatile("st.release.cta.shared::cta.u32 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)), "r"(v)
                 : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// generic-proxy writes acquired from other CTAs, ordered before this thread's
// later TMA (async-proxy) reads of global memory
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
__device__ __forceinline__ unsigned ld_acquire_cta(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.cta.shared::cta.u32 %0, [%1];"
                 : "=r"(v)
                 : "r"((unsigned)__cvta_generic_to_shared(p))
                 : "memory");
    return v;
}
// named barrier 1 over the first `nthreads` threads (whole warps)
__device__ __forceinline__ void bar_sync_part(unsigned nthreads) {
    asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}
// the same barrier, returning whether any participating thread passed true
__device__ __forceinline__ bool bar_or_part(unsigned nthreads, bool flag) {
    unsigned out;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 q, %1, 0;\n\t"
        "bar.red.or.pred p, 1, %2, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(out)
        : "r"((unsigned)flag), "r"(nthreads)
        : "memory");
    return out != 0;
}

// ---- TMA tiled load (tensor map), completion counted on an mbarrier ----
__device__ __forceinline__ void tma_load_3d(void *dst, const void *tmap, int x, int y, int z,
                                            unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(z),
        "r"((unsigned)__cvta_generic_to_shared(bar))
        : "memory");
}

}  // namespace iqg
