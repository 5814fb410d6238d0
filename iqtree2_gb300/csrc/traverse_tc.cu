// Mixed-precision path, part 3: the pattern-node update on the tensor cores
// (tcgen05, split-TF32 in three passes) for 20- and 61-state models.
//
// For one op, one rate category c and one internal child, the update is a
// small GEMM over a tile of 128 patterns:
//     D[p][x] = sum_y A[p][y] * P_c[x][y]        (M = 128, N = NP, K = KP)
// A is the child's partial block of category c. In the partial layout every
// (8 patterns x 4 states) block is one contiguous 128-byte core matrix, so a
// tile's category-c slice is 16 row groups of npad/4 core matrices: the K-major
// operand the MMA reads, with LBO = 128 B and SBO = npad * 32 B. When npad is
// not a multiple of the K step (npad = 20, K padded to 24), the last K step
// reads one core matrix past the category: the next row group's first chunk
// (or a zeroed pad after the last group), multiplied by the zero columns
// 20..23 of B. B = P_c(t) is prepared once per op in core-matrix order
// (k_tc_prep_b), N padded to 32 or 64 (columns >= n of D are never read).
//
// Split TF32: x = hi + lo with hi = x rounded to TF32 (exact) and lo = x - hi
// (exact in FP32); D = A_lo B_hi + A_hi B_lo + A_hi B_hi, accumulated in FP32
// in tensor memory, which carries the product to about FP32 accuracy (the
// dropped A_lo B_lo term is below 2^-22 of it and has zero mean).
//
// Pipeline per CTA (128 threads, one pattern row per thread): the child slices
// are "stages" (item, category, side). Thread 0 keeps up to NSTAGE stages in
// flight, each one tiled TMA copy of the A slice (tensor map over all slots)
// and one bulk copy of B, into a ring of shared-memory slots; every thread
// converts its own row of a landed stage into hi/lo, thread 0 issues the MMAs
// and commits them to the slot's mbarrier (slot reuse) and, after the last
// side of a category, to the category parity's mbarrier. While the MMAs of
// category c run, each thread reads its row of category c-1 (tcgen05.ld),
// multiplies the children, stores the outputs and keeps the running maximum;
// after the last category it applies the exact power-of-two rescale and
// writes the pattern's exponent. Accumulators are double-buffered by
// category parity (4 * NP TMEM columns).
//
// Two schedules, as on the CUDA cores: fused (a CTA walks the level-ordered op
// list for its pattern tile; a stage whose child is written by an op of the
// same CTA that has not finished yet waits until it has) and level-synchronous
// (one launch per tree level; a grid of resident CTAs strides over the level's
// (tile, op) pairs, so copies for the next pair overlap the current one).
//
// Every wait is bounded: a copy or an MMA that does not complete sets the
// engine's status word; the CTA then waits (bounded) for what it has in
// flight, releases its tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "mixed.cuh"
#include "tc.cuh"

namespace iqg {

constexpr int kTcRows = 128;  // patterns per tile = MMA M

struct TcParams {
    MixParams M;
    const float *tcb;      // per op: [child 2][cat C][hi, lo][NP*KP] core-matrix order
    long long tcb_stride;  // floats per op
    int kq;                // npad / 4 core matrices per category
    int kp;                // K padded to the TF32 K step (8)
    int ksplit;            // stages per (category, side): K is split into ksplit pieces
    int kqs;               // core matrices of A per stage = kq / ksplit
    int kps;               // K per stage = kp / ksplit
    int ksteps;            // MMA K steps per stage = kps / 8
    int a_bytes;           // one FP32 A buffer: 16 * kqs * 128 + 128 (pad)
    int b_bytes;           // one B buffer (TF32: hi or lo, NP * kps * 4; BF16: NP * kpb * 2)
    int kpb;               // BF16: K per stage padded to 16
    int a2_off;            // second A buffer in a slot: TF32 lo, or the BF16 operand
    int b_off;             // B in a slot
    int b_total;           // bytes of B per stage (TF32: hi + lo)
    int slot_bytes;        // TF32 [A hi (copied, rounded in place)][A lo][B hi][B lo];
                           // BF16 [A as copied][A bf16][B bf16]
    long long b_stage;     // floats between consecutive stages' B blocks in tcb
    int ntiles;            // Ppad / 128
    int groups_per_slot;   // Ppad / 8 (third coordinate of the partial tensor map)
};

struct TcItem {
    int k, tile, dad, lref, rref, lch;  // lch: original child index of the left side (after the tip-left swap)
    int cat;                            // the item's one rate category (category-split items), else -1
    bool lint, rint;
    int prod0, prod1;                   // dataflow: uploaded-list index of the op writing each child, or -1
};

constexpr int kTcOpCache = 128;  // ops whose (dad, child0, child1) are staged in shared memory

// Item j of this CTA. Fused: every op of the (level-ordered) list for pattern
// tile blockIdx.x. Level: (tile, op) pairs of one level, strided over the
// grid, tiles of the same op adjacent (their B operands share L2 lines).
// Category-split (csplit): (tile, op, category) triples, the categories of a
// pair on adjacent CTAs; the last of them to finish applies the rescale.
// Per tile (ntl > 0): this CTA's ntl tiles blockIdx.x + t * gridDim.x, each
// through every op of the launch, ops in level order and the tiles of an op
// adjacent (item j = (op, tile t) with t = j % ntl).
__device__ __forceinline__ TcItem tc_item(const TcParams &T, int j, bool fused, int op0, const int4 *opc,
                                          bool csplit = false, int flow_id = -1, int ntl = 0) {
    const MixParams &P = T.M;
    TcItem it;
    it.cat = -1;
    it.prod0 = it.prod1 = -1;
    if (flow_id >= 0) {  // dataflow ticket: (op, tile[, category]) in level order
        if (csplit) it.cat = flow_id % P.ncat;
        const int i = csplit ? flow_id / P.ncat : flow_id;
        it.tile = i % T.ntiles;
        it.k = op0 + i / T.ntiles;
        const OpDev &od = P.ops[it.k];
        it.prod0 = od.prod0;
        it.prod1 = od.prod1;
    } else if (fused) {
        it.k = j;
        it.tile = blockIdx.x;
    } else if (ntl > 0) {
        it.tile = (int)blockIdx.x + (j % ntl) * (int)gridDim.x;
        it.k = op0 + j / ntl;
        const OpDev &od = P.ops[it.k];
        it.prod0 = od.prod0;
        it.prod1 = od.prod1;
    } else {
        int i = blockIdx.x + j * gridDim.x;
        if (csplit) {
            it.cat = i % P.ncat;
            i /= P.ncat;
        }
        it.tile = i % T.ntiles;
        it.k = op0 + i / T.ntiles;
    }
    const int ci = it.k - (fused ? 0 : op0);
    if (ci < kTcOpCache) {
        const int4 o = opc[ci];
        it.dad = o.x;
        it.lref = o.y;
        it.rref = o.z;
    } else {
        const OpDev op = P.ops[it.k];
        it.dad = op.dad_slot;
        it.lref = op.child[0];
        it.rref = op.child[1];
    }
    it.lch = 0;
    if (it.lref >= 0 && it.rref < 0) {  // the tip goes on the left (tree/phylokernelnew.h:1390-1400)
        int t = it.lref; it.lref = it.rref; it.rref = t;
        it.lch = 1;
    }
    it.lint = it.lref >= 0;
    it.rint = it.rref >= 0;
    return it;
}

// stages of an item: for each category, the internal sides in order L, R,
// each in ksplit pieces of K
__device__ __forceinline__ int tc_nstages(const TcItem &it, int C, int ksplit) {
    return (it.cat >= 0 ? 1 : C) * ((int)it.lint + (int)it.rint) * ksplit;
}
__device__ __forceinline__ void tc_stage(const TcItem &it, int st, int ksplit, int &c, int &side, int &kh) {
    const int per = (int)it.lint + (int)it.rint;
    c = it.cat >= 0 ? it.cat : st / (per * ksplit);
    const int rem = st % (per * ksplit);
    side = per == 2 ? rem / ksplit : (it.lint ? 0 : 1);
    kh = rem % ksplit;
}

// This thread's row of a landed stage: TF32 hi in place and lo beside it, or
// the BF16 operand (zero beyond the category's states).
template <bool BF>
__device__ __forceinline__ void tc_convert_row(const TcParams &T, int r, float *ah, unsigned char *a2) {
    const int kqs = T.kqs;
    const int base = (r >> 3) * kqs * 32 + (r & 7) * 4;
    if constexpr (BF) {
        const int nch = T.kpb / 8;
        uint4 *dst = reinterpret_cast<uint4 *>(a2 + (r >> 3) * nch * 128 + (r & 7) * 16);
        for (int j = 0; j < nch; j++) {
            const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 v0 = 2 * j < kqs ? *reinterpret_cast<const float4 *>(ah + base + 2 * j * 32) : z;
            const float4 v1 = 2 * j + 1 < kqs ? *reinterpret_cast<const float4 *>(ah + base + (2 * j + 1) * 32) : z;
            dst[j * 8] = make_uint4(bf16x2(v0.x, v0.y), bf16x2(v0.z, v0.w), bf16x2(v1.x, v1.y), bf16x2(v1.z, v1.w));
        }
    } else {
        float *al = reinterpret_cast<float *>(a2);
        for (int q = 0; q < kqs; q++) {
            const float4 v = *reinterpret_cast<const float4 *>(ah + base + q * 32);
            const float4 h = make_float4(tf32_hi(v.x), tf32_hi(v.y), tf32_hi(v.z), tf32_hi(v.w));
            *reinterpret_cast<float4 *>(ah + base + q * 32) = h;
            *reinterpret_cast<float4 *>(al + base + q * 32) = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
        }
    }
}

// One stage's MMAs into accumulator d (one thread): three split-TF32 passes
// per K step, or one BF16 pass; the first K step of the first piece starts the
// accumulation.
template <int NP, bool BF>
__device__ __forceinline__ void tc_stage_mmas(const TcParams &T, unsigned d, unsigned char *slot, int kh) {
    const unsigned ub = smem_u32(slot + T.b_off);
    if constexpr (BF) {
        const uint32_t idesc = idesc_bf16(kTcRows, NP);
        const unsigned ua = smem_u32(slot + T.a2_off), sbo = (unsigned)(T.kpb / 8 * 128);
        for (int ks = 0; ks < T.kpb / 16; ks++)
            mma_bf16(d, smem_desc(ua + ks * 256, 128, sbo), smem_desc(ub + ks * 256, 128, sbo), idesc,
                     ks > 0 || kh > 0);
    } else {
        const uint32_t idesc = idesc_tf32(kTcRows, NP);
        const unsigned a_sbo = (unsigned)(T.kqs * 128), b_sbo = (unsigned)(T.kps / 4 * 128);
        const unsigned uah = smem_u32(slot), ual = smem_u32(slot + T.a2_off);
        const unsigned ubl = ub + (unsigned)T.b_bytes;
        for (int ks = 0; ks < T.ksteps; ks++) {
            const uint64_t dah = smem_desc(uah + ks * 256, 128, a_sbo);
            const uint64_t dal = smem_desc(ual + ks * 256, 128, a_sbo);
            const uint64_t dbh = smem_desc(ub + ks * 256, 128, b_sbo);
            const uint64_t dbl = smem_desc(ubl + ks * 256, 128, b_sbo);
            mma_tf32(d, dal, dbh, idesc, ks > 0 || kh > 0);
            mma_tf32(d, dah, dbl, idesc, true);
            mma_tf32(d, dah, dbh, idesc, true);
        }
    }
}

// BF: one BF16 pass (kind::f16, FP32 accumulate) instead of three TF32 passes.
template <int NP, int NSTAGE, bool BF>
__global__ void __launch_bounds__(kTcRows, 1) k_traverse_tc(const __grid_constant__ CUtensorMap tmA, const TcParams T,
                                                         const int op0, const int nl, const int fused_nops) {
    const MixParams &P = T.M;
    const int C = P.ncat, n = P.n, npad = P.npad, kq = T.kq;
    const int r = threadIdx.x, warp = r >> 5;
    const long long ld = P.ldp;
    const bool fused = fused_nops > 0;
    int nitems;
    if (fused) {
        nitems = fused_nops;
    } else {
        const int total = T.ntiles * nl;
        nitems = (int)blockIdx.x < total ? (total - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;
    }
    const long long PM = (long long)C * n * npad;
    const long long TB = (long long)(P.state_unknown + 1) * C * npad;
    const int kqs = T.kqs, ksplit = T.ksplit;
    const int a_raw = 16 * kqs * 128;  // one stage's A slice as copied
    const unsigned stage_tx = (unsigned)(a_raw + T.b_total);

    extern __shared__ __align__(128) unsigned char tc_smem_raw[];
    // full: slot filled by TMA; mmab: the slot's MMAs complete; ebar: a
    // category's MMAs complete (by category parity)
    __shared__ unsigned long long full[NSTAGE], mmab[NSTAGE], ebar[2];
    __shared__ unsigned tmem_base_s;
    __shared__ int4 opc[kTcOpCache];
    // tiled TMA destinations want 128-byte alignment: round the dynamic base up (128 B spare requested)
    unsigned char *const tc_smem = tc_smem_raw + ((128u - (smem_u32(tc_smem_raw) & 127u)) & 127u);
    auto slot_at = [&](int s) { return tc_smem + s * T.slot_bytes; };

    // pads after each slot's TF32 A buffers must hold finite values (zero)
    if (!BF) {
        for (int i = r; i < NSTAGE * 2 * 32; i += kTcRows) {
            float *pad = (float *)(slot_at(i / 64) + ((i / 32) & 1) * T.a2_off + a_raw);
            pad[i & 31] = 0.f;
        }
    }
    {
        const int base = fused ? 0 : op0, cnt = fused ? fused_nops : nl;
        for (int i = r; i < cnt && i < kTcOpCache; i += kTcRows) {
            const OpDev op = P.ops[base + i];
            opc[i] = make_int4(op.dad_slot, op.child[0], op.child[1], 0);
        }
    }
    if (r == 0) {
        for (int s = 0; s < NSTAGE; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&mmab[s], 1);
        }
        mbar_init(&ebar[0], 1);
        mbar_init(&ebar[1], 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(smem_u32(&tmem_base_s), 4 * NP);
        tmem_relinquish();
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = tmem_base_s;
    const unsigned lane_off = (unsigned)(warp * 32) << 16;

    // ---- issue side (thread 0 only) ----
    int iss_item = 0, iss_st = 0;  // next stage to issue
    int issued = 0, consumed = 0, finalized = 0;
    bool failed = false;
    TcItem iss_it;
    if (r == 0 && nitems > 0) iss_it = tc_item(T, 0, fused, op0, opc);

    auto next_issue_item = [&]() {
        iss_item++;
        iss_st = 0;
        if (iss_item < nitems) iss_it = tc_item(T, iss_item, fused, op0, opc);
    };
    // Issue stages while ring slots are free. `ahead` bounds the stages in
    // flight beyond the consumed ones: NSTAGE - 1 right after an MMA commit (so
    // the slot to refill is the one whose MMAs were committed a stage earlier),
    // NSTAGE when every committed MMA is known to be complete.
    auto try_issue = [&](int ahead) {
        if (r != 0 || failed) return;
        while (iss_item < nitems && iss_st >= tc_nstages(iss_it, C, ksplit)) next_issue_item();
        while (iss_item < nitems && issued < consumed + ahead) {
            int c, side, kh;
            tc_stage(iss_it, iss_st, ksplit, c, side, kh);
            const int child = side == 0 ? iss_it.lref : iss_it.rref;
            if (fused) {  // a child written by an op of this CTA that has not finished yet
                for (int j = finalized; j < iss_item; j++)
                    if ((j < kTcOpCache ? opc[j].x : P.ops[j].dad_slot) == child) return;
            }
            const int s = issued % NSTAGE;
            if (issued >= NSTAGE) {  // the slot's previous stage must be out of the tensor cores
                if (!mbar_wait(&mmab[s], (unsigned)((issued / NSTAGE - 1) & 1), kWaitPolls)) {
                    failed = true;
                    return;
                }
            }
            unsigned char *slot = slot_at(s);
            mbar_expect_tx(&full[s], stage_tx);
            // A: 16 row groups x kqs core matrices of category c, K piece kh (one tiled copy)
            tma_load_3d(slot, &tmA, 0, c * kq + kh * kqs, child * T.groups_per_slot + iss_it.tile * 16, &full[s]);
            const int ch = side == 0 ? iss_it.lch : 1 - iss_it.lch;
            const float *bsrc =
                T.tcb + (long long)iss_it.k * T.tcb_stride + (long long)((ch * C + c) * ksplit + kh) * T.b_stage;
            tma_load_1d(slot + T.b_off, bsrc, (unsigned)T.b_total, &full[s]);
            issued++;
            iss_st++;
            while (iss_item < nitems && iss_st >= tc_nstages(iss_it, C, ksplit)) next_issue_item();
        }
    };

    int ecount0 = 0, ecount1 = 0;  // commits made to ebar[0], ebar[1]
    bool abort = false;
    try_issue(NSTAGE);

    // products of category c for this thread's pattern; running maximum in cmax
    auto epilogue = [&](const TcItem &it, int c, float *dad, long long p, const float *TL, int sl, int sr,
                        float &cmax) -> bool {
        const int per = (int)it.lint + (int)it.rint;
        const float *tl = it.lint ? nullptr : TL + (long long)sl * C * npad + c * npad;
        const float *tr = it.rint ? nullptr : TL + (it.lch ? -TB : TB) + (long long)sr * C * npad + c * npad;
        if (per > 0) {
            const int ec = (c & 1) ? ecount1 : ecount0;
            const bool ok = mbar_wait(&ebar[c & 1], (unsigned)((ec - 1) & 1), kWaitPolls);
            if (__syncthreads_or(!ok)) return false;
            tc_fence_after();
        }
        const unsigned dL = tmem + lane_off + (unsigned)((c & 1) * 2 * NP), dR = dL + NP;
        float *out = dad + (p >> 3) * (8LL * C * npad) + (p & 7) * 4 + (long long)c * kq * 32;
        for (int q = 0; q < kq; q++) {
            float lv[4], rv[4];
            if (it.lint && it.rint) {
                tmem_ld4x2(dL + 4 * q, dR + 4 * q, lv, rv);
            } else if (it.rint) {
                tmem_ld4(dR + 4 * q, rv);
                const float4 t4 = ld4(tl + 4 * q);
                lv[0] = t4.x; lv[1] = t4.y; lv[2] = t4.z; lv[3] = t4.w;
            } else {
                const float4 a4 = ld4(tl + 4 * q), b4 = ld4(tr + 4 * q);
                lv[0] = a4.x; lv[1] = a4.y; lv[2] = a4.z; lv[3] = a4.w;
                rv[0] = b4.x; rv[1] = b4.y; rv[2] = b4.z; rv[3] = b4.w;
            }
            float o[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                o[i] = (4 * q + i < n) ? lv[i] * rv[i] : 0.f;
                cmax = fmaxf(cmax, o[i]);
            }
            *reinterpret_cast<float4 *>(out + q * 32) = make_float4(o[0], o[1], o[2], o[3]);
        }
        tc_fence_before();
        return true;
    };

    for (int j = 0; j < nitems && !abort; j++) {
        const TcItem it = tc_item(T, j, fused, op0, opc);
        const long long p = (long long)it.tile * kTcRows + r;
        // per-pattern inputs of the item, loaded up front so their latency overlaps the stages
        const int sl = it.lint ? 0 : P.states[(long long)(-1 - it.lref) * ld + p];
        const int sr = it.rint ? 0 : P.states[(long long)(-1 - it.rref) * ld + p];
        const int e_in = (it.lint ? P.expo[(long long)it.lref * ld + p] : 0) +
                         (it.rint ? P.expo[(long long)it.rref * ld + p] : 0);
        const int per = (int)it.lint + (int)it.rint;
        const float *TL = P.opmats + (long long)it.k * P.op_stride + 2 * PM + (it.lch ? TB : 0);
        float *dad = P.part + (long long)it.dad * P.slot_floats;
        float cmax = 0.f;
        for (int c = 0; c < C && !abort; c++) {
            // ---- this category's stages: convert to hi/lo, MMAs ----
            for (int sk = 0; sk < per * ksplit; sk++) {
                const int sd = sk / ksplit, kh = sk % ksplit;
                const bool last = sk == per * ksplit - 1;
                const int side = per == 2 ? sd : (it.lint ? 0 : 1);
                const int s = consumed % NSTAGE;
                const bool ok = mbar_wait(&full[s], (unsigned)((consumed / NSTAGE) & 1), kWaitPolls);
                float *ah = reinterpret_cast<float *>(slot_at(s));
                unsigned char *a2 = slot_at(s) + T.a2_off;
                if (ok) tc_convert_row<BF>(T, r, ah, a2);
                fence_proxy_async_smem();
                if (__syncthreads_or(!ok || (r == 0 && failed))) { abort = true; break; }
                if (r == 0) {
                    tc_fence_after();
                    const unsigned d = tmem + (unsigned)((c & 1) * 2 * NP + side * NP);
                    tc_stage_mmas<NP, BF>(T, d, slot_at(s), kh);
                    mma_commit(&mmab[s]);
                    if (last) mma_commit(&ebar[c & 1]);
                }
                if (last) {
                    if (c & 1) ecount1++;
                    else ecount0++;
                }
                consumed++;
                try_issue(NSTAGE - 1);
            }
            if (abort) break;
            // ---- the previous category's outputs, while this one's MMAs run ----
            if (c > 0 && !epilogue(it, c - 1, dad, p, TL, sl, sr, cmax)) { abort = true; break; }
        }
        if (abort) break;
        if (!epilogue(it, C - 1, dad, p, TL, sl, sr, cmax)) { abort = true; break; }
        // ---- rescale (exact power of two) and exponent ----
        int sh = 0;
        if (cmax < kMixThreshold && cmax > 0.f) {
            int ex;
            frexpf(cmax, &ex);
            sh = 1 - ex;
            const float mul = __int_as_float((127 + sh) << 23);
            float *row = dad + (p >> 3) * (8LL * C * npad) + (p & 7) * 4;
            for (int q = 0; q < C * kq; q++) {
                float4 v = *reinterpret_cast<float4 *>(row + q * 32);
                v.x *= mul; v.y *= mul; v.z *= mul; v.w *= mul;
                *reinterpret_cast<float4 *>(row + q * 32) = v;
            }
        }
        P.expo[(long long)it.dad * ld + p] = e_in - sh;
        if (fused) {
            // the outputs may be read next by this CTA's TMA copies (async proxy)
            asm volatile("fence.proxy.async.global;" ::: "memory");
            __syncthreads();
            finalized = j + 1;
        }
        try_issue(NSTAGE);
    }

    if (r == 0 && (abort || failed)) {
        atomicExch(P.status, kStatusTimeout);
        // bounded waits for the copies and MMAs still in flight before the memory is released
        for (int i = consumed; i < issued; i++) mbar_wait(&full[i % NSTAGE], (unsigned)((i / NSTAGE) & 1), kWaitPolls);
        if (consumed > 0)
            mbar_wait(&mmab[(consumed - 1) % NSTAGE], (unsigned)(((consumed - 1) / NSTAGE) & 1), kWaitPolls);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 4 * NP);
}

// ---------------------------------------------------------------------------
// Warp-specialised form of the level schedule. Warps 0-3 ("workers", one
// pattern row per thread) convert landed stages and run the epilogues; warp 4
// lane 0 ("issuer") keeps the copies and the MMAs going on its own:
//  * it refills a ring slot the moment the slot's previous MMAs complete
//    (mmab), instead of after the next stage's conversion;
//  * it issues a stage's MMAs as soon as all 128 workers have converted it
//    (conv mbarrier, 128 arrivals) and, for the first stage of a category,
//    once the workers have read out the category that last used the same
//    accumulator buffer (epi_done counter, release/acquire in shared memory).
// Categories are numbered g = item * CI + c over the CTA's items (CI = ncat
// categories per item, or 1 for category-split items); buffer g % NACC holds
// category g (NACC = 2; NACC = 1 halves the tensor memory of a CTA, for
// category-split items only, which read out each item before the next one's
// MMAs start). Workers synchronise among themselves only with a 128-thread
// named barrier per category epilogue. Every wait is bounded; a wait that
// gives up raises the shared abort flag and the status word.
// csplit: items are (tile, op, category) triples (narrow levels: ncat times
// the parallelism); an item stores its category's products unscaled and the
// category's per-pattern maximum in cmax[(op - op0) * ncat + c][pattern]; the
// item that completes a (tile, op) pair applies the rescale and writes the
// exponents.
//
// FLOW (dataflow schedule): one launch for the ops [op0, op0 + nl) of several
// levels. The issuer takes (op, tile, category) items (CSPLIT) or whole
// (op, tile) items from a global ticket in level order and passes their ids to the
// workers through a shared-memory FIFO; it issues an item's copies once the
// (op, tile) pairs writing its internal children have raised their flags in
// flow_done (polled without blocking, so the MMAs of earlier items keep
// going), and the workers acquire the same flags before reading the
// children's exponents. The item that completes a pair raises the pair's
// flag after its rescale (a whole item raises it after its own). Tickets go only to running CTAs in increasing
// order and every producer has a smaller ticket, so every wait ends whatever
// the residency; the waits are bounded all the same.
constexpr int kFlowFifo = 8;  // item ids between the issuer and the workers

template <int NP, int NSTAGE, bool BF, bool CSPLIT, bool FLOW = false, int NACC = 2>
__global__ void __launch_bounds__(kTcRows + 32, 4)
    k_traverse_tc_ws(const __grid_constant__ CUtensorMap tmA, const TcParams T, const int op0, const int nl,
                     float *__restrict__ cmax_out, unsigned *__restrict__ pair_cnt,
                     unsigned *__restrict__ flow_done, unsigned *__restrict__ ticket, const unsigned epoch) {
    static_assert(NACC == 2 || (NACC == 1 && CSPLIT),
                  "one accumulator buffer needs category-split items: a whole item converts category g's "
                  "stages before reading out g - 1, which a single buffer would stall");
    constexpr bool csplit = CSPLIT;
    const MixParams &P = T.M;
    const int C = P.ncat, n = P.n, npad = P.npad, kq = T.kq;
    const int CI = csplit ? 1 : C;
    const int tid = threadIdx.x, warp = tid >> 5;
    const bool worker = tid < kTcRows;
    const long long ld = P.ldp;
    const int total = T.ntiles * nl * (csplit ? C : 1);
    const int nitems =
        (int)blockIdx.x < total ? (total - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;
    const long long PM = (long long)C * n * npad;
    const long long TB = (long long)(P.state_unknown + 1) * C * npad;
    const int kqs = T.kqs, ksplit = T.ksplit;
    const int a_raw = 16 * kqs * 128;
    const unsigned stage_tx = (unsigned)(a_raw + T.b_total);

    extern __shared__ __align__(128) unsigned char tc_smem_raw[];
    __shared__ unsigned long long full[NSTAGE], conv[NSTAGE], mmab[NSTAGE], ebar[2];
    __shared__ unsigned tmem_base_s, epi_done, abort_flag;
    __shared__ bool s_last;
    __shared__ int4 opc[kTcOpCache];
    __shared__ int fifo_id[kFlowFifo];
    __shared__ unsigned fifo_seq[kFlowFifo], fifo_taken;
    const int flow_first = op0 + P.op_base;  // producers below it finished before this launch
    unsigned char *const tc_smem = tc_smem_raw + ((128u - (smem_u32(tc_smem_raw) & 127u)) & 127u);
    auto slot_at = [&](int s) { return tc_smem + s * T.slot_bytes; };

    if (!BF) {
        for (int i = tid; i < NSTAGE * 2 * 32; i += blockDim.x) {
            float *pad = (float *)(slot_at(i / 64) + ((i / 32) & 1) * T.a2_off + a_raw);
            pad[i & 31] = 0.f;
        }
    }
    for (int i = tid; i < nl && i < kTcOpCache; i += blockDim.x) {
        const OpDev op = P.ops[op0 + i];
        opc[i] = make_int4(op.dad_slot, op.child[0], op.child[1], 0);
    }
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&conv[s], kTcRows);
            mbar_init(&mmab[s], 1);
        }
        mbar_init(&ebar[0], 1);
        mbar_init(&ebar[1], 1);
        epi_done = 0;
        abort_flag = 0;
        for (int i = 0; i < kFlowFifo; i++) fifo_seq[i] = 0;
        fifo_taken = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(smem_u32(&tmem_base_s), NACC * 2 * NP);
        tmem_relinquish();
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // a level launched as a programmatic dependent of the one before reads its
    // outputs only after this wait (the op records were uploaded before both)
    pdl_wait();
    pdl_trigger();
    const unsigned tmem = tmem_base_s;

    // producers' flags of an item, polled once each (issuer) or waited for (workers)
    auto flow_ready = [&](const TcItem &it) -> bool {
        const int pr[2] = {it.prod0, it.prod1};
        for (int q = 0; q < 2; q++)
            if (pr[q] >= flow_first && ld_acquire_gpu(flow_done + (long long)pr[q] * T.ntiles + it.tile) != epoch)
                return false;
        return true;
    };
    auto flow_wait = [&](const TcItem &it) -> bool {
        const int pr[2] = {it.prod0, it.prod1};
        for (int q = 0; q < 2; q++) {
            if (pr[q] < flow_first) continue;
            const unsigned *f = flow_done + (long long)pr[q] * T.ntiles + it.tile;
            unsigned polls = 0;
            while (ld_acquire_gpu(f) != epoch)
                if (++polls >= P.wait_polls || *(volatile unsigned *)&abort_flag || *(volatile int *)P.status != 0)
                    return false;
        }
        return true;
    };
    if (!worker && FLOW) {
        // ---------------- issuer, dataflow ----------------
        if ((tid & 31) == 0) {
            TcItem fit[kFlowFifo];
            bool fready[kFlowFifo];
            int nf = 0;  // items taken
            bool exhausted = false;
            int ti = 0, ts = 0, issued = 0;  // copy cursor
            int mi = 0, ms = 0, mdone = 0;   // MMA cursor
            unsigned idle = 0;
            auto push = [&](int id) {
                fifo_id[nf % kFlowFifo] = id;
                st_release_cta(&fifo_seq[nf % kFlowFifo], (unsigned)(nf + 1));
            };
            for (;;) {
                bool progress = false;
                // copies: as far ahead as the ring allows, in item order, each item once its producers are done
                while (issued < mdone + NSTAGE) {
                    const int s = issued % NSTAGE;
                    if (issued >= NSTAGE && !mbar_test(&mmab[s], (unsigned)((issued / NSTAGE - 1) & 1))) break;
                    if (ti == nf) {  // take the next ticket once the workers have read the FIFO entry it reuses
                        // (and never over an item the MMA cursor has not passed)
                        if (exhausted || nf - mi >= kFlowFifo || nf - (int)ld_acquire_cta(&fifo_taken) >= kFlowFifo)
                            break;
                        const int id = (int)atomicAdd(ticket, 1u);
                        if (id >= total) {
                            exhausted = true;
                            push(-1);
                            break;
                        }
                        fit[nf % kFlowFifo] = tc_item(T, 0, false, op0, opc, csplit, id);
                        fready[nf % kFlowFifo] = false;
                        push(id);
                        nf++;
                        progress = true;
                    }
                    const TcItem &tit = fit[ti % kFlowFifo];
                    const int nst = tc_nstages(tit, C, ksplit);
                    if (nst == 0) {  // tip-tip item: the workers alone
                        ti++;
                        ts = 0;
                        continue;
                    }
                    if (!fready[ti % kFlowFifo]) {
                        if (!flow_ready(tit)) break;
                        fence_proxy_async_global();
                        fready[ti % kFlowFifo] = true;
                    }
                    int c, side, kh;
                    tc_stage(tit, ts, ksplit, c, side, kh);
                    const int child = side == 0 ? tit.lref : tit.rref;
                    unsigned char *slot = slot_at(s);
                    mbar_expect_tx(&full[s], stage_tx);
                    tma_load_3d(slot, &tmA, 0, c * kq + kh * kqs, child * T.groups_per_slot + tit.tile * 16,
                                &full[s]);
                    const int ch = side == 0 ? tit.lch : 1 - tit.lch;
                    const float *bsrc = T.tcb + (long long)tit.k * T.tcb_stride +
                                        (long long)((ch * C + c) * ksplit + kh) * T.b_stage;
                    tma_load_1d(slot + T.b_off, bsrc, (unsigned)T.b_total, &full[s]);
                    issued++;
                    if (++ts >= nst) {
                        ti++;
                        ts = 0;
                    }
                    progress = true;
                }
                // MMAs of the next converted stage, once its accumulator buffer is free
                while (mi < ti && tc_nstages(fit[mi % kFlowFifo], C, ksplit) == 0) {
                    mi++;
                    ms = 0;
                }
                if (mdone < issued) {
                    const TcItem &mit = fit[mi % kFlowFifo];
                    const int s = mdone % NSTAGE;
                    int c, side, kh;
                    tc_stage(mit, ms, ksplit, c, side, kh);
                    const int per = (int)mit.lint + (int)mit.rint;
                    const int sk = ms % (per * ksplit);
                    const int g = mi * CI + (csplit ? 0 : c);
                    const bool first = sk == 0, last = sk == per * ksplit - 1;
                    if (mbar_test(&conv[s], (unsigned)((mdone / NSTAGE) & 1)) &&
                        (!first || g < NACC || ld_acquire_cta(&epi_done) >= (unsigned)(g - NACC + 1))) {
                        tc_fence_after();
                        const unsigned d = tmem + (unsigned)((g % NACC) * 2 * NP + side * NP);
                        tc_stage_mmas<NP, BF>(T, d, slot_at(s), kh);
                        mma_commit(&mmab[s]);
                        if (last) mma_commit(&ebar[g % NACC]);
                        mdone++;
                        if (++ms >= tc_nstages(mit, C, ksplit)) {
                            mi++;
                            ms = 0;
                        }
                        progress = true;
                    }
                }
                if (exhausted && ti >= nf && mdone == issued) break;
                if (progress) {
                    idle = 0;
                } else if (__nanosleep(64), ++idle >= kWaitPolls / 16 || *(volatile unsigned *)&abort_flag) {
                    if (idle >= kWaitPolls / 16) {
                        atomicExch(&abort_flag, 1u);
                        atomicExch(P.status, kStatusTimeout);
                    }
                    break;
                }
            }
            for (int i = mdone; i < issued; i++) mbar_wait(&full[i % NSTAGE], (unsigned)((i / NSTAGE) & 1), kWaitPolls);
            if (mdone > 0)
                mbar_wait(&mmab[(mdone - 1) % NSTAGE], (unsigned)(((mdone - 1) / NSTAGE) & 1), kWaitPolls);
        }
        __syncwarp();
    } else if (!worker) {
        // ---------------- issuer ----------------
        if ((tid & 31) == 0 && nitems > 0) {
            int ti = 0, ts = 0, issued = 0;  // copy cursor: item, stage within item, stages issued
            int mi = 0, ms = 0, mdone = 0;   // MMA cursor
            TcItem tit = tc_item(T, 0, false, op0, opc, csplit), mit = tit;
            auto skip = [&](int &item, int &st, TcItem &it) {
                while (item < nitems && st >= tc_nstages(it, C, ksplit)) {
                    item++;
                    st = 0;
                    if (item < nitems) it = tc_item(T, item, false, op0, opc, csplit);
                }
            };
            skip(ti, ts, tit);
            skip(mi, ms, mit);
            unsigned idle = 0;
            while (mi < nitems) {
                bool progress = false;
                // copies: as far ahead as the ring allows
                while (ti < nitems && issued < mdone + NSTAGE) {
                    const int s = issued % NSTAGE;
                    if (issued >= NSTAGE && !mbar_test(&mmab[s], (unsigned)((issued / NSTAGE - 1) & 1))) break;
                    int c, side, kh;
                    tc_stage(tit, ts, ksplit, c, side, kh);
                    const int child = side == 0 ? tit.lref : tit.rref;
                    unsigned char *slot = slot_at(s);
                    mbar_expect_tx(&full[s], stage_tx);
                    tma_load_3d(slot, &tmA, 0, c * kq + kh * kqs, child * T.groups_per_slot + tit.tile * 16,
                                &full[s]);
                    const int ch = side == 0 ? tit.lch : 1 - tit.lch;
                    const float *bsrc = T.tcb + (long long)tit.k * T.tcb_stride +
                                        (long long)((ch * C + c) * ksplit + kh) * T.b_stage;
                    tma_load_1d(slot + T.b_off, bsrc, (unsigned)T.b_total, &full[s]);
                    issued++;
                    ts++;
                    skip(ti, ts, tit);
                    progress = true;
                }
                // the next stage's MMAs, once converted and its accumulator is free
                {
                    const int s = mdone % NSTAGE;
                    int c, side, kh;
                    tc_stage(mit, ms, ksplit, c, side, kh);
                    const int per = (int)mit.lint + (int)mit.rint;
                    const int sk = ms % (per * ksplit);
                    const int g = mi * CI + (csplit ? 0 : c);
                    const bool first = sk == 0, last = sk == per * ksplit - 1;
                    if (mdone < issued && mbar_test(&conv[s], (unsigned)((mdone / NSTAGE) & 1)) &&
                        (!first || g < NACC || ld_acquire_cta(&epi_done) >= (unsigned)(g - NACC + 1))) {
                        tc_fence_after();
                        const unsigned d = tmem + (unsigned)((g % NACC) * 2 * NP + side * NP);
                        tc_stage_mmas<NP, BF>(T, d, slot_at(s), kh);
                        mma_commit(&mmab[s]);
                        if (last) mma_commit(&ebar[g % NACC]);
                        mdone++;
                        ms++;
                        skip(mi, ms, mit);
                        progress = true;
                    }
                }
                if (progress) {
                    idle = 0;
                } else if (__nanosleep(64), ++idle >= kWaitPolls / 16 || *(volatile unsigned *)&abort_flag) {
                    if (idle >= kWaitPolls / 16) {
                        atomicExch(&abort_flag, 1u);
                        atomicExch(P.status, kStatusTimeout);
                    }
                    break;
                }
            }
            // bounded waits for copies and MMAs still in flight before the memory is released
            for (int i = mdone; i < issued; i++) mbar_wait(&full[i % NSTAGE], (unsigned)((i / NSTAGE) & 1), kWaitPolls);
            if (mdone > 0)
                mbar_wait(&mmab[(mdone - 1) % NSTAGE], (unsigned)(((mdone - 1) / NSTAGE) & 1), kWaitPolls);
        }
        __syncwarp();  // the issuer warp reconverges before the final barrier
    } else {
        // ---------------- workers ----------------
        const int r = tid;
        const unsigned lane_off = (unsigned)(warp * 32) << 16;
        int consumed = 0, ecount[2] = {0, 0};  // commits made to ebar[0], ebar[1]
        bool abort = false;
        auto epilogue = [&](const TcItem &it, int c, int g, float *dad, long long p, const float *TL, int sl, int sr,
                            float &cmax) -> bool {
            const int per = (int)it.lint + (int)it.rint;
            const float *tl = it.lint ? nullptr : TL + (long long)sl * C * npad + c * npad;
            const float *tr = it.rint ? nullptr : TL + (it.lch ? -TB : TB) + (long long)sr * C * npad + c * npad;
            bool ok = !*(volatile unsigned *)&abort_flag;
            if (per > 0 && ok) {
                const int ec = ecount[g % NACC];
                ok = mbar_wait(&ebar[g % NACC], (unsigned)((ec - 1) & 1), kWaitPolls);
            }
            if (bar_or_part(kTcRows, !ok)) return false;  // uniform stop for every worker
            if (per > 0) tc_fence_after();
            const unsigned dL = tmem + lane_off + (unsigned)((g % NACC) * 2 * NP), dR = dL + NP;
            float *out = dad + (p >> 3) * (8LL * C * npad) + (p & 7) * 4 + (long long)c * kq * 32;
            for (int q = 0; q < kq; q++) {
                float lv[4], rv[4];
                if (it.lint && it.rint) {
                    tmem_ld4x2(dL + 4 * q, dR + 4 * q, lv, rv);
                } else if (it.rint) {
                    tmem_ld4(dR + 4 * q, rv);
                    const float4 t4 = ld4(tl + 4 * q);
                    lv[0] = t4.x; lv[1] = t4.y; lv[2] = t4.z; lv[3] = t4.w;
                } else {
                    const float4 a4 = ld4(tl + 4 * q), b4 = ld4(tr + 4 * q);
                    lv[0] = a4.x; lv[1] = a4.y; lv[2] = a4.z; lv[3] = a4.w;
                    rv[0] = b4.x; rv[1] = b4.y; rv[2] = b4.z; rv[3] = b4.w;
                }
                float o[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    o[i] = (4 * q + i < n) ? lv[i] * rv[i] : 0.f;
                    cmax = fmaxf(cmax, o[i]);
                }
                *reinterpret_cast<float4 *>(out + q * 32) = make_float4(o[0], o[1], o[2], o[3]);
            }
            // every worker has read its row of buffer g % NACC: the issuer may reuse it
            tc_fence_before();
            bar_sync_part(kTcRows);
            if (r == 0) st_release_cta(&epi_done, (unsigned)(g + 1));
            return true;
        };
        for (int j = 0; (FLOW || j < nitems) && !abort; j++) {
            TcItem it;
            if constexpr (FLOW) {
                // the next item id from the issuer, then the producers' flags
                const int e = j % kFlowFifo;
                unsigned polls = 0;
                bool ok = true;
                while (ld_acquire_cta(&fifo_seq[e]) != (unsigned)(j + 1))
                    if (*(volatile unsigned *)&abort_flag || ++polls >= kWaitPolls) {
                        ok = false;
                        break;
                    }
                const int id = ok ? fifo_id[e] : -1;
                if (bar_or_part(kTcRows, !ok)) {
                    abort = true;
                    break;
                }
                if (id < 0) break;
                it = tc_item(T, 0, false, op0, opc, csplit, id);
                const bool dep_ok = r != 0 || flow_wait(it);
                if (bar_or_part(kTcRows, !dep_ok)) {  // also: every worker has read the FIFO entry
                    abort = true;
                    break;
                }
                if (r == 0) st_release_cta(&fifo_taken, (unsigned)(j + 1));
            } else {
                it = tc_item(T, j, false, op0, opc, csplit);
            }
            const long long p = (long long)it.tile * kTcRows + r;
            const int sl = it.lint ? 0 : P.states[(long long)(-1 - it.lref) * ld + p];
            const int sr = it.rint ? 0 : P.states[(long long)(-1 - it.rref) * ld + p];
            // (dataflow: written in this launch by other CTAs, read through L2)
            const int e_in = (it.lint ? (FLOW ? __ldcg(P.expo + (long long)it.lref * ld + p)
                                              : P.expo[(long long)it.lref * ld + p])
                                      : 0) +
                             (it.rint ? (FLOW ? __ldcg(P.expo + (long long)it.rref * ld + p)
                                              : P.expo[(long long)it.rref * ld + p])
                                      : 0);
            const int per = (int)it.lint + (int)it.rint;
            const float *TL = P.opmats + (long long)it.k * P.op_stride + 2 * PM + (it.lch ? TB : 0);
            float *dad = P.part + (long long)it.dad * P.slot_floats;
            float cmax = 0.f;
            for (int cc = 0; cc < CI && !abort; cc++) {
                const int c = csplit ? it.cat : cc;
                const int g = j * CI + cc;
                for (int sk = 0; sk < per * ksplit; sk++) {
                    // no barrier per stage: a wait that gives up raises the abort flag, the
                    // stage is skipped, and the next epilogue's vote stops every worker
                    const int s = consumed % NSTAGE;
                    const bool ok = !*(volatile unsigned *)&abort_flag &&
                                    mbar_wait(&full[s], (unsigned)((consumed / NSTAGE) & 1), kWaitPolls);
                    if (ok) {
                        tc_convert_row<BF>(T, r, reinterpret_cast<float *>(slot_at(s)), slot_at(s) + T.a2_off);
                        fence_proxy_async_smem();
                    } else {
                        atomicExch(&abort_flag, 1u);
                    }
                    mbar_arrive(&conv[s]);
                    consumed++;
                }
                if (abort) break;
                if (per > 0) ecount[g % NACC]++;  // category g's last stage commits ebar[g % NACC]
                if (cc > 0 && !epilogue(it, c - 1, g - 1, dad, p, TL, sl, sr, cmax)) { abort = true; break; }
            }
            if (abort) break;
            if (!epilogue(it, csplit ? it.cat : C - 1, j * CI + CI - 1, dad, p, TL, sl, sr, cmax)) {
                abort = true;
                break;
            }
            if constexpr (CSPLIT) {
                // The rescale and the exponent need every category's maximum: the
                // item that completes its (tile, op) pair applies them (last-arriver
                // pattern: fences and one counter per pair, no waiting).
                const long long pair = (long long)(it.k - op0) * T.ntiles + it.tile;
                cmax_out[((long long)(it.k - op0) * C + it.cat) * ld + p] = cmax;
                __threadfence();  // this thread's products and maximum are visible device-wide
                bar_sync_part(kTcRows);
                if (r == 0) s_last = atomicAdd(pair_cnt + pair, 1u) == (unsigned)(C - 1);
                bar_sync_part(kTcRows);
                if (s_last) {
                    __threadfence();
                    float mx = 0.f;
                    for (int cc = 0; cc < C; cc++)
                        mx = fmaxf(mx, __ldcg(cmax_out + ((long long)(it.k - op0) * C + cc) * ld + p));
                    int sh = 0;
                    if (mx < kMixThreshold && mx > 0.f) {
                        int ex;
                        frexpf(mx, &ex);
                        sh = 1 - ex;
                    }
                    // rows that need the rescale, one warp-wide pass per row (lane q: chunks q, q + 32, ...)
                    const int lane = r & 31;
                    unsigned todo = __ballot_sync(0xffffffffu, sh != 0);
                    while (todo) {
                        const int src = __ffs(todo) - 1;
                        todo &= todo - 1;
                        const int shs = __shfl_sync(0xffffffffu, sh, src);
                        const long long ps = p - lane + src;
                        const float mul = __int_as_float((127 + shs) << 23);
                        float *row = dad + (ps >> 3) * (8LL * C * npad) + (ps & 7) * 4;
                        for (int q = lane; q < C * kq; q += 32) {
                            float4 v = __ldcg(reinterpret_cast<const float4 *>(row + q * 32));
                            v.x *= mul; v.y *= mul; v.z *= mul; v.w *= mul;
                            *reinterpret_cast<float4 *>(row + q * 32) = v;
                        }
                    }
                    P.expo[(long long)it.dad * ld + p] = e_in - sh;
                    if (r == 0) pair_cnt[pair] = 0u;  // re-armed for the next level and evaluation
                    if constexpr (FLOW) {  // the pair is complete: raise its flag
                        __threadfence();
                        bar_sync_part(kTcRows);
                        if (r == 0) atomicExch(flow_done + (long long)(it.k + P.op_base) * T.ntiles + it.tile, epoch);
                    }
                }
                continue;
            }
            int sh = 0;
            if (cmax < kMixThreshold && cmax > 0.f) {  // exact power-of-two rescale
                int ex;
                frexpf(cmax, &ex);
                sh = 1 - ex;
                const float mul = __int_as_float((127 + sh) << 23);
                float *row = dad + (p >> 3) * (8LL * C * npad) + (p & 7) * 4;
                for (int q = 0; q < C * kq; q++) {
                    float4 v = *reinterpret_cast<float4 *>(row + q * 32);
                    v.x *= mul; v.y *= mul; v.z *= mul; v.w *= mul;
                    *reinterpret_cast<float4 *>(row + q * 32) = v;
                }
            }
            P.expo[(long long)it.dad * ld + p] = e_in - sh;
            if constexpr (FLOW) {  // the (op, tile) item is complete: raise its flag
                __threadfence();
                bar_sync_part(kTcRows);
                if (r == 0) atomicExch(flow_done + (long long)(it.k + P.op_base) * T.ntiles + it.tile, epoch);
            }
        }
        if (abort && r == 0) {
            atomicExch(&abort_flag, 1u);
            atomicExch(P.status, kStatusTimeout);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, NACC * 2 * NP);
}

// ---------------------------------------------------------------------------
// A in tensor memory (20 states, split TF32, level schedule 4)
// ---------------------------------------------------------------------------
// The shared-memory-operand kernels above move every A byte through shared
// memory about seven times per stage (copy in, conversion read, hi and lo
// writes, and three MMA passes that re-read A for an N of only 32), so shared
// memory, not HBM, bounds them. Here A never touches shared memory: each
// worker thread loads its own pattern row of a category straight from HBM (a
// warp's 32 rows of one 4-state chunk are four whole 128-byte lines), splits
// it into TF32 hi/lo in registers and writes both into tensor memory with
// tcgen05.st (row r = lane r). The issuer runs the MMAs with A read from
// tensor memory and only B = P_c(t) (hi, lo) from shared memory, staged by
// bulk copies up to kTmNB stages ahead.
//
// Stage m = (item, category) of an item with at least one internal child.
// TMEM (256 columns per CTA, two CTAs per SM): accumulators D[m & 1][side] at
// column (m & 1) * 64 + side * 32; A hi of side s at 128 + s * 2 KP, A lo KP
// further. A is single-buffered: workers write stage m's A once the MMAs of
// stage m-1 have completed (mdone), then arrive on conv; the issuer waits for
// conv and the stage's B, issues the MMAs and commits them to mdone and to the
// B slot's empty barrier. Workers read stage m-1's accumulators (epilogue)
// while stage m's MMAs run, and the loads of the next stage's rows are in
// flight meanwhile (two register buffers, used alternately). An item whose
// children are both tips has no stage: its categories come from the leaf
// tables alone.
constexpr int kTmNB = 4;      // B slots
constexpr int kTmKQ = 5;      // 4-state chunks per category (npad = 20)
constexpr int kTmKP = 24;     // K padded to the TF32 K step
constexpr int kTmCols = 256;  // TMEM columns per CTA

__global__ void __launch_bounds__(kTcRows + 32, 2) k_traverse_tc_tm(const TcParams T, const int op0, const int nl) {
    constexpr int KQ = kTmKQ, KP = kTmKP, NP = 32, KSTEPS = KP / 8;
    const MixParams &P = T.M;
    const int C = P.ncat, n = P.n, npad = P.npad;
    const int tid = threadIdx.x, warp = tid >> 5;
    const long long ld = P.ldp;
    const int total = T.ntiles * nl;
    const int nitems =
        (int)blockIdx.x < total ? (total - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;
    const long long PM = (long long)C * n * npad;
    const long long TB = (long long)(P.state_unknown + 1) * C * npad;
    const unsigned bside = (unsigned)T.b_total;  // B hi + lo of one side

    extern __shared__ __align__(128) unsigned char tc_smem_raw[];
    __shared__ unsigned long long bfull[kTmNB], bempty[kTmNB], conv, mdone;
    __shared__ unsigned tmem_base_s, abort_flag;
    __shared__ int4 opc[kTcOpCache];
    unsigned char *const bring = tc_smem_raw + ((128u - (smem_u32(tc_smem_raw) & 127u)) & 127u);

    for (int i = tid; i < nl && i < kTcOpCache; i += blockDim.x) {
        const OpDev op = P.ops[op0 + i];
        opc[i] = make_int4(op.dad_slot, op.child[0], op.child[1], 0);
    }
    if (tid == 0) {
        for (int s = 0; s < kTmNB; s++) {
            mbar_init(&bfull[s], 1);
            mbar_init(&bempty[s], 1);
        }
        mbar_init(&conv, kTcRows);
        mbar_init(&mdone, 1);
        abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(smem_u32(&tmem_base_s), kTmCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = tmem_base_s;

    // (item, category) cursors over the stages: skip items without an internal child
    auto skip_tips = [&](int &j, int &c, TcItem &it) {
        while (j < nitems && !(it.lint || it.rint)) {
            j++;
            c = 0;
            if (j < nitems) it = tc_item(T, j, false, op0, opc);
        }
    };
    auto advance = [&](int &j, int &c, TcItem &it) {
        if (++c == C) {
            c = 0;
            j++;
            if (j < nitems) it = tc_item(T, j, false, op0, opc);
        }
        skip_tips(j, c, it);
    };

    if (warp == kTcRows / 32) {
        // ---------------- issuer ----------------
        if ((tid & 31) == 0 && nitems > 0) {
            const uint32_t idesc = idesc_tf32(kTcRows, NP);
            const unsigned b_sbo = (unsigned)(KP / 4 * 128);
            int bj = 0, bc = 0, mj = 0, mc = 0, bissued = 0, mdone_n = 0;
            TcItem bit = tc_item(T, 0, false, op0, opc), mit = bit;
            skip_tips(bj, bc, bit);
            skip_tips(mj, mc, mit);
            unsigned idle = 0;
            while (mj < nitems) {
                bool progress = false;
                // B of the coming stages, as far ahead as the slots allow
                while (bj < nitems && bissued < mdone_n + kTmNB) {
                    const int s = bissued % kTmNB;
                    if (bissued >= kTmNB && !mbar_test(&bempty[s], (unsigned)((bissued / kTmNB - 1) & 1))) break;
                    unsigned char *slot = bring + s * 2 * bside;
                    mbar_expect_tx(&bfull[s], bside * ((unsigned)bit.lint + (unsigned)bit.rint));
                    for (int side = 0; side < 2; side++) {
                        if (!(side == 0 ? bit.lint : bit.rint)) continue;
                        const int ch = side == 0 ? bit.lch : 1 - bit.lch;
                        const float *src =
                            T.tcb + (long long)bit.k * T.tcb_stride + (long long)(ch * C + bc) * T.b_stage;
                        tma_load_1d(slot + side * bside, src, bside, &bfull[s]);
                    }
                    bissued++;
                    advance(bj, bc, bit);
                    progress = true;
                }
                // the next stage's MMAs, once its A is in tensor memory and its B has landed
                if (mdone_n < bissued && mbar_test(&conv, (unsigned)(mdone_n & 1)) &&
                    mbar_test(&bfull[mdone_n % kTmNB], (unsigned)((mdone_n / kTmNB) & 1))) {
                    tc_fence_after();
                    const int s = mdone_n % kTmNB;
                    const unsigned ub = smem_u32(bring + s * 2 * bside);
                    for (int side = 0; side < 2; side++) {
                        if (!(side == 0 ? mit.lint : mit.rint)) continue;
                        const unsigned d = tmem + (unsigned)((mdone_n & 1) * 2 * NP + side * NP);
                        const unsigned ah = tmem + 128u + (unsigned)(side * 2 * KP), al = ah + (unsigned)KP;
                        const unsigned bh = ub + (unsigned)side * bside, bl = bh + bside / 2;
#pragma unroll
                        for (int ks = 0; ks < KSTEPS; ks++) {
                            const uint64_t dbh = smem_desc(bh + ks * 256, 128, b_sbo);
                            const uint64_t dbl = smem_desc(bl + ks * 256, 128, b_sbo);
                            mma_tf32_ts(d, al + 8 * ks, dbh, idesc, ks > 0);
                            mma_tf32_ts(d, ah + 8 * ks, dbl, idesc, true);
                            mma_tf32_ts(d, ah + 8 * ks, dbh, idesc, true);
                        }
                    }
                    mma_commit(&bempty[s]);
                    mma_commit(&mdone);
                    mdone_n++;
                    advance(mj, mc, mit);
                    progress = true;
                }
                if (progress) {
                    idle = 0;
                } else if (__nanosleep(64), ++idle >= kWaitPolls / 16 || *(volatile unsigned *)&abort_flag) {
                    if (idle >= kWaitPolls / 16) {
                        atomicExch(&abort_flag, 1u);
                        atomicExch(P.status, kStatusTimeout);
                    }
                    break;
                }
            }
            // bounded waits for the copies and MMAs still in flight before the memory is released
            for (int i = mdone_n; i < bissued; i++)
                mbar_wait(&bfull[i % kTmNB], (unsigned)((i / kTmNB) & 1), kWaitPolls);
            if (mdone_n > 0)
                mbar_wait(&bempty[(mdone_n - 1) % kTmNB], (unsigned)(((mdone_n - 1) / kTmNB) & 1), kWaitPolls);
        }
        __syncwarp();
    } else {
        // ---------------- workers: one pattern row each ----------------
        const int r = tid;
        const unsigned lane_off = (unsigned)(warp * 32) << 16;
        float4 bufA[2][KQ], bufB[2][KQ];
        int m = 0;  // stages whose A this thread has written
        bool abort = false;

        // load cursor: the next stage whose rows are not requested yet
        int lj = 0, lc = 0;
        TcItem lit = tc_item(T, 0, false, op0, opc);
        if (nitems > 0) skip_tips(lj, lc, lit);
        auto load = [&](float4 (&b)[2][KQ]) {
            if (lj >= nitems) return;
            const long long p = (long long)lit.tile * kTcRows + r;
            const long long off = (p >> 3) * (8LL * C * npad) + (p & 7) * 4 + (long long)lc * KQ * 32;
            if (lit.lint) {
                const float *s = P.part + (long long)lit.lref * P.slot_floats + off;
#pragma unroll
                for (int q = 0; q < KQ; q++) b[0][q] = __ldcg(reinterpret_cast<const float4 *>(s + q * 32));
            }
            if (lit.rint) {
                const float *s = P.part + (long long)lit.rref * P.slot_floats + off;
#pragma unroll
                for (int q = 0; q < KQ; q++) b[1][q] = __ldcg(reinterpret_cast<const float4 *>(s + q * 32));
            }
            advance(lj, lc, lit);
        };

        // the item being computed
        int j = 0, c = 0, sl = 0, sr = 0, e_in = 0;
        long long p = 0;
        TcItem it{};
        const float *TL = nullptr;
        float *row = nullptr;  // this pattern's output block in the dad slot
        float cmax = 0.f;
        auto begin_item = [&]() {
            it = tc_item(T, j, false, op0, opc);
            p = (long long)it.tile * kTcRows + r;
            sl = it.lint ? 0 : P.states[(long long)(-1 - it.lref) * ld + p];
            sr = it.rint ? 0 : P.states[(long long)(-1 - it.rref) * ld + p];
            e_in = (it.lint ? P.expo[(long long)it.lref * ld + p] : 0) +
                   (it.rint ? P.expo[(long long)it.rref * ld + p] : 0);
            TL = P.opmats + (long long)it.k * P.op_stride + 2 * PM + (it.lch ? TB : 0);
            row = P.part + (long long)it.dad * P.slot_floats + (p >> 3) * (8LL * C * npad) + (p & 7) * 4;
            cmax = 0.f;
        };
        // category cc of the current item: internal sides from accumulator buffer pb
        auto epilogue = [&](int cc, int pb) {
            float lv[4 * KQ], rv[4 * KQ];
            if (it.lint) {
                tmem_ld20(tmem + lane_off + (unsigned)(pb * 2 * NP), lv);
            } else {
                const float *tl = TL + (long long)sl * C * npad + cc * npad;
#pragma unroll
                for (int q = 0; q < KQ; q++) {
                    const float4 t4 = ld4(tl + 4 * q);
                    lv[4 * q] = t4.x; lv[4 * q + 1] = t4.y; lv[4 * q + 2] = t4.z; lv[4 * q + 3] = t4.w;
                }
            }
            if (it.rint) {
                tmem_ld20(tmem + lane_off + (unsigned)(pb * 2 * NP + NP), rv);
            } else {
                const float *tr = TL + (it.lch ? -TB : TB) + (long long)sr * C * npad + cc * npad;
#pragma unroll
                for (int q = 0; q < KQ; q++) {
                    const float4 t4 = ld4(tr + 4 * q);
                    rv[4 * q] = t4.x; rv[4 * q + 1] = t4.y; rv[4 * q + 2] = t4.z; rv[4 * q + 3] = t4.w;
                }
            }
            float *out = row + (long long)cc * KQ * 32;
#pragma unroll
            for (int q = 0; q < KQ; q++) {
                float o[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    o[i] = (4 * q + i < n) ? lv[4 * q + i] * rv[4 * q + i] : 0.f;
                    cmax = fmaxf(cmax, o[i]);
                }
                *reinterpret_cast<float4 *>(out + q * 32) = make_float4(o[0], o[1], o[2], o[3]);
            }
        };
        auto finish_item = [&]() {
            int sh = 0;
            if (cmax < kMixThreshold && cmax > 0.f) {  // exact power-of-two rescale
                int ex;
                frexpf(cmax, &ex);
                sh = 1 - ex;
                const float mul = __int_as_float((127 + sh) << 23);
                for (int q = 0; q < C * KQ; q++) {
                    float4 v = *reinterpret_cast<float4 *>(row + q * 32);
                    v.x *= mul; v.y *= mul; v.z *= mul; v.w *= mul;
                    *reinterpret_cast<float4 *>(row + q * 32) = v;
                }
            }
            P.expo[(long long)it.dad * ld + p] = e_in - sh;
        };
        // next item with an internal child; items of two tips are completed on the way
        auto begin_next = [&]() -> bool {
            while (j < nitems) {
                begin_item();
                if (it.lint || it.rint) return true;
                for (int cc = 0; cc < C; cc++) epilogue(cc, 0);
                finish_item();
                j++;
            }
            return false;
        };
        // this thread's row of one side into A hi / lo (zero in the K padding)
        auto put_a = [&](const float4 (&v)[KQ], unsigned col) {
            float h[KP], l[KP];
#pragma unroll
            for (int q = 0; q < KQ; q++) {
                const float x[4] = {v[q].x, v[q].y, v[q].z, v[q].w};
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    h[4 * q + i] = tf32_hi(x[i]);
                    l[4 * q + i] = x[i] - h[4 * q + i];
                }
            }
#pragma unroll
            for (int k = 4 * KQ; k < KP; k++) h[k] = l[k] = 0.f;
            const unsigned a = tmem + lane_off + col;
#pragma unroll
            for (int t = 0; t < KSTEPS; t++) {
                tmem_st8(a + 8 * t, &h[8 * t]);
                tmem_st8(a + KP + 8 * t, &l[8 * t]);
            }
        };
        // one stage: `use` holds its rows; the next stage's rows go to `nxt`
        auto stage = [&](float4 (&use)[2][KQ], float4 (&nxt)[2][KQ]) -> bool {
            load(nxt);
            bool ok = m == 0 || (!*(volatile unsigned *)&abort_flag &&
                                 mbar_wait(&mdone, (unsigned)((m - 1) & 1), kWaitPolls));
            if (bar_or_part(kTcRows, !ok)) { abort = true; return false; }
            tc_fence_after();
            if (it.lint) put_a(use[0], 128u);
            if (it.rint) put_a(use[1], 128u + 2 * KP);
            tmem_st_wait();
            tc_fence_before();
            mbar_arrive(&conv);
            if (c > 0) epilogue(c - 1, (m - 1) & 1);
            m++;
            if (c < C - 1) {
                c++;
                return true;
            }
            ok = !*(volatile unsigned *)&abort_flag && mbar_wait(&mdone, (unsigned)((m - 1) & 1), kWaitPolls);
            if (bar_or_part(kTcRows, !ok)) { abort = true; return false; }
            tc_fence_after();
            epilogue(C - 1, (m - 1) & 1);
            finish_item();
            j++;
            c = 0;
            return begin_next();
        };

        load(bufA);
        if (begin_next()) {
            for (;;) {
                if (!stage(bufA, bufB)) break;
                if (!stage(bufB, bufA)) break;
            }
        }
        if (abort && r == 0) {
            atomicExch(&abort_flag, 1u);
            atomicExch(P.status, kStatusTimeout);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, kTmCols);
}

// ---------------------------------------------------------------------------
// Deep-ring level kernel (schedules 8 and 9; 20 states, split TF32)
// ---------------------------------------------------------------------------
// The kernels above hold a shared-memory slot from its copy until its MMAs
// complete and fit two slots per CTA, four CTAs per SM: about eight child
// slices in flight per SM, too few to cover HBM latency at full bandwidth.
// Here one CTA per SM owns the whole shared memory as a ring of kRgNS stages;
// a stage is one (item, category): both children's A slices and both sides'
// B = P_c(t) hi/lo, landed by TMA (32 KB), so six categories (about 120 KB of
// partials) are in flight per SM. Four roles run side by side on different
// stages:
//  * converter warps 0-7: warps 0-3 take the left child's rows of a stage and
//    warps 4-7 the right child's, each thread reading its pattern row from the
//    slice once, splitting it into TF32 hi/lo in registers and writing both
//    into one of kRgNA A buffers in tensor memory with tcgen05.st (A never goes
//    back to shared memory); for an item with one tip child (always on the
//    left after the swap), warps 0-3 write the tip's leaf-table rows into the
//    left accumulator columns instead, which its MMAs leave alone;
//  * a copy warp (16, lane 0) keeps the copies kRgNS stages ahead; MMA warps
//    17 and 18 (lane 0, even and odd stages) run a stage's MMAs (A from
//    tensor memory, B from the slot; the same three
//    passes in the same order as the other split-TF32 kernels, so results are
//    bit-identical) into one of kRgNACC accumulator buffers once the stage is
//    converted and the buffer's previous stage has been read out; their
//    completion frees the slot and the A buffer. (Measured with clock
//    stamps per stage: one thread issuing both the copies and the MMAs took
//    about 2,300 cycles per stage, one thread issuing the MMAs alone about
//    1,700, the 18 MMAs of a stage taking some 800 cycles to issue; with two
//    accumulator buffers an epilogue's pause at an item's end stalled the MMAs
//    two stages later. Separate rings for A (freed on conversion) and B
//    were slower: the copy queue then held far-ahead A slices in front of the
//    B operands the next MMAs needed.)
//  * epilogue warps 8-15: warps 8-11 form the products of states 0-11 of their
//    rows, warps 12-15 of states 12-19; at an item's end the two halves of a
//    row exchange their maxima through shared memory and each rescales its
//    own states; items of two tips are computed here from the leaf tables.
// Warps w, w + 4, w + 8 and w + 12 share tensor-memory lanes 32 (w % 4) ...
// Tensor memory (512 columns): accumulators D[a][side] at a * 64 + side * 32
// (a < kRgNACC); A buffer b, side s: hi at kRgAcol + b * 96 + s * 48, lo 24
// columns further.
// A global load issued where it stands in the program (volatile: the compiler
// neither sinks it to its first use nor merges it).
__device__ __forceinline__ int ld_issue_s32(const int32_t *p) {
    int v;
    asm volatile("ld.global.s32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

constexpr int kRgConv = 256;                // converter threads (warps 0-7)
constexpr int kRgEpi = 256;                 // epilogue threads (warps 8-15)
constexpr int kRgMma = 2;                   // MMA-issuing warps
constexpr int kRgThreads = kRgConv + kRgEpi + 32 * (1 + kRgMma);  // + a copy warp and the MMA warps
constexpr int kRgNS = 6;                    // shared-memory stages
constexpr int kRgNA = 2;                    // A buffers in tensor memory
constexpr int kRgNACC = 4;                  // accumulator buffers in tensor memory
constexpr unsigned kRgAcol = kRgNACC * 64;  // first column of the A buffers
constexpr int kRgA = 16 * kTmKQ * 128;      // one side's A slice as copied (10,240 B)
constexpr int kRgB = 2 * 32 * kTmKP * 4;    // one side's B, hi and lo (6,144 B)
constexpr int kRgSlot = 2 * kRgA + 2 * kRgB;
static_assert(kRgAcol + kRgNA * 96 <= 512, "tensor memory of the ring kernel");

template <bool PER_TILE>
__global__ void __launch_bounds__(kRgThreads, 1)
    k_traverse_tc_ring(const __grid_constant__ CUtensorMap tmA, const TcParams T, const int op0, const int nl) {
    constexpr bool per_tile = PER_TILE;
    constexpr int KQ = kTmKQ, KP = kTmKP, NP = 32, KSTEPS = KP / 8;
    const MixParams &P = T.M;
    const int C = P.ncat, n = P.n, npad = P.npad;
    const int tid = threadIdx.x, warp = tid >> 5;
    const long long ld = P.ldp;
    const int total = T.ntiles * nl;
    // per tile: this CTA's tiles through every op of the launch (a child written
    // in this launch comes from an earlier item of the same CTA)
    const int ntl = !per_tile ? 0
                    : (int)blockIdx.x < T.ntiles ? (T.ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x
                                                 : 0;
    const int nitems = per_tile ? ntl * nl
                       : (int)blockIdx.x < total ? (total - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x
                                                 : 0;
    const long long PM = (long long)C * n * npad;
    const long long TB = (long long)(P.state_unknown + 1) * C * npad;

    extern __shared__ __align__(128) unsigned char tc_smem_raw[];
    // full: a stage landed; mmab: its MMAs complete (slot free); conv: A buffer
    // written by the converters; adone: the A buffer's MMAs complete; ebar: an
    // accumulator buffer holds its stage's products; efree: read out again
    __shared__ unsigned long long full[kRgNS], mmab[kRgNS], conv[kRgNA], adone[kRgNA], ebar[kRgNACC], efree[kRgNACC];
    __shared__ unsigned tmem_base_s, abort_flag, fin_cnt;  // fin_cnt: items written out (per tile)
    __shared__ int4 opc[kTcOpCache];
    __shared__ float rmax[2][2][kTcRows];  // [item parity][half][row]: maxima of the two halves of a row
    unsigned char *const ring = tc_smem_raw + ((128u - (smem_u32(tc_smem_raw) & 127u)) & 127u);

    for (int i = tid; i < nl && i < kTcOpCache; i += blockDim.x) {
        const OpDev op = P.ops[op0 + i];
        opc[i] = make_int4(op.dad_slot, op.child[0], op.child[1], 0);
    }
    if (tid == 0) {
        for (int s = 0; s < kRgNS; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&mmab[s], 1);
        }
        for (int b = 0; b < kRgNA; b++) {
            mbar_init(&conv[b], kRgConv);
            mbar_init(&adone[b], 1);
        }
        for (int a = 0; a < kRgNACC; a++) {
            mbar_init(&ebar[a], 1);
            mbar_init(&efree[a], kRgEpi);
        }
        abort_flag = 0;
        fin_cnt = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(smem_u32(&tmem_base_s), 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // Launched as a programmatic dependent of the previous level: everything
    // above (the op records, uploaded before any level, barriers, tensor
    // memory) overlaps that level's last items; its outputs are read only
    // after this wait, and the next level may be scheduled from here on.
    pdl_wait();
    pdl_trigger();
    const unsigned tmem = tmem_base_s;
    const unsigned lane_off = (unsigned)((warp & 3) * 32) << 16;
    const int r = (warp & 3) * 32 + (tid & 31);  // pattern row of the tile = tensor-memory lane

    // (item, category) cursors over the stages: items of two tips have none
    auto skip_tips = [&](int &j, int &c, TcItem &it) {
        while (j < nitems && !(it.lint || it.rint)) {
            j++;
            c = 0;
            if (j < nitems) it = tc_item(T, j, false, op0, opc, false, -1, ntl);
        }
    };
    auto advance = [&](int &j, int &c, TcItem &it) {
        if (++c == C) {
            c = 0;
            j++;
            if (j < nitems) it = tc_item(T, j, false, op0, opc, false, -1, ntl);
        }
        skip_tips(j, c, it);
    };

    // per tile: the item of this CTA that writes the child on `side`, or -1
    auto producer = [&](const TcItem &x, int j, int side) -> int {
        if (!PER_TILE || !(side == 0 ? x.lint : x.rint)) return -1;
        const int ch = side == 0 ? x.lch : 1 - x.lch;
        const int prod = ch == 0 ? x.prod0 : x.prod1;
        return prod >= op0 + P.op_base ? (prod - P.op_base - op0) * ntl + (ntl > 0 ? j % ntl : 0) : -1;
    };
    auto chained = [&](const TcItem &x, int side) { return producer(x, 0, side) >= 0; };
    constexpr int kWarpCopy = (kRgConv + kRgEpi) / 32, kWarpM = kWarpCopy + 1;
    if (warp == kWarpCopy) {
        // ---------------- copies (lane 0) ----------------
        // A wait that gives up raises the abort flag and the status word; every
        // role then skips its remaining waits and runs to its end.
        if ((tid & 31) == 0 && nitems > 0) {
            int bj = 0, bc = 0, issued = 0;
            TcItem bit = tc_item(T, 0, false, op0, opc, false, -1, ntl);
            skip_tips(bj, bc, bit);
            for (; bj < nitems; issued++) {
                const int s = issued % kRgNS;
                if (issued >= kRgNS) {  // the slot's previous stage is out of the tensor cores
                    if (*(volatile unsigned *)&abort_flag ||
                        !mbar_wait(&mmab[s], (unsigned)((issued / kRgNS - 1) & 1), kWaitPolls)) {
                        atomicExch(&abort_flag, 1u);
                        atomicExch(P.status, kStatusTimeout);
                        break;
                    }
                }
                unsigned char *slot = ring + s * kRgSlot;
                // per tile, a child written by an earlier item of this CTA is read by the
                // converters from global memory, not copied
                const bool chl = chained(bit, 0), chr = chained(bit, 1);
                mbar_expect_tx(&full[s], (unsigned)kRgB * ((unsigned)bit.lint + (unsigned)bit.rint) +
                                             (unsigned)kRgA * ((unsigned)(bit.lint && !chl) + (unsigned)(bit.rint && !chr)));
                for (int side = 0; side < 2; side++) {
                    if (!(side == 0 ? bit.lint : bit.rint)) continue;
                    const int child = side == 0 ? bit.lref : bit.rref;
                    if (!(side == 0 ? chl : chr))
                        tma_load_3d(slot + side * kRgA, &tmA, 0, bc * KQ, child * T.groups_per_slot + bit.tile * 16,
                                    &full[s]);
                    const int ch = side == 0 ? bit.lch : 1 - bit.lch;
                    tma_load_1d(slot + 2 * kRgA + side * kRgB,
                                T.tcb + (long long)bit.k * T.tcb_stride + (long long)(ch * C + bc) * T.b_stage,
                                (unsigned)kRgB, &full[s]);
                }
                advance(bj, bc, bit);
            }
            // the last copies have landed before the shared memory is released
            for (int i = issued > kRgNS ? issued - kRgNS : 0; i < issued; i++)
                mbar_wait(&full[i % kRgNS], (unsigned)((i / kRgNS) & 1), kWaitPolls);
        }
        __syncwarp();
    } else if (warp >= kWarpM) {
        // ---------------- MMAs (lane 0 of kRgMma warps, stages round-robin) ----------------
        // Each barrier still sees its commits in stage order: a stage's gates
        // (conv, efree) complete only after the previous stage using the same A
        // buffer or accumulator buffer has completed.
        const int mw = warp - kWarpM;
        if ((tid & 31) == 0 && nitems > 0) {
            const uint32_t idesc = idesc_tf32(kTcRows, NP);
            const unsigned b_sbo = (unsigned)(KP / 4 * 128);
            int mj = 0, mc = 0, mdone = 0;
            TcItem mit = tc_item(T, 0, false, op0, opc, false, -1, ntl);
            skip_tips(mj, mc, mit);
            for (int i = 0; i < mw && mj < nitems; i++, mdone++) advance(mj, mc, mit);
            for (; mj < nitems; mdone += kRgMma) {
                const int b = mdone % kRgNA, a = mdone % kRgNACC, s = mdone % kRgNS;
                // A converted (the stage landed before that), and the accumulator buffer read out
                if (*(volatile unsigned *)&abort_flag) break;
                if (!mbar_wait(&conv[b], (unsigned)((mdone / kRgNA) & 1), kWaitPolls) ||
                    (mdone >= kRgNACC &&
                     !mbar_wait(&efree[a], (unsigned)((mdone / kRgNACC - 1) & 1), kWaitPolls))) {
                    atomicExch(&abort_flag, 1u);
                    atomicExch(P.status, kStatusTimeout);
                    break;
                }
                tc_fence_after();
                const unsigned ub = smem_u32(ring + s * kRgSlot + 2 * kRgA);
                for (int side = 0; side < 2; side++) {
                    if (!(side == 0 ? mit.lint : mit.rint)) continue;
                    const unsigned d = tmem + (unsigned)(a * 2 * NP + side * NP);
                    const unsigned ah = tmem + kRgAcol + (unsigned)(b * 96 + side * 48), al = ah + (unsigned)KP;
                    const unsigned bh = ub + (unsigned)(side * kRgB), bl = bh + (unsigned)(kRgB / 2);
#pragma unroll
                    for (int ks = 0; ks < KSTEPS; ks++) {
                        const uint64_t dbh = smem_desc(bh + ks * 256, 128, b_sbo);
                        const uint64_t dbl = smem_desc(bl + ks * 256, 128, b_sbo);
                        mma_tf32_ts(d, al + 8 * ks, dbh, idesc, ks > 0);
                        mma_tf32_ts(d, ah + 8 * ks, dbl, idesc, true);
                        mma_tf32_ts(d, ah + 8 * ks, dbh, idesc, true);
                    }
                }
                mma_commit(&mmab[s]);
                mma_commit(&adone[b]);
                mma_commit(&ebar[a]);
                for (int i = 0; i < kRgMma && mj < nitems; i++) advance(mj, mc, mit);
            }
            // this thread's MMAs are complete before the tensor memory is released
            const int last = mdone - kRgMma;
            if (last >= 0) mbar_wait(&mmab[last % kRgNS], (unsigned)((last / kRgNS) & 1), kWaitPolls);
        }
        __syncwarp();
    } else if (warp < kRgConv / 32) {
        // ---------------- converters ----------------
        // A wait that gives up raises the abort flag; every later wait is then
        // skipped (the data is garbage, the status reports the timeout), so
        // every role runs to its end without blocking. For an item with one
        // tip child (always on the left after the swap), warps 0-3 write the
        // tip's leaf-table rows of the stage's category into the left
        // accumulator columns (which its MMAs leave alone) once the epilogue
        // has read that buffer's previous stage: the epilogue then reads both
        // sides from tensor memory and loads nothing per stage.
        const int side = warp >> 2;
        int j = 0, c = 0;
        TcItem it = tc_item(T, 0, false, op0, opc, false, -1, ntl);
        if (nitems > 0) skip_tips(j, c, it);
        int tsl = 0, tj = -1;  // this row's tip state, for item tj
        for (int m = 0; j < nitems; m++) {
            const int s = m % kRgNS, b = m % kRgNA, a = m % kRgNACC;
            const bool tipside = side == 0 && !it.lint;
            const bool mine = side == 0 ? it.lint : it.rint;  // this side has an A slice
            float tv[4 * KQ];
            if (tipside) {
                if (tj != j) {
                    tsl = P.states[(long long)(-1 - it.lref) * ld + (long long)it.tile * kTcRows + r];
                    tj = j;
                }
                const float *tl = P.opmats + (long long)it.k * P.op_stride + 2 * PM + (it.lch ? TB : 0) +
                                  (long long)tsl * C * npad + c * npad;
#pragma unroll
                for (int q = 0; q < KQ; q++) {
                    const float4 t4 = ld4(tl + 4 * q);
                    tv[4 * q] = t4.x; tv[4 * q + 1] = t4.y; tv[4 * q + 2] = t4.z; tv[4 * q + 3] = t4.w;
                }
            }
            // every converter waits for the A buffer's previous stage (its MMAs imply
            // that stage's conv phase is complete, so arrivals never run a phase ahead)
            const int jp = producer(it, j, side);  // per tile: an earlier item writes this child
            bool ok = *(volatile unsigned *)&abort_flag == 0;
            if (ok && mine && jp < 0) ok = mbar_wait(&full[s], (unsigned)((m / kRgNS) & 1), kWaitPolls);
            if (ok && jp >= 0) {  // written out (the epilogue's release after its barrier)
                unsigned polls = 0;
                while ((int)ld_acquire_cta(&fin_cnt) <= jp) {
                    if (*(volatile unsigned *)&abort_flag || ++polls >= kWaitPolls / 8) {
                        ok = false;
                        break;
                    }
                    __nanosleep(32);
                }
            }
            if (ok && m >= kRgNA) ok = mbar_wait(&adone[b], (unsigned)((m / kRgNA - 1) & 1), kWaitPolls);
            if (ok && tipside && m >= kRgNACC)
                ok = mbar_wait(&efree[a], (unsigned)((m / kRgNACC - 1) & 1), kWaitPolls);
            ok = __all_sync(0xffffffffu, ok);  // tcgen05.st is warp-collective
            if (!ok) atomicExch(&abort_flag, 1u);
            if (ok && tipside) {
                tc_fence_after();
                const unsigned ad = tmem + lane_off + (unsigned)(a * 2 * NP);
                float z[8];
#pragma unroll
                for (int i = 0; i < 8; i++) z[i] = i < 4 * KQ - 16 ? tv[16 + i] : 0.f;
                tmem_st8(ad, &tv[0]);
                tmem_st8(ad + 8, &tv[8]);
                tmem_st8(ad + 16, z);
                tmem_st_wait();
            } else if (ok && mine) {
                tc_fence_after();
                const long long pr = (long long)it.tile * kTcRows + r;
                const float *ar = jp >= 0 ? P.part + (long long)(side == 0 ? it.lref : it.rref) * P.slot_floats +
                                                (pr >> 3) * (8LL * C * npad) + (pr & 7) * 4 + (long long)c * KQ * 32
                                          : reinterpret_cast<const float *>(ring + s * kRgSlot + side * kRgA) +
                                                (r >> 3) * KQ * 32 + (r & 7) * 4;
                const unsigned ad = tmem + lane_off + kRgAcol + (unsigned)(b * 96 + side * 48);
#pragma unroll
                for (int t = 0; t < KSTEPS; t++) {  // K step t: states 8t .. 8t + 7 (zero beyond the 20)
                    float h[8], l[8];
#pragma unroll
                    for (int u = 0; u < 2; u++) {
                        const int q = 2 * t + u;
                        const float4 v = q >= KQ ? make_float4(0.f, 0.f, 0.f, 0.f)
                                         : jp >= 0 ? __ldcg(reinterpret_cast<const float4 *>(ar + q * 32))
                                                   : *reinterpret_cast<const float4 *>(ar + q * 32);
                        const float xv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                        for (int i = 0; i < 4; i++) {
                            h[4 * u + i] = tf32_hi(xv[i]);
                            l[4 * u + i] = xv[i] - h[4 * u + i];
                        }
                    }
                    tmem_st8(ad + 8 * t, h);
                    tmem_st8(ad + KP + 8 * t, l);
                }
                tmem_st_wait();
            }
            tc_fence_before();
            mbar_arrive(&conv[b]);
            advance(j, c, it);
        }
    } else {
        // ---------------- epilogue ----------------
        // Both sides of a staged item come from tensor memory (a tip's rows
        // were written there by the converters); the children's exponents are
        // loaded one item ahead. Items of two tips use the leaf tables.
        const int half = (warp - kRgConv / 32) >> 2;
        const int q0 = half ? 3 : 0, nq = half ? KQ - 3 : 3;  // this thread's 4-state chunks
        // (volatile loads: issued here, not sunk to their first use an item later)
        auto expo_in = [&](const TcItem &x, long long px, int &e_l, int &e_r) {
            e_l = (x.lint && half == 0) ? ld_issue_s32(P.expo + (long long)x.lref * ld + px) : 0;
            e_r = (x.rint && half == 0) ? ld_issue_s32(P.expo + (long long)x.rref * ld + px) : 0;
        };
        int m = 0;  // stages read out
        TcItem it = tc_item(T, 0, false, op0, opc, false, -1, ntl);
        long long p = (long long)it.tile * kTcRows + r;
        int e_l = 0, e_r = 0;
        if (nitems > 0) expo_in(it, p, e_l, e_r);
        for (int j = 0; j < nitems; j++) {
            // the next item's exponents, in flight while this one is read out (per tile: a
            // child may be the item just finished, so they are loaded as the item starts)
            TcItem nit = it;
            long long np_ = p;
            int nel = 0, ner = 0;
            if (j + 1 < nitems) {
                nit = tc_item(T, j + 1, false, op0, opc, false, -1, ntl);
                np_ = (long long)nit.tile * kTcRows + r;
                if (!per_tile) expo_in(nit, np_, nel, ner);
            }
            float *row = P.part + (long long)it.dad * P.slot_floats + (p >> 3) * (8LL * C * npad) + (p & 7) * 4;
            const bool staged = it.lint || it.rint;
            const float *TL = P.opmats + (long long)it.k * P.op_stride + 2 * PM + (it.lch ? TB : 0);
            const int sl = staged ? 0 : P.states[(long long)(-1 - it.lref) * ld + p];
            const int sr = staged ? 0 : P.states[(long long)(-1 - it.rref) * ld + p];
            float cmax = 0.f;
            for (int c = 0; c < C; c++) {
                float lv[12], rv[12];
                if (staged) {
                    const int a = m % kRgNACC;
                    if (!*(volatile unsigned *)&abort_flag &&
                        !mbar_wait(&ebar[a], (unsigned)((m / kRgNACC) & 1), kWaitPolls))
                        atomicExch(&abort_flag, 1u);
                    __syncwarp();  // tcgen05.ld is warp-collective
                    tc_fence_after();
                    const unsigned dL = tmem + lane_off + (unsigned)(a * 2 * NP + 4 * q0), dR = dL + NP;
                    if (half == 0) {
                        tmem_ld12x2(dL, dR, lv, rv);
                    } else {
                        float l8[8], r8[8];
                        tmem_ld8x2(dL, dR, l8, r8);
#pragma unroll
                        for (int i = 0; i < 8; i++) {
                            lv[i] = l8[i];
                            rv[i] = r8[i];
                        }
                    }
                    tc_fence_before();
                    mbar_arrive(&efree[a]);  // this thread's reads of buffer a are done
                    m++;
                } else {  // two tips
                    const float *tl = TL + (long long)sl * C * npad + c * npad + 4 * q0;
                    const float *tr = TL + (it.lch ? -TB : TB) + (long long)sr * C * npad + c * npad + 4 * q0;
#pragma unroll
                    for (int q = 0; q < 3; q++)
                        if (q < nq) {
                            const float4 a4 = ld4(tl + 4 * q), b4 = ld4(tr + 4 * q);
                            lv[4 * q] = a4.x; lv[4 * q + 1] = a4.y; lv[4 * q + 2] = a4.z; lv[4 * q + 3] = a4.w;
                            rv[4 * q] = b4.x; rv[4 * q + 1] = b4.y; rv[4 * q + 2] = b4.z; rv[4 * q + 3] = b4.w;
                        }
                }
                float *out = row + (long long)c * KQ * 32 + q0 * 32;
#pragma unroll
                for (int q = 0; q < 3; q++)
                    if (q < nq) {
                        float o[4];
#pragma unroll
                        for (int i = 0; i < 4; i++) {
                            o[i] = (4 * (q0 + q) + i < n) ? lv[4 * q + i] * rv[4 * q + i] : 0.f;
                            cmax = fmaxf(cmax, o[i]);
                        }
                        *reinterpret_cast<float4 *>(out + q * 32) = make_float4(o[0], o[1], o[2], o[3]);
                    }
            }
            // the row maximum over both halves (one vote per item: the epilogue warps stop together),
            // the exact power-of-two rescale and the exponent
            rmax[j & 1][half][r] = cmax;
            if (bar_or_part(kRgEpi, *(volatile unsigned *)&abort_flag != 0)) break;
            const float mx = fmaxf(rmax[j & 1][0][r], rmax[j & 1][1][r]);
            int sh = 0;
            if (mx < kMixThreshold && mx > 0.f) {
                int ex;
                frexpf(mx, &ex);
                sh = 1 - ex;
                const float mul = __int_as_float((127 + sh) << 23);
                // this thread's chunks q0 .. q0 + nq - 1 of every category
                rescale_chunks(row, C * nq, mul, [&](int i) { return ((i / nq) * KQ + q0 + i % nq) * 32; });
            }
            if (half == 0) P.expo[(long long)it.dad * ld + p] = e_l + e_r - sh;
            if (per_tile) {  // the item is written out: later items of this CTA may read it
                bar_sync_part(kRgEpi);
                if (tid == kRgConv) st_release_cta(&fin_cnt, (unsigned)(j + 1));
            }
            it = nit;
            p = np_;
            if (per_tile) {
                if (j + 1 < nitems) expo_in(it, p, e_l, e_r);
            } else {
                e_l = nel;
                e_r = ner;
            }
        }
        if (*(volatile unsigned *)&abort_flag && tid == kRgConv) atomicExch(P.status, kStatusTimeout);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

// B operands: per op, child, category and K piece kh: hi and lo of
// P_c(t)[x][y] for y in piece kh, in [x/8][y'/4][x%8][y'%4] order (y' = y - kh
// KS), zero outside x < n, y < n.
__global__ void k_tc_prep_b(const float *opmats, long long op_stride, float *tcb, long long tcb_stride, int n,
                            int npad, int C, int NP, int KP, int ksplit) {
    pdl_wait();  // the P(t) matrices come from the kernel before
    pdl_trigger();
    const int k = blockIdx.x, ch = blockIdx.y / C, c = blockIdx.y % C;
    const int KS = KP / ksplit;
    const float *Pm = opmats + (long long)k * op_stride + (long long)ch * C * n * npad + (long long)c * n * npad;
    float *blk = tcb + (long long)k * tcb_stride + (long long)((ch * C + c) * ksplit) * 2 * NP * KS;
    for (int i = threadIdx.x; i < NP * KP; i += blockDim.x) {
        const int x = i / KP, y = i % KP;
        const int kh = y / KS, yy = y % KS;
        const float v = (x < n && y < n) ? Pm[x * npad + y] : 0.f;
        const float h = tf32_hi(v);
        float *hi = blk + (long long)kh * 2 * NP * KS;
        const int off = (x >> 3) * (KS / 4) * 32 + (yy >> 2) * 32 + (x & 7) * 4 + (yy & 3);
        hi[off] = h;
        hi[NP * KS + off] = v - h;
    }
}

// BF16 B operands: per op, child, category and K piece kh: P_c(t)[x][y] rounded
// to BF16 for y = kh * KS + yy, in [x/8][yy/8][x%8][yy%8] order (KB = KS padded to
// 16 columns), zero outside x < n, y < n.
__global__ void k_tc_prep_b16(const float *opmats, long long op_stride, unsigned short *tcb, long long stride_h,
                              int n, int npad, int C, int NP, int KS, int KB, int ksplit) {
    const int k = blockIdx.x, ch = blockIdx.y / C, c = blockIdx.y % C;
    const float *Pm = opmats + (long long)k * op_stride + (long long)ch * C * n * npad + (long long)c * n * npad;
    for (int kh = 0; kh < ksplit; kh++) {
        unsigned short *blk = tcb + (long long)k * stride_h + (long long)((ch * C + c) * ksplit + kh) * NP * KB;
        for (int i = threadIdx.x; i < NP * KB; i += blockDim.x) {
            const int x = i / KB, yy = i % KB, y = kh * KS + yy;
            const float v = (x < n && yy < KS && y < n) ? Pm[x * npad + y] : 0.f;
            const int off = (x >> 3) * (KB / 8) * 64 + (yy >> 3) * 64 + (x & 7) * 8 + (yy & 7);
            blk[off] = (unsigned short)(bf16x2(v, 0.f) & 0xFFFFu);
        }
    }
}

int tc_np(int npad) { return npad <= 32 ? 32 : 64; }
int tc_kp(int npad) { return (npad + 7) / 8 * 8; }
// 61-state models: each stage carries half of K (32 states), so a stage is half
// the shared memory and two CTAs fit per SM; needs npad a multiple of 16
// K pieces per stage (iqgpu_set_kpieces): 2 halves a stage's shared memory
// (two 61-state CTAs per SM instead of one) at twice the stages per op; needs
// npad > 32 and a multiple of 16.
int tc_ksplit(const iqgpu_engine *e) {
    if (e->npad <= 32 || e->npad % 16 != 0) return 1;
    return e->tc_kpieces == 4 ? 4 : e->tc_kpieces == 2 ? 2 : 1;
}

int launch_tc_prep(iqgpu_engine *e, int nops) {
    if (nops <= 0) return IQGPU_OK;
    if (e->cfg.precision == IQGPU_BF16) {
        const int NP = tc_np(e->npad), ks = tc_ksplit(e), KS = e->npad / ks, KB = (KS + 15) / 16 * 16;
        k_tc_prep_b16<<<dim3(nops, 2 * e->C), 256, 0, e->st>>>(e->d_opmats32, e->op_stride32,
                                                                 reinterpret_cast<unsigned short *>(e->d_tcb),
                                                                 e->tcb_stride * 2, e->n, e->npad, e->C, NP, KS, KB, ks);
        e->launches++;
        return cuda_fail(cudaGetLastError(), "tc_prep_b16");
    }
    const int NP = tc_np(e->npad), KP = tc_kp(e->npad);
    cudaError_t err = pdl_launch(k_tc_prep_b, dim3(nops, 2 * e->C), dim3(256), 0, e->st, (const float *)e->d_opmats32,
                                 e->op_stride32, e->d_tcb, e->tcb_stride, e->n, e->npad, e->C, NP, KP, tc_ksplit(e));
    e->launches++;
    if (err != cudaSuccess) return cuda_fail(err, "tc_prep_b");
    return cuda_fail(cudaGetLastError(), "tc_prep_b");
}

// Tensor map over all partial slots, viewed as [slot * Ppad/8 + group][C*kq core
// matrices][32 floats]; a box of {32, kq, 16} is one category of a 128-pattern
// tile in the operand layout. Built once per engine (the slots do not move).
static int tc_tensor_map(iqgpu_engine *e) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (err != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
            set_error("cuTensorMapEncodeTiled is not available from the driver");
            return IQGPU_ERR_CUDA;
        }
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const int kq = e->npad / 4, kqs = kq / tc_ksplit(e);
    if (e->tc_tmap_ready && e->tc_tmap_kqs == kqs) return IQGPU_OK;
    const cuuint64_t dims[3] = {32, (cuuint64_t)e->C * kq, (cuuint64_t)e->cfg.nslots * (cuuint64_t)(e->Ppad / 8)};
    const cuuint64_t strides[2] = {128, (cuuint64_t)e->C * kq * 128};
    const cuuint32_t box[3] = {32, (cuuint32_t)kqs, 16};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult res = encode(reinterpret_cast<CUtensorMap *>(e->tc_tmap), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, e->d_part32,
                          dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (res != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed for the partial slots");
        return IQGPU_ERR_CUDA;
    }
    e->tc_tmap_ready = true;
    e->tc_tmap_kqs = kqs;
    return IQGPU_OK;
}

// Stage geometry of the tensor-core kernel for this engine.
static TcParams tc_params(const iqgpu_engine *e, const MixParams &M, int NP, bool BF) {
    TcParams T;
    T.M = M;
    T.tcb = e->d_tcb;
    T.tcb_stride = e->tcb_stride;
    T.kq = e->npad / 4;
    T.kp = tc_kp(e->npad);
    T.ksplit = tc_ksplit(e);
    T.kqs = T.kq / T.ksplit;
    T.kps = T.kp / T.ksplit;
    T.ksteps = T.kps / 8;
    T.a_bytes = 16 * T.kqs * 128 + 128;
    T.kpb = (T.kqs * 4 + 15) / 16 * 16;
    T.a2_off = T.a_bytes;
    if (BF) {  // [A as copied][A bf16][B bf16]
        T.b_off = T.a_bytes + 16 * (T.kpb / 8) * 128;
        T.b_bytes = NP * T.kpb * 2;
        T.b_total = T.b_bytes;
        T.b_stage = (long long)NP * T.kpb / 2;
    } else {   // [A hi][A lo][B hi][B lo]
        T.b_off = 2 * T.a_bytes;
        T.b_bytes = NP * T.kps * 4;
        T.b_total = 2 * T.b_bytes;
        T.b_stage = 2LL * NP * T.kps;
    }
    T.slot_bytes = T.b_off + T.b_total;
    T.ntiles = (int)(e->Ppad / kTcRows);
    T.groups_per_slot = (int)(e->Ppad / 8);
    return T;
}

static size_t tc_smem_bytes(const TcParams &T, int nstage) {
    return (size_t)nstage * T.slot_bytes + 128;  // + alignment spare
}

template <int NP, int NSTAGE, bool BF, int NACC = 2>
static int launch_tc_t(iqgpu_engine *e, const MixParams &M, int *rest) {
    int rc = tc_tensor_map(e);
    if (rc) return rc;
    const TcParams T = tc_params(e, M, NP, BF);
    const CUtensorMap &tm = *reinterpret_cast<const CUtensorMap *>(e->tc_tmap);
    const size_t smem = tc_smem_bytes(T, NSTAGE);
    auto kern = k_traverse_tc<NP, NSTAGE, BF>;
    auto kern_ws = k_traverse_tc_ws<NP, NSTAGE, BF, false>;
    auto kern_ws_cs = k_traverse_tc_ws<NP, NSTAGE, BF, true>;
    auto kern_flow = k_traverse_tc_ws<NP, NSTAGE, BF, true, true, NACC>;
    auto kern_flow_whole = k_traverse_tc_ws<NP, NSTAGE, BF, false, true>;
    const bool split_ok = NP == 64 || e->tc_split;  // 61 states always; fewer states with schedule 5
    const bool ws = e->level_sync && (e->tc_ws || e->tc_tm);  // warp-specialised level kernel
    const int nthr = ws ? kTcRows + 32 : kTcRows;
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err == cudaSuccess && ws)
        err = cudaFuncSetAttribute(kern_ws, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err == cudaSuccess && ws && split_ok)
        err = cudaFuncSetAttribute(kern_ws_cs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // the whole unified L1/shared array as shared memory: residency is set by shared memory
    if (err == cudaSuccess)
        err = ws ? cudaFuncSetAttribute(kern_ws, cudaFuncAttributePreferredSharedMemoryCarveout, 100)
                 : cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (err == cudaSuccess && ws && split_ok)
        err = cudaFuncSetAttribute(kern_ws_cs, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (err == cudaSuccess && ws && split_ok && e->tc_flow)
        err = cudaFuncSetAttribute(kern_flow, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err == cudaSuccess && ws && split_ok && e->tc_flow)
        err = cudaFuncSetAttribute(kern_flow, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (err == cudaSuccess && ws && e->tc_flow_whole)
        err = cudaFuncSetAttribute(kern_flow_whole, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err == cudaSuccess && ws && e->tc_flow_whole)
        err = cudaFuncSetAttribute(kern_flow_whole, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (err != cudaSuccess) return cuda_fail(err, "traverse_tc smem attribute");
    // Residency per SM: bounded by shared memory (dynamic + static + the per-CTA
    // reserve) and by tensor memory (512 columns, 4 * NP per CTA).
    int sms = 1, smem_sm = 0, reserve = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->dev) != cudaSuccess || sms < 1) sms = 1;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, e->dev);
    cudaDeviceGetAttribute(&reserve, cudaDevAttrReservedSharedMemoryPerBlock, e->dev);
    cudaFuncAttributes fa;
    size_t stat = 0;
    int regs = 0;
    if ((NACC == 1 ? cudaFuncGetAttributes(&fa, kern_flow)
                   : ws ? cudaFuncGetAttributes(&fa, kern_ws) : cudaFuncGetAttributes(&fa, kern)) == cudaSuccess) {
        stat = fa.sharedSizeBytes;
        regs = fa.numRegs;
    }
    const size_t per_cta = smem + stat + (size_t)reserve;
    int per_sm = (int)std::min<size_t>(512 / (NACC * 2 * NP), per_cta ? (size_t)smem_sm / per_cta : 1);
    if (regs > 0) {  // and by the register file (allocated per warp in units of 256)
        const int per_warp = ((regs * 32 + 255) / 256) * 256;
        per_sm = std::min(per_sm, 65536 / (per_warp * (nthr / 32)));
    }
    if (per_sm < 1) per_sm = 1;
    const long long resident = (long long)per_sm * sms;
    // Narrow tail: from the first level whose (tile, op) pairs no longer fill
    // the resident CTAs, a tensor-core CTA would hold a single pair and expose
    // its whole stage latency; for up to 32 padded states the fused CUDA-core
    // kernel takes those ops instead (same split in both schedules).
    // Category-split items (warp-specialised kernel): levels with fewer than
    // four (tile, op) pairs per resident CTA run as (tile, op, category)
    // triples, each pair's chain of stages cut into ncat independent ones
    // (61 states only: a 20-state item is 8 short stages and the narrow levels
    // run faster on the CUDA-core tail than split plus the fix-up launch)
    const bool can_split = ws && split_ok && e->d_cmax != nullptr;
    if (ws && e->tc_flow_whole && e->d_flow_done) {
        // Dataflow over whole (op, tile) items: leading tip-tip levels as store
        // streams, then every other op in one launch
        int l = 0;
        for (; l < e->nlevels; l++) {
            const int op0 = e->level_off[l], nl = e->level_off[l + 1] - op0;
            if (nl > 0 && !level_all_tiptip(e, op0, nl)) break;
            if (nl > 0 && (rc = launch_tiptip_level(e, M, op0, nl))) return rc;
        }
        const int op_first = l < e->nlevels ? e->level_off[l] : M.nops;
        const int nflow = M.nops - op_first;
        *rest = M.nops;
        if (nflow <= 0) return IQGPU_OK;
        const long long ntiles = T.ntiles;
        err = cudaMemsetAsync(e->d_flow_done, 0, (size_t)(M.op_base + M.nops) * ntiles * 4, e->st);
        if (err == cudaSuccess) err = cudaMemsetAsync(e->d_flow_ticket, 0, 4, e->st);
        if (err != cudaSuccess) return cuda_fail(err, "flow flag reset");
        const int grid = (int)std::min<long long>((long long)nflow * ntiles, resident);
        kern_flow_whole<<<grid, nthr, smem, e->st>>>(tm, T, op_first, nflow, e->d_cmax, e->d_pair_cnt, e->d_flow_done,
                                                     e->d_flow_ticket, 1u);
        e->launches++;
        return cuda_fail(cudaGetLastError(), "traverse_tc flow");
    }
    if (can_split && e->tc_flow && e->d_flow_done) {
        // Dataflow: leading levels of tip-tip ops as store streams, then every
        // other op in one launch of category-split items (no CUDA-core tail)
        int l = 0;
        for (; l < e->nlevels; l++) {
            const int op0 = e->level_off[l], nl = e->level_off[l + 1] - op0;
            if (nl > 0 && !level_all_tiptip(e, op0, nl)) break;
        }
        const int op_first = l < e->nlevels ? e->level_off[l] : M.nops;
        const int nflow = M.nops - op_first;
        const long long ntiles = T.ntiles;
        // ops per launch: as many as the pair counters and the maxima hold
        const long long window = std::min<long long>(e->pair_cap / ntiles,
                                                     (long long)(e->cmax_bytes / ((size_t)e->C * e->Ppad * 4)));
        if (window >= 1) {
            for (int q = 0; q < l; q++) {
                const int op0 = e->level_off[q], nl = e->level_off[q + 1] - op0;
                if (nl > 0 && (rc = launch_tiptip_level(e, M, op0, nl))) return rc;
            }
            *rest = M.nops;
            if (nflow <= 0) return IQGPU_OK;
            err = cudaMemsetAsync(e->d_flow_done, 0, (size_t)(M.op_base + M.nops) * ntiles * 4, e->st);
            if (err != cudaSuccess) return cuda_fail(err, "flow flag reset");
            for (int w0 = op_first; w0 < M.nops; w0 += (int)window) {
                const int nw = (int)std::min<long long>(window, M.nops - w0);
                if ((err = cudaMemsetAsync(e->d_flow_ticket, 0, 4, e->st)) != cudaSuccess)
                    return cuda_fail(err, "flow ticket reset");
                const long long items = (long long)nw * ntiles * e->C;
                const int grid = (int)std::min<long long>(items, resident);
                kern_flow<<<grid, nthr, smem, e->st>>>(tm, T, w0, nw, e->d_cmax, e->d_pair_cnt, e->d_flow_done,
                                                       e->d_flow_ticket, 1u);
                e->launches++;
                if ((err = cudaGetLastError()) != cudaSuccess) return cuda_fail(err, "traverse_tc flow");
            }
            return IQGPU_OK;
        }
    }
    if constexpr (NACC == 1) {  // the level kernels keep two accumulator buffers
        set_error("one accumulator buffer (four K pieces) runs on the dataflow schedule only");
        return IQGPU_ERR_STATE;
    }
    int lt = e->nlevels;
    if (NP == 32)
        for (int l = 0; l < e->nlevels; l++)
            if ((long long)(e->level_off[l + 1] - e->level_off[l]) * T.ntiles * (can_split ? e->C : 1) < resident) {
                lt = l;
                break;
            }
    *rest = e->nlevels > 0 ? (lt < e->nlevels ? e->level_off[lt] : M.nops) : M.nops;
    if (*rest <= 0) return IQGPU_OK;
    if (!e->level_sync) {
        kern<<<T.ntiles, kTcRows, smem, e->st>>>(tm, T, 0, 0, *rest);
        e->launches++;
        return cuda_fail(cudaGetLastError(), "traverse_tc");
    }
    // level schedule: a persistent grid of resident CTAs walks each level's (tile, op) pairs;
    // a level of tip-tip ops only (no contraction) is a store stream on the CUDA cores
    for (int l = 0; l < lt; l++) {
        const int op0 = e->level_off[l], nl = e->level_off[l + 1] - op0;
        if (nl <= 0) continue;
        if (level_all_tiptip(e, op0, nl)) {
            rc = launch_tiptip_level(e, M, op0, nl);
            if (rc) return rc;
            continue;
        }
        const long long items = (long long)T.ntiles * nl;
        const bool cs = can_split && items < 4 * resident && items <= e->pair_cap &&
                        (size_t)nl * e->C * (size_t)e->Ppad * sizeof(float) <= e->cmax_bytes;
        const int grid = (int)std::min<long long>(items * (cs ? e->C : 1), resident);
        if (ws && cs)
            err = pdl_launch(kern_ws_cs, dim3((unsigned)grid), dim3(nthr), smem, e->st, tm, T, op0, nl, e->d_cmax,
                             e->d_pair_cnt, (unsigned *)nullptr, (unsigned *)nullptr, 1u);
        else if (ws)
            err = pdl_launch(kern_ws, dim3((unsigned)grid), dim3(nthr), smem, e->st, tm, T, op0, nl, e->d_cmax,
                             e->d_pair_cnt, (unsigned *)nullptr, (unsigned *)nullptr, 1u);
        else
            kern<<<grid, kTcRows, smem, e->st>>>(tm, T, op0, nl, 0);
        e->launches++;
        if (err == cudaSuccess) err = cudaGetLastError();
        if (err != cudaSuccess) return cuda_fail(err, "traverse_tc level");
    }
    return IQGPU_OK;
}

// Level schedule on k_traverse_tc_tm (20 states, split TF32). Residency: two
// CTAs per SM by tensor memory (256 columns each), lowered if shared memory or
// registers allow fewer; the narrow tail goes to the CUDA cores as above.
static int launch_tc_tm(iqgpu_engine *e, const MixParams &M, int *rest) {
    const TcParams T = tc_params(e, M, 32, false);
    const size_t smem = (size_t)kTmNB * 2 * T.b_total + 128;
    cudaError_t err = cudaFuncSetAttribute(k_traverse_tc_tm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err == cudaSuccess) err = cudaFuncSetAttribute(k_traverse_tc_tm, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (err != cudaSuccess) return cuda_fail(err, "traverse_tc_tm smem attribute");
    int sms = 1, smem_sm = 0, reserve = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->dev) != cudaSuccess || sms < 1) sms = 1;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, e->dev);
    cudaDeviceGetAttribute(&reserve, cudaDevAttrReservedSharedMemoryPerBlock, e->dev);
    cudaFuncAttributes fa;
    size_t stat = 0;
    int regs = 0;
    if (cudaFuncGetAttributes(&fa, k_traverse_tc_tm) == cudaSuccess) {
        stat = fa.sharedSizeBytes;
        regs = fa.numRegs;
    }
    const int nthr = kTcRows + 32;
    const size_t per_cta = smem + stat + (size_t)reserve;
    int per_sm = (int)std::min<size_t>(512 / kTmCols, per_cta ? (size_t)smem_sm / per_cta : 1);
    if (regs > 0) {
        const int per_warp = ((regs * 32 + 255) / 256) * 256;
        per_sm = std::min(per_sm, 65536 / (per_warp * (nthr / 32)));
    }
    if (per_sm < 1) per_sm = 1;
    const long long resident = (long long)per_sm * sms;
    // narrow tail: levels with fewer than two items per resident CTA (an item
    // is a serial chain of ncat stages, so one item per CTA exposes all of it)
    int lt = e->nlevels;
    for (int l = 0; l < e->nlevels; l++)
        if ((long long)(e->level_off[l + 1] - e->level_off[l]) * T.ntiles < 2 * resident) { lt = l; break; }
    *rest = e->nlevels > 0 ? (lt < e->nlevels ? e->level_off[lt] : M.nops) : M.nops;
    for (int l = 0; l < lt; l++) {
        const int op0 = e->level_off[l], nl = e->level_off[l + 1] - op0;
        if (nl <= 0) continue;
        if (level_all_tiptip(e, op0, nl)) {
            const int rc = launch_tiptip_level(e, M, op0, nl);
            if (rc) return rc;
            continue;
        }
        const long long items = (long long)T.ntiles * nl;
        const int grid = (int)std::min<long long>(items, resident);
        k_traverse_tc_tm<<<grid, nthr, smem, e->st>>>(T, op0, nl);
        e->launches++;
        err = cudaGetLastError();
        if (err != cudaSuccess) return cuda_fail(err, "traverse_tc_tm level");
    }
    return IQGPU_OK;
}

// Level schedule on k_traverse_tc_ring: one CTA per SM (its shared memory
// and its 512 tensor-memory columns). From the first level with fewer than
// three (tile, op) pairs per SM (the one-op levels near the root), schedule 8
// leaves the ops to the CUDA-core tail and schedule 9 runs them in one more
// launch per tile: each CTA takes its tiles through all of those ops in level
// order, waiting only for its own earlier items, with no launch per level.
static int launch_tc_ring(iqgpu_engine *e, const MixParams &M, int *rest) {
    int rc = tc_tensor_map(e);
    if (rc) return rc;
    const TcParams T = tc_params(e, M, 32, false);
    const CUtensorMap &tm = *reinterpret_cast<const CUtensorMap *>(e->tc_tmap);
    const size_t smem = (size_t)kRgNS * kRgSlot + 128;
    cudaError_t err = cudaSuccess;
    for (auto kern : {k_traverse_tc_ring<false>, k_traverse_tc_ring<true>}) {
        if (err == cudaSuccess) err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err == cudaSuccess) err = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    }
    if (err != cudaSuccess) return cuda_fail(err, "traverse_tc_ring smem attribute");
    int sms = 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->dev) != cudaSuccess || sms < 1) sms = 1;
    const long long resident = sms;
    int lt = e->nlevels;
    for (int l = 0; l < e->nlevels; l++)
        if ((long long)(e->level_off[l + 1] - e->level_off[l]) * T.ntiles < 3 * resident) {
            lt = l;
            break;
        }
    const int tail0 = e->nlevels > 0 ? (lt < e->nlevels ? e->level_off[lt] : M.nops) : M.nops;
    for (int l = 0; l < lt; l++) {
        const int op0 = e->level_off[l], nl = e->level_off[l + 1] - op0;
        if (nl <= 0) continue;
        if (level_all_tiptip(e, op0, nl)) {
            rc = launch_tiptip_level(e, M, op0, nl);
            if (rc) return rc;
            continue;
        }
        const long long items = (long long)T.ntiles * nl;
        const int grid = (int)std::min<long long>(items, resident);
        err = pdl_launch(k_traverse_tc_ring<false>, dim3((unsigned)grid), dim3(kRgThreads), smem, e->st, tm, T, op0, nl);
        e->launches++;
        if (err == cudaSuccess) err = cudaGetLastError();
        if (err != cudaSuccess) return cuda_fail(err, "traverse_tc_ring level");
    }
    *rest = tail0;
    if (e->tc_ring_all && tail0 < M.nops) {
        const int grid = (int)std::min<long long>(T.ntiles, resident);
        k_traverse_tc_ring<true><<<grid, kRgThreads, smem, e->st>>>(tm, T, tail0, M.nops - tail0);
        e->launches++;
        err = cudaGetLastError();
        if (err != cudaSuccess) return cuda_fail(err, "traverse_tc_ring per tile");
        *rest = M.nops;
    }
    return IQGPU_OK;
}

template <int NP, bool BF>
static int launch_tc_depth(iqgpu_engine *e, const MixParams &M, int depth, int *rest) {
    if constexpr (NP == 64 && !BF) {
        // four K pieces with one accumulator buffer: the category-split dataflow schedule only
        if (e->tc_flow && tc_ksplit(e) == 4) {
            switch (depth) {
            case 2: return launch_tc_t<NP, 2, BF, 1>(e, M, rest);
            case 3: return launch_tc_t<NP, 3, BF, 1>(e, M, rest);
            default: return launch_tc_t<NP, 4, BF, 1>(e, M, rest);
            }
        }
    }
    switch (depth) {
    case 2: return launch_tc_t<NP, 2, BF>(e, M, rest);
    case 3: return launch_tc_t<NP, 3, BF>(e, M, rest);
    default: return launch_tc_t<NP, 4, BF>(e, M, rest);
    }
}

// Ring depth actually used: the requested one (iqgpu_set_stages; 0 = 2),
// lowered until the CTA's shared memory fits the 227 KB a CTA may use.
int tc_depth(const iqgpu_engine *e) {
    const int NP = tc_np(e->npad);
    const bool BF = e->cfg.precision == IQGPU_BF16;
    MixParams M{};
    const TcParams T = tc_params(e, M, NP, BF);
    int depth = e->tc_stages ? e->tc_stages : 2;
    while (depth > 2 && tc_smem_bytes(T, depth) + 4096 > 227u * 1024u) depth--;
    return depth;
}

// The ops of a traversal on the tensor cores (the narrow tail of a <= 32-state
// traversal and the branch epilogue run on the fused CUDA-core kernel). Per CTA: a ring of `depth` shared-memory slots; the
// residency per SM follows from their size and from the 4 * NP tensor-memory
// columns each CTA holds (depth 2: four CTAs per SM for 20 states, two for 61).
// Sets *rest to the first op left to the CUDA cores (M.nops when none).
int launch_traverse_tc(iqgpu_engine *e, const MixParams &M, int *rest) {
    *rest = M.nops;
    if (M.nops <= 0) return IQGPU_OK;
    const int depth = tc_depth(e);
    const bool BF = e->cfg.precision == IQGPU_BF16;
    if (e->level_sync && e->tc_ring && !BF && e->npad == 4 * kTmKQ && tc_ksplit(e) == 1)
        return launch_tc_ring(e, M, rest);
    if (e->level_sync && e->tc_tm && !BF && e->npad == 4 * kTmKQ && tc_ksplit(e) == 1)
        return launch_tc_tm(e, M, rest);
    if (tc_np(e->npad) == 64)
        return BF ? launch_tc_depth<64, true>(e, M, depth, rest) : launch_tc_depth<64, false>(e, M, depth, rest);
    return BF ? launch_tc_depth<32, true>(e, M, depth, rest) : launch_tc_depth<32, false>(e, M, depth, rest);
}

}  // namespace iqg
