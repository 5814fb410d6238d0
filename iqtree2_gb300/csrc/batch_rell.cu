// UFBoot RELL scores on the device.
//
// For every candidate tree t and bootstrap replicate r the RELL log-likelihood
// is sum_ptn lnL_t(ptn) * w_r(ptn), where w_r are the replicate's pattern
// counts (a multinomial resampling of the sites, Alignment::createBootstrapAlignment,
// alignment/alignment.cpp:3795-3830). IQ-TREE evaluates it per replicate with a
// float dot product inside saveCurrentTree (tree/iqtree.cpp:3551-3630,
// tree/phylokernel.h:64-70). Here the replicate weights stay resident in HBM
// and every call is one split-K pass over them (a CTA per 32 replicates x 1024
// patterns, up to 8 trees per pass), with FP32 products, FP64 partial sums
// and a fixed-order reduction over the pattern chunks.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "engine.cuh"

namespace iqg {

constexpr int kRellReps = 32;    // replicates per CTA (4 per warp)
constexpr int kRellChunk = 1024; // patterns per CTA
constexpr int kRellTrees = 8;    // trees per pass

// Split-K product: CTA (x, y) computes, for replicates 32 x .. 32 x + 31 and
// the trees t0 .. t0 + nt - 1, the sums over patterns 1024 y .. 1024 y + 1023
// and writes them to part[y][t][r]. The chunk's pattern lnL (FP64 in memory)
// are staged in shared memory as FP32; each lane multiplies in FP32 over its 32
// patterns (coalesced along the weight rows) and the warp adds the lane sums in
// FP64.
__global__ void __launch_bounds__(256) k_rell_part(const float *__restrict__ w, const double *__restrict__ plh,
                                                   long long plh_ld, int nreps, int t0, int nt, long long ldp,
                                                   int nptn, double *__restrict__ part) {
    __shared__ float Ls[kRellTrees][kRellChunk];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long pc = (long long)blockIdx.y * kRellChunk;
    for (int i = threadIdx.x; i < kRellTrees * kRellChunk; i += blockDim.x) {
        const int t = i / kRellChunk, pp = i % kRellChunk;
        const long long p = pc + pp;
        Ls[t][pp] = (t < nt && p < nptn) ? (float)plh[(long long)(t0 + t) * plh_ld + p] : 0.f;
    }
    __syncthreads();
    for (int q = 0; q < kRellReps / 8; q++) {
        const int r = blockIdx.x * kRellReps + warp * (kRellReps / 8) + q;
        if (r >= nreps) break;  // warp-uniform
        const float *wr = w + (long long)r * ldp + pc;
        float acc[kRellTrees];
#pragma unroll
        for (int t = 0; t < kRellTrees; t++) acc[t] = 0.f;
        for (int pp = lane; pp < kRellChunk; pp += 32) {
            const float wv = (pc + pp < nptn) ? __ldcs(wr + pp) : 0.f;
#pragma unroll
            for (int t = 0; t < kRellTrees; t++) acc[t] = fmaf(wv, Ls[t][pp], acc[t]);
        }
#pragma unroll
        for (int t = 0; t < kRellTrees; t++) {
            double v = (double)acc[t];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0 && t < nt) part[((long long)blockIdx.y * nt + t) * nreps + r] = v;
        }
    }
}

// out[t0 + t][r] = sum over chunks, in chunk order (deterministic).
__global__ void k_rell_reduce(const double *__restrict__ part, int nchunks, int nreps, int t0, int nt,
                              double *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nt * nreps) return;
    double s = 0.0;
    for (int c = 0; c < nchunks; c++) s += part[(long long)c * nt * nreps + i];
    out[(long long)t0 * nreps + i] = s;
}

}  // namespace iqg

using namespace iqg;

namespace {
struct RellBuffers {
    float *w = nullptr;
    double *plh = nullptr, *out = nullptr, *part = nullptr, *h_stage = nullptr;
    int nreps = 0, tcap = 0;
};
std::map<iqgpu_engine *, RellBuffers> g_rell;
std::mutex g_rell_mu;

void rell_free(RellBuffers &b) {
    if (b.w) cudaFree(b.w);
    if (b.plh) cudaFree(b.plh);
    if (b.out) cudaFree(b.out);
    if (b.part) cudaFree(b.part);
    if (b.h_stage) cudaFreeHost(b.h_stage);
    b = RellBuffers();
}
}  // namespace

namespace iqg {
void rell_release(iqgpu_engine *e) {
    std::lock_guard<std::mutex> lock(g_rell_mu);
    auto it = g_rell.find(e);
    if (it != g_rell.end()) {
        rell_free(it->second);
        g_rell.erase(it);
    }
}
}  // namespace iqg

#define CKR(call)                                                 \
    do {                                                          \
        cudaError_t err__ = (call);                               \
        if (err__ != cudaSuccess) return cuda_fail(err__, #call); \
    } while (0)

extern "C" int iqgpu_set_boot_weights(iqgpu_engine *e, const float *weights, int32_t nreps) {
    if (!e || !weights || nreps < 1) {
        set_error("bad argument");
        return IQGPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_rell_mu);
    RellBuffers &b = g_rell[e];
    CKR(cudaSetDevice(e->dev));
    CKR(cudaStreamSynchronize(e->st));
    rell_free(b);  // every buffer is sized by the replicate count
    const size_t bytes = (size_t)nreps * e->Ppad * 4;
    size_t free_b = 0, total_b = 0;
    CKR(cudaMemGetInfo(&free_b, &total_b));
    if (bytes > free_b) {
        set_error("admission refused: bootstrap weights need " + std::to_string(bytes) + " bytes");
        return IQGPU_ERR_OOM;
    }
    CKR(cudaMalloc(&b.w, bytes));
    CKR(cudaMemsetAsync(b.w, 0, bytes, e->st));
    CKR(cudaMemcpy2DAsync(b.w, (size_t)e->Ppad * 4, weights, (size_t)e->P * 4, (size_t)e->P * 4, (size_t)nreps,
                          cudaMemcpyHostToDevice, e->st));
    CKR(cudaStreamSynchronize(e->st));
    b.nreps = nreps;
    return IQGPU_OK;
}

namespace {
// Scores of ntrees pattern-lnL vectors (device, row stride plh_ld) against
// every replicate into b.out [ntrees][nreps] (device).
int rell_launch(iqgpu_engine *e, RellBuffers &b, const double *d_plh, long long plh_ld, int ntrees) {
    const int nchunks = (int)((e->P + kRellChunk - 1) / kRellChunk);
    const size_t part_bytes = (size_t)nchunks * kRellTrees * b.nreps * 8;
    if (!b.part) CKR(cudaMalloc(&b.part, part_bytes));
    for (int t0 = 0; t0 < ntrees; t0 += kRellTrees) {
        const int nt = std::min(kRellTrees, ntrees - t0);
        dim3 grid((b.nreps + kRellReps - 1) / kRellReps, nchunks);
        k_rell_part<<<grid, 256, 0, e->st>>>(b.w, d_plh, plh_ld, b.nreps, t0, nt, e->Ppad, (int)e->P, b.part);
        e->launches++;
        CKR(cudaGetLastError());
        const long long n = (long long)nt * b.nreps;
        k_rell_reduce<<<(unsigned)((n + 255) / 256), 256, 0, e->st>>>(b.part, nchunks, b.nreps, t0, nt, b.out);
        e->launches++;
        CKR(cudaGetLastError());
    }
    return IQGPU_OK;
}

int rell_buffers(iqgpu_engine *e, RellBuffers &b, int ntrees) {
    if (b.tcap < ntrees) {
        if (b.plh) cudaFree(b.plh);
        if (b.out) cudaFree(b.out);
        if (b.h_stage) cudaFreeHost(b.h_stage);
        b.plh = b.out = b.h_stage = nullptr;
        CKR(cudaMalloc(&b.plh, (size_t)ntrees * e->P * 8));
        CKR(cudaMalloc(&b.out, (size_t)ntrees * b.nreps * 8));
        CKR(cudaMallocHost(&b.h_stage, (size_t)ntrees * e->P * 8));
        b.tcap = ntrees;
    }
    return IQGPU_OK;
}
}  // namespace

extern "C" int iqgpu_rell(iqgpu_engine *e, const double *pattern_lh, int32_t ntrees, double *out) {
    if (!e || !pattern_lh || !out || ntrees < 1) {
        set_error("bad argument");
        return IQGPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_rell_mu);
    auto it = g_rell.find(e);
    if (it == g_rell.end() || !it->second.w) {
        set_error("set the bootstrap weights first (iqgpu_set_boot_weights)");
        return IQGPU_ERR_STATE;
    }
    RellBuffers &b = it->second;
    CKR(cudaSetDevice(e->dev));
    int rc = rell_buffers(e, b, ntrees);
    if (rc) return rc;
    // pattern lnL go up in FP64 through a cached pinned buffer; the products run
    // in FP32 like the reference's float RELL
    std::memcpy(b.h_stage, pattern_lh, (size_t)ntrees * e->P * 8);
    CKR(cudaMemcpyAsync(b.plh, b.h_stage, (size_t)ntrees * e->P * 8, cudaMemcpyHostToDevice, e->st));
    if ((rc = rell_launch(e, b, b.plh, e->P, ntrees))) return rc;
    CKR(cudaMemcpyAsync(out, b.out, (size_t)ntrees * b.nreps * 8, cudaMemcpyDeviceToHost, e->st));
    CKR(cudaStreamSynchronize(e->st));
    return IQGPU_OK;
}

// RELL scores of the tree whose lnL was computed last (its pattern lnL are
// still on the device), against every replicate: the per-tree step of
// UFBoot's saveCurrentTree (tree/iqtree.cpp:3551-3630) without a host copy.
extern "C" int iqgpu_rell_current(iqgpu_engine *e, double *out) {
    if (!e || !out) {
        set_error("bad argument");
        return IQGPU_ERR_ARG;
    }
    if (e->asc_n > 0) {
        set_error("+ASC engines: pass iqgpu_get_pattern_lh's corrected values to iqgpu_rell");
        return IQGPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_rell_mu);
    auto it = g_rell.find(e);
    if (it == g_rell.end() || !it->second.w) {
        set_error("set the bootstrap weights first (iqgpu_set_boot_weights)");
        return IQGPU_ERR_STATE;
    }
    RellBuffers &b = it->second;
    CKR(cudaSetDevice(e->dev));
    int rc = rell_buffers(e, b, 1);
    if (rc) return rc;
    if ((rc = rell_launch(e, b, e->d_plh, e->Ppad, 1))) return rc;
    CKR(cudaMemcpyAsync(out, b.out, (size_t)b.nreps * 8, cudaMemcpyDeviceToHost, e->st));
    CKR(cudaStreamSynchronize(e->st));
    return IQGPU_OK;
}
