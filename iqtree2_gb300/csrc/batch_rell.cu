// UFBoot RELL scores on the device.
//
// For every candidate tree t and bootstrap replicate r the RELL log-likelihood
// is sum_ptn lnL_t(ptn) * w_r(ptn), where w_r are the replicate's pattern
// counts (a multinomial resampling of the sites, Alignment::createBootstrapAlignment,
// alignment/alignment.cpp:3795-3830). IQ-TREE evaluates it per replicate with a
// float dot product inside saveCurrentTree (tree/iqtree.cpp:3551-3630,
// tree/phylokernel.h:64-70). Here all trees x replicates are one tiled
// product: the replicate weights stay resident in HBM, each CTA computes a
// 64 x 64 (replicate x tree) block from shared-memory tiles with FP32 products,
// and partial sums are folded into FP64 every 256 patterns.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>

#include "engine.cuh"

namespace iqg {

constexpr int kRR = 64, kRT = 64, kRK = 32;  // replicates, trees, patterns per tile

__global__ void __launch_bounds__(256) k_rell(const float *__restrict__ w, const float *__restrict__ plh, int nreps,
                                              int ntrees, long long ldp, int nptn, double *__restrict__ out) {
    __shared__ __align__(16) float Ws[kRK][kRR];
    __shared__ __align__(16) float Ls[kRK][kRT];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int r0 = blockIdx.x * kRR, t0 = blockIdx.y * kRT;
    float acc[4][4];
    double dacc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) { acc[i][j] = 0.f; dacc[i][j] = 0.0; }
    int chunks = 0;
    for (int p0 = 0; p0 < nptn; p0 += kRK) {
        // 64 rows x 32 patterns of each operand: 2048 floats, 8 per thread, coalesced along patterns
        for (int e = threadIdx.x; e < kRK * kRR; e += blockDim.x) {
            const int row = e / kRK, pp = e % kRK;
            const int p = p0 + pp;
            const int r = r0 + row, t = t0 + row;
            Ws[pp][row] = (r < nreps && p < nptn) ? w[(long long)r * ldp + p] : 0.f;
            Ls[pp][row] = (t < ntrees && p < nptn) ? plh[(long long)t * ldp + p] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int pp = 0; pp < kRK; pp++) {
            const float4 a = *reinterpret_cast<const float4 *>(&Ws[pp][tx * 4]);
            const float4 b = *reinterpret_cast<const float4 *>(&Ls[pp][ty * 4]);
            const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
        if (++chunks == 8) {  // fold into FP64 every 256 patterns
            chunks = 0;
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) { dacc[i][j] += (double)acc[i][j]; acc[i][j] = 0.f; }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int r = r0 + tx * 4 + i, t = t0 + ty * 4 + j;
            if (r < nreps && t < ntrees) out[(long long)t * nreps + r] = dacc[i][j] + (double)acc[i][j];
        }
}

}  // namespace iqg

using namespace iqg;

namespace {
struct RellBuffers {
    float *w = nullptr, *plh = nullptr;
    double *out = nullptr;
    int nreps = 0, tcap = 0;
};
std::map<iqgpu_engine *, RellBuffers> g_rell;
std::mutex g_rell_mu;

void rell_free(RellBuffers &b) {
    if (b.w) cudaFree(b.w);
    if (b.plh) cudaFree(b.plh);
    if (b.out) cudaFree(b.out);
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
    if (b.w) cudaFree(b.w);
    b.w = nullptr;
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
    if (b.tcap < ntrees) {
        if (b.plh) cudaFree(b.plh);
        if (b.out) cudaFree(b.out);
        b.plh = nullptr;
        b.out = nullptr;
        CKR(cudaMalloc(&b.plh, (size_t)ntrees * e->Ppad * 4));
        CKR(cudaMalloc(&b.out, (size_t)ntrees * b.nreps * 8));
        b.tcap = ntrees;
    }
    // pattern lnL arrive in FP64; the products run in FP32 like the reference's float RELL
    std::string err;
    {
        float *h = nullptr;
        CKR(cudaMallocHost(&h, (size_t)ntrees * e->Ppad * 4));
        for (long long t = 0; t < ntrees; t++)
            for (long long p = 0; p < e->Ppad; p++) h[t * e->Ppad + p] = p < e->P ? (float)pattern_lh[t * e->P + p] : 0.f;
        cudaError_t ce = cudaMemcpyAsync(b.plh, h, (size_t)ntrees * e->Ppad * 4, cudaMemcpyHostToDevice, e->st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->st);
        cudaFreeHost(h);
        if (ce != cudaSuccess) return cuda_fail(ce, "upload pattern lnL");
    }
    dim3 grid((b.nreps + kRR - 1) / kRR, (ntrees + kRT - 1) / kRT);
    k_rell<<<grid, 256, 0, e->st>>>(b.w, b.plh, b.nreps, ntrees, e->Ppad, (int)e->P, b.out);
    e->launches++;
    CKR(cudaGetLastError());
    CKR(cudaMemcpyAsync(out, b.out, (size_t)ntrees * b.nreps * 8, cudaMemcpyDeviceToHost, e->st));
    CKR(cudaStreamSynchronize(e->st));
    return IQGPU_OK;
}
