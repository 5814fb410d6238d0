// Branch-length derivative sums without any device allocation.
//
// Some callers cannot allocate device memory at the point where they need a
// derivative: a host program whose GPU memory is owned by a pool or arena it
// must not bypass, code running between the kernels of a latency-critical
// pipeline (cudaMalloc and cudaFree synchronise the device), or a caller that
// only holds borrowed device buffers. The regular engine entry points keep a
// per-engine workspace allocated at iqgpu_create; this entry point instead
// takes every input and output as device pointers from the caller and keeps
// its only scratch -- the per-CTA partial sums and the completion ticket of
// the grid reduction -- in one statically sized __device__ array that every
// GPU loading the library holds until the process exits.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "engine.cuh"

namespace iqg {
namespace {

constexpr int kNATPB = 128;                  // patterns per CTA
constexpr int kNAMaxBlocks = 4096;           // scratch rows
constexpr long long kNAMaxPatterns = (long long)kNAMaxBlocks * kNATPB;  // 524,288
constexpr int kNAMaxDevices = 64;

struct NoAllocScratch {
    double partials[kNAMaxBlocks * kRedSlots];  // 128 KiB
    unsigned ticket;
};

// The scratch array: file scope, 256-byte aligned, shared by every call on a device.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

struct NoAllocArgs {
    int n, ncat, nptn;
    long long ldp;
    double len;
    double eval[kMaxStates];
    double rates[kMaxCat];
    double props[kMaxCat];
    const double *theta, *buffer_scale, *freq, *invar;
    double *out;
    NoAllocScratch *scratch;  // device address of g_noalloc_scratch
};

__global__ void __launch_bounds__(kNATPB) k_derv_noalloc(const NoAllocArgs A) {
    __shared__ double v0[kMaxCat * kMaxStates], v1[kMaxCat * kMaxStates], v2[kMaxCat * kMaxStates];
    __shared__ double sw[kNATPB / 32][kRedSlots];
    __shared__ bool last;
    const int n = A.n, C = A.ncat, B = n * C;
    for (int t = threadIdx.x; t < B; t += blockDim.x) {
        const int c = t / n, i = t % n;
        const double cof = A.eval[i] * A.rates[c];
        const double val = exp(cof * A.len) * A.props[c];
        const double val1 = cof * val;
        v0[t] = val;
        v1[t] = val1;
        v2[t] = cof * val1;
    }
    __syncthreads();
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double r[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
    if (p < A.nptn) {
        const double *th = A.theta + p;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        for (int k = 0; k < B; k++) {
            const double t0 = th[(long long)k * A.ldp];
            a0 = fma(v0[k], t0, a0);
            a1 = fma(v1[k], t0, a1);
            a2 = fma(v2[k], t0, a2);
        }
        const double lh = fabs(a0) + A.invar[p];
        const double inv = 1.0 / lh;
        const double df_frac = a1 * inv, ddf_frac = a2 * inv;
        const double f = A.freq[p];
        const double tmp1 = df_frac * f, tmp2 = ddf_frac * f;
        r[0] = tmp1;
        r[1] = fma(-tmp1, df_frac, tmp2);
        r[2] = (log(lh) + A.buffer_scale[p]) * f;
    }
    // CTA sums -> scratch rows; the last CTA to finish adds them in CTA order
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int k = 0; k < kRedSlots; k++) r[k] += __shfl_xor_sync(0xffffffffu, r[k], off);
    if (lane == 0)
        for (int k = 0; k < kRedSlots; k++) sw[wid][k] = r[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < kRedSlots; k++) {
            double s = 0.0;
            for (int w = 0; w < kNATPB / 32; w++) s += sw[w][k];
            A.scratch->partials[(long long)blockIdx.x * kRedSlots + k] = s;
        }
        __threadfence();
        last = (atomicAdd(&A.scratch->ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    for (int k = 0; k < 3; k++) {
        double s = 0.0;
        for (unsigned b = 0; b < gridDim.x; b++) s += __ldcg(A.scratch->partials + (long long)b * kRedSlots + k);
        A.out[k] = s;
    }
    A.scratch->ticket = 0u;
}

std::mutex g_setup_mutex;
NoAllocScratch *g_scratch_ptr[kNAMaxDevices] = {};

// Resolve the device address of the scratch array once per device (host code
// may not use the symbol itself as a device pointer).
int scratch_for_current_device(NoAllocScratch **out) {
    int dev = -1;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return cuda_fail(err, "cudaGetDevice");
    if (dev < 0 || dev >= kNAMaxDevices) {
        set_error("device ordinal beyond the no-allocation table");
        return IQGPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void *ptr = nullptr;
        err = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (err != cudaSuccess) return cuda_fail(err, "cudaGetSymbolAddress(no-allocation scratch)");
        g_scratch_ptr[dev] = static_cast<NoAllocScratch *>(ptr);
    }
    *out = g_scratch_ptr[dev];
    return IQGPU_OK;
}

}  // namespace
}  // namespace iqg

using namespace iqg;

extern "C" int iqgpu_derv_noalloc(const double *theta_dev, const double *buffer_scale_dev, const double *freq_dev,
                                  const double *invar_dev, int32_t nptn, int64_t ldp, int32_t nstates, int32_t ncat,
                                  const double *eval, const double *rates, const double *props, double len,
                                  double *out_dev, void *cuda_stream) {
    if (!theta_dev || !buffer_scale_dev || !freq_dev || !invar_dev || !eval || !rates || !props || !out_dev) {
        set_error("null argument");
        return IQGPU_ERR_ARG;
    }
    if (nptn < 1 || nptn > kNAMaxPatterns) {
        set_error("iqgpu_derv_noalloc handles 1.." + std::to_string(kNAMaxPatterns) +
                  " patterns (its static scratch holds " + std::to_string(kNAMaxBlocks) + " CTA rows)");
        return IQGPU_ERR_ARG;
    }
    if (nstates < 2 || nstates > kMaxStates || ncat < 1 || ncat > kMaxCat || ldp < nptn || !(len >= 0.0)) {
        set_error("need 2<=nstates<=64, 1<=ncat<=16, ldp>=nptn, len>=0");
        return IQGPU_ERR_ARG;
    }
    NoAllocScratch *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    NoAllocArgs A;
    A.n = nstates;
    A.ncat = ncat;
    A.nptn = nptn;
    A.ldp = ldp;
    A.len = len;
    for (int i = 0; i < nstates; i++) A.eval[i] = eval[i];
    for (int c = 0; c < ncat; c++) {
        A.rates[c] = rates[c];
        A.props[c] = props[c];
    }
    A.theta = theta_dev;
    A.buffer_scale = buffer_scale_dev;
    A.freq = freq_dev;
    A.invar = invar_dev;
    A.out = out_dev;
    A.scratch = scratch;
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    // the ticket must start at zero even if an earlier call was abandoned
    cudaError_t err = cudaMemsetAsync(&scratch->ticket, 0, sizeof(unsigned), st);
    if (err != cudaSuccess) return cuda_fail(err, "clear no-allocation ticket");
    const int grid = (int)((nptn + kNATPB - 1) / kNATPB);
    k_derv_noalloc<<<grid, kNATPB, 0, st>>>(A);
    return cuda_fail(cudaGetLastError(), "derv_noalloc");
}
