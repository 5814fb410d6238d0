// Seeded sequence simulation on the device, for serving-size benchmark inputs
// (up to thousands of taxa x hundreds of thousands of sites), where a host
// simulator would dominate the benchmark's set-up time.
//
// One thread per site: draw the site's rate category and root state, then walk
// the edges in preorder, drawing each child's state from the row of the
// cumulative transition matrix P(r_c t_e) selected by the parent's state.
// Uniform variates come from a counter-based generator: the SplitMix64
// finaliser (Steele, Lea & Flood 2014) applied to (seed, site, edge), so every
// site is independent of the launch shape.
#include <cuda_runtime.h>

#include <string>

#include "../../include/iqgpu.h"

namespace iqg {
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
}  // namespace iqg

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ float uniform(unsigned long long seed, long long site, int k) {
    const unsigned long long h = mix64(seed ^ mix64((unsigned long long)site * 0x100000001B3ull + (unsigned)k));
    return (float)(h >> 40) * (1.0f / 16777216.0f);  // 24 random bits in [0, 1)
}

__device__ __forceinline__ int draw(const float *cum, int n, float u) {
    int y = 0;
    while (y < n - 1 && u >= cum[y]) y++;
    return y;
}

__global__ void k_simulate(int n, int ncat, int nedge, int ntaxa, long long nsites, const int *__restrict__ edge_parent,
                           const int *__restrict__ edge_child, const float *__restrict__ cumP,
                           const float *__restrict__ cumpi, unsigned long long seed, unsigned char *__restrict__ node_states,
                           unsigned char *__restrict__ out) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsites) return;
    const int cat = min((int)(uniform(seed, s, -1) * ncat), ncat - 1);
    const int root = edge_parent[0];
    node_states[(long long)root * nsites + s] = (unsigned char)draw(cumpi, n, uniform(seed, s, -2));
    for (int k = 0; k < nedge; k++) {
        const int par = edge_parent[k], ch = edge_child[k];
        const int x = node_states[(long long)par * nsites + s];
        const float *row = cumP + (((long long)k * ncat + cat) * n + x) * n;
        const int y = draw(row, n, uniform(seed, s, k));
        node_states[(long long)ch * nsites + s] = (unsigned char)y;
        if (ch < ntaxa) out[(long long)ch * nsites + s] = (unsigned char)y;
    }
}

}  // namespace

extern "C" int iqgpu_simulate(int32_t ntaxa, int64_t nsites, int32_t nstates, int32_t ncat, const int32_t *edge_parent,
                              const int32_t *edge_child, const float *cum_trans, const float *cum_freq, uint64_t seed,
                              int32_t device, uint8_t *states_out) {
    using namespace iqg;
    if (ntaxa < 3 || nsites < 1 || nstates < 2 || nstates > 64 || ncat < 1 || !edge_parent || !edge_child ||
        !cum_trans || !cum_freq || !states_out) {
        set_error("bad simulation argument");
        return IQGPU_ERR_ARG;
    }
    const int nedge = 2 * ntaxa - 3, nnode = 2 * ntaxa - 2;
    for (int k = 0; k < nedge; k++)
        if (edge_parent[k] < 0 || edge_parent[k] >= nnode || edge_child[k] < 0 || edge_child[k] >= nnode) {
            set_error("edge endpoint out of range");
            return IQGPU_ERR_ARG;
        }
    cudaError_t err = cudaSetDevice(device);
    if (err != cudaSuccess) return cuda_fail(err, "cudaSetDevice");
    int *d_par = nullptr, *d_ch = nullptr;
    float *d_cum = nullptr, *d_pi = nullptr;
    unsigned char *d_nodes = nullptr, *d_out = nullptr;
    const size_t cum_bytes = (size_t)nedge * ncat * nstates * nstates * 4;
    int rc = IQGPU_OK;
    auto ck = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && rc == IQGPU_OK) rc = cuda_fail(e, what);
        return rc == IQGPU_OK;
    };
    if (ck(cudaMalloc(&d_par, nedge * 4), "alloc") && ck(cudaMalloc(&d_ch, nedge * 4), "alloc") &&
        ck(cudaMalloc(&d_cum, cum_bytes), "alloc") && ck(cudaMalloc(&d_pi, nstates * 4), "alloc") &&
        ck(cudaMalloc(&d_nodes, (size_t)nnode * nsites), "alloc") &&
        ck(cudaMalloc(&d_out, (size_t)ntaxa * nsites), "alloc") &&
        ck(cudaMemcpy(d_par, edge_parent, nedge * 4, cudaMemcpyHostToDevice), "copy") &&
        ck(cudaMemcpy(d_ch, edge_child, nedge * 4, cudaMemcpyHostToDevice), "copy") &&
        ck(cudaMemcpy(d_cum, cum_trans, cum_bytes, cudaMemcpyHostToDevice), "copy") &&
        ck(cudaMemcpy(d_pi, cum_freq, nstates * 4, cudaMemcpyHostToDevice), "copy")) {
        const int tpb = 256;
        k_simulate<<<(unsigned)((nsites + tpb - 1) / tpb), tpb>>>(nstates, ncat, nedge, ntaxa, nsites, d_par, d_ch,
                                                                   d_cum, d_pi, seed, d_nodes, d_out);
        if (ck(cudaGetLastError(), "simulate launch"))
            ck(cudaMemcpy(states_out, d_out, (size_t)ntaxa * nsites, cudaMemcpyDeviceToHost), "copy back");
    }
    cudaFree(d_par);
    cudaFree(d_ch);
    cudaFree(d_cum);
    cudaFree(d_pi);
    cudaFree(d_nodes);
    cudaFree(d_out);
    return rc;
}
