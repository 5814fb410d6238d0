// Batched NNI-candidate evaluation: every candidate's two new partials in one
// traversal launch, then theta, Newton-Raphson on the central branch and the
// final lnL for all candidates in one CUDA graph (captured once per batch
// shape, replayed afterwards).
//
// Reference: PhyloTree::getBestNNIForBran (tree/phylotree.cpp:4069-4320) with
// one optimised branch per candidate (the -nni1 behaviour: nni5 off), which
// calls optimizeOneBranch(node1, node2, false, NNI_MAX_NR_STEP) and then
// computeLikelihoodFromBuffer() once per swap. The Newton-Raphson loop is
// Optimization::minimizeNewton (utils/optimization.cpp:422-499) turned into a
// per-candidate state machine that advances one derivative evaluation per
// graph step; converged candidates make their CTAs exit at once.
//
// Mixed-precision engines only (FP32 standard-basis partials, FP64 sums).
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "mixed.cuh"

namespace iqg {

struct NRState {
    double rts, xl, xh, dx, rts_old, f, df, out, start;
    int j, status, first, pad;
};
enum { NR_RUNNING = 0, NR_DONE = 1, NR_FAILED = 2 };

struct NniDev {
    const int32_t *ab;      // [ncand][2] scratch slots (node1 side, node2 side)
    float *theta;           // [ncand][B][ldp]
    double *bscale;         // [ncand][ldp]
    NRState *st;            // [ncand]
    double *red;            // [ncand][tiles][kRedSlots]
    unsigned *ticket;       // [ncand]
    double *out;            // [ncand][2]: lnl, length
    double min_bl, max_bl;
    int max_nr_step, tiles;
};

// ---------------------------------------------------------------------------
// theta_k[c][i] = (U^-1 a_c)_i (U^-1 b_c)_i and the exponent offset
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTPB) k_nni_theta(const MixParams P, const NniDev D) {
    const int k = blockIdx.y;
    const long long p = (long long)blockIdx.x * kTPB + threadIdx.x;
    const int n = P.n, npad = P.npad, C = P.ncat, nq = npad >> 2;
    const long long ld = P.ldp;
    const int a = D.ab[2 * k], b = D.ab[2 * k + 1];
    const long long pg = (p >> 3) * (8LL * C * npad) + (p & 7) * 4;
    const float *pa = P.part + (long long)a * P.slot_floats + pg;
    const float *pb = P.part + (long long)b * P.slot_floats + pg;
    float *th = D.theta + (long long)k * n * C * ld + p;
    for (int c = 0; c < C; c++)
        for (int i = 0; i < n; i++) {
            const float *urow = P.inv32 + (long long)i * npad;
            float ua = 0.f, ub = 0.f;
            for (int q = 0; q < nq; q++) {
                const float4 u = ld4(urow + 4 * q);
                const float4 av = *reinterpret_cast<const float4 *>(pa + (c * nq + q) * 32);
                const float4 bv = *reinterpret_cast<const float4 *>(pb + (c * nq + q) * 32);
                ua = fmaf(u.x, av.x, fmaf(u.y, av.y, fmaf(u.z, av.z, fmaf(u.w, av.w, ua))));
                ub = fmaf(u.x, bv.x, fmaf(u.y, bv.y, fmaf(u.z, bv.z, fmaf(u.w, bv.w, ub))));
            }
            th[(long long)(c * n + i) * ld] = ua * ub;
        }
    D.bscale[(long long)k * ld + p] = (double)(P.expo[(long long)a * ld + p] + P.expo[(long long)b * ld + p]) * kLn2;
}

// per-candidate deterministic reduction: CTA sums -> rows; the last CTA of the
// candidate adds them in CTA order
__device__ bool nni_reduce(double (&v)[kRedSlots], const NniDev &D, int k, double (&tot)[kRedSlots]) {
    __shared__ double sw[32][kRedSlots];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    mix_warp_reduce(v);
    if (lane == 0)
        for (int q = 0; q < kRedSlots; q++) sw[wid][q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
        double s[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
        for (int w = 0; w < nw; w++)
            for (int q = 0; q < kRedSlots; q++) s[q] += sw[w][q];
        double *row = D.red + ((long long)k * D.tiles + blockIdx.x) * kRedSlots;
        for (int q = 0; q < kRedSlots; q++) row[q] = s[q];
        __threadfence();
        last = (atomicAdd(D.ticket + k, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return false;
    __threadfence();
    for (int q = 0; q < kRedSlots; q++) {
        double s = 0.0;
        for (unsigned t = 0; t < gridDim.x; t++) s += __ldcg(D.red + ((long long)k * D.tiles + t) * kRedSlots + q);
        tot[q] = s;
    }
    D.ticket[k] = 0u;
    return true;
}

// ---------------------------------------------------------------------------
// derivative sums at the candidate's current trial length (computeFuncDerv)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTPB) k_nni_derv(const MixParams P, const NniDev D) {
    const int k = blockIdx.y;
    if (D.st[k].status != NR_RUNNING) return;  // uniform per CTA
    __shared__ float whi[3][kMaxCat * kMaxStates], wlo[3][kMaxCat * kMaxStates];
    const int n = P.n, C = P.ncat, B = n * C;
    const double len = D.st[k].rts;
    for (int t = threadIdx.x; t < B; t += blockDim.x) {
        const int c = t / n, i = t % n;
        const double cof = P.eval[i] * P.rates[c];
        const double val = exp(cof * len) * P.props[c];
        const double v[3] = {val, cof * val, cof * cof * val};
        for (int j = 0; j < 3; j++) {
            whi[j][t] = (float)v[j];
            wlo[j][t] = (float)(v[j] - (double)whi[j][t]);
        }
    }
    __syncthreads();
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double r[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
    if (p < P.nptn) {
        double a[3];
        theta_sums_df<3>(whi, wlo, D.theta + (long long)k * B * P.ldp + p, P.ldp, B, a);
        const double a0 = a[0], a1 = a[1], a2 = a[2];
        const double bs = D.bscale[(long long)k * P.ldp + p];
        const double lh = fabs(a0) + P.invar[p] * exp(-bs);
        const double inv = 1.0 / lh;
        const double df_frac = a1 * inv, ddf_frac = a2 * inv, f = P.freq[p];
        const double tmp1 = df_frac * f;
        r[0] = tmp1;
        r[1] = fma(-tmp1, df_frac, ddf_frac * f);
    }
    double tot[kRedSlots];
    if (nni_reduce(r, D, k, tot)) {
        D.st[k].f = -tot[0];  // computeFuncDerv negates
        D.st[k].df = -tot[1];
    }
}

// ---------------------------------------------------------------------------
// one Newton-Raphson step per candidate (minimizeNewton as a state machine)
// ---------------------------------------------------------------------------
__device__ void nr_done(NRState &s, double x) {
    s.out = x;
    s.status = NR_DONE;
}

__global__ void k_nni_init(const NniDev D, const double *start, int ncand) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ncand) return;
    NRState s;
    s.start = start[k];
    s.rts = fmin(fmax(start[k], D.min_bl), D.max_bl);
    s.xl = s.xh = s.dx = s.rts_old = s.f = s.df = 0.0;
    s.out = s.rts;
    s.j = 1;
    s.status = NR_RUNNING;
    s.first = 1;
    s.pad = 0;
    D.st[k] = s;
}

__global__ void k_nni_step(const NniDev D, int ncand) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ncand) return;
    NRState s = D.st[k];
    if (s.status != NR_RUNNING) return;
    const double xacc = D.min_bl, x1 = D.min_bl, x2 = D.max_bl;
    const double f = s.f, df = s.df;
    if (!isfinite(f) || !isfinite(df)) {  // nrerror("Wrong computeFuncDerv")
        s.status = NR_FAILED;
        D.st[k] = s;
        return;
    }
    if (s.first) {
        s.first = 0;
        if (df >= 0.0 && fabs(f) < xacc) { nr_done(s, s.rts); D.st[k] = s; return; }
        if (f < 0.0) { s.xl = s.rts; s.xh = x2; } else { s.xh = s.rts; s.xl = x1; }
        s.dx = fabs(s.xh - s.xl);
    } else {
        if (df > 0.0 && fabs(f) < xacc) { nr_done(s, s.rts); D.st[k] = s; return; }
        if (f < 0.0) s.xl = s.rts;
        else if (f > 0.0) s.xh = s.rts;
        s.j++;
    }
    if (s.j > D.max_nr_step) {  // "Maximum number of iterations exceeded"
        s.status = NR_FAILED;
        D.st[k] = s;
        return;
    }
    s.rts_old = s.rts;
    if ((df <= 0.0) || (((s.rts - s.xh) * df - f) * ((s.rts - s.xl) * df - f) >= 0.0)) {
        s.dx = 0.5 * (s.xh - s.xl);
        s.rts = s.xl + s.dx;
        if (s.xl == s.rts) { nr_done(s, s.rts); D.st[k] = s; return; }
    } else {
        s.dx = f / df;
        const double temp = s.rts;
        s.rts -= s.dx;
        if (temp == s.rts) { nr_done(s, s.rts); D.st[k] = s; return; }
    }
    if (fabs(s.dx) < xacc || s.j == D.max_nr_step) { nr_done(s, s.rts_old); D.st[k] = s; return; }
    D.st[k] = s;  // next graph step evaluates the derivatives at the new rts
}

// ---------------------------------------------------------------------------
// final lnL from theta at the optimised length; the divergence check of
// optimizeOneBranch (tree/phylotree.cpp:2612-2624) compares with the start length
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTPB) k_nni_lnl(const MixParams P, const NniDev D) {
    const int k = blockIdx.y;
    const NRState s = D.st[k];
    const double opt = s.status == NR_DONE ? s.out : s.rts;
    __shared__ double w0[kMaxCat * kMaxStates], w1[kMaxCat * kMaxStates];
    const int n = P.n, C = P.ncat, B = n * C;
    for (int t = threadIdx.x; t < B; t += blockDim.x) {
        const int c = t / n, i = t % n;
        w0[t] = exp(P.eval[i] * (P.rates[c] * opt)) * P.props[c];
        w1[t] = exp(P.eval[i] * (P.rates[c] * s.start)) * P.props[c];
    }
    __syncthreads();
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double r[kRedSlots] = {0.0, 0.0, 0.0, 0.0};
    if (p < P.nptn) {
        const float *th = D.theta + (long long)k * B * P.ldp + p;
        double a0 = 0.0, a1 = 0.0;
        for (int q = 0; q < B; q++) {
            const double t0 = (double)th[(long long)q * P.ldp];
            a0 = fma(w0[q], t0, a0);
            a1 = fma(w1[q], t0, a1);
        }
        const double bs = D.bscale[(long long)k * P.ldp + p];
        const double iv = P.invar[p] * exp(-bs), f = P.freq[p];
        r[0] = (log(fabs(a0) + iv) + bs) * f;
        r[1] = (log(fabs(a1) + iv) + bs) * f;
    }
    double tot[kRedSlots];
    if (nni_reduce(r, D, k, tot)) {
        double len = opt, lnl = tot[0];
        if (opt > D.max_bl * 0.95 && tot[1] > tot[0]) {  // Newton diverged: keep the start length
            len = s.start;
            lnl = tot[1];
        }
        if (s.status == NR_FAILED) lnl = NAN;
        D.out[2 * k] = lnl;
        D.out[2 * k + 1] = len;
    }
}

}  // namespace iqg

using namespace iqg;

namespace {

struct NniBuffers {
    int cap = 0, tiles = 0;
    int32_t *ab = nullptr;
    float *theta = nullptr;
    double *bscale = nullptr, *red = nullptr, *out = nullptr, *start = nullptr;
    NRState *st = nullptr;
    unsigned *ticket = nullptr;
    double *h_out = nullptr, *h_start = nullptr;
    int32_t *h_ab = nullptr;
    cudaGraphExec_t exec = nullptr;
    int g_ncand = -1, g_steps = -1;
    double g_min = -1, g_max = -1;
};

}  // namespace

// The engine keeps the NNI buffers in an opaque side table keyed by engine.
#include <map>
#include <mutex>
static std::map<iqgpu_engine *, NniBuffers> g_nni;
static std::mutex g_nni_mu;

static void nni_free(NniBuffers &b) {
    void *d[] = {b.ab, b.theta, b.bscale, b.red, b.out, b.start, b.st, b.ticket};
    for (void *p : d)
        if (p) cudaFree(p);
    if (b.h_out) cudaFreeHost(b.h_out);
    if (b.h_start) cudaFreeHost(b.h_start);
    if (b.h_ab) cudaFreeHost(b.h_ab);
    if (b.exec) cudaGraphExecDestroy(b.exec);
    b = NniBuffers();
}

namespace iqg {
void nni_release(iqgpu_engine *e) {
    std::lock_guard<std::mutex> lock(g_nni_mu);
    auto it = g_nni.find(e);
    if (it != g_nni.end()) {
        nni_free(it->second);
        g_nni.erase(it);
    }
}
}  // namespace iqg

#define CKN(call)                                                 \
    do {                                                          \
        cudaError_t err__ = (call);                               \
        if (err__ != cudaSuccess) return cuda_fail(err__, #call); \
    } while (0)

static int nni_reserve(iqgpu_engine *e, NniBuffers &b, int ncand) {
    const int tiles = (int)(e->Ppad / kTPB);
    if (b.cap >= ncand && b.tiles == tiles) return IQGPU_OK;
    nni_free(b);
    const long long B = e->B;
    const size_t need = (size_t)ncand * (B * e->Ppad * 4 + e->Ppad * 8 + (size_t)tiles * kRedSlots * 8);
    size_t free_b = 0, total_b = 0;
    CKN(cudaMemGetInfo(&free_b, &total_b));
    if (need > free_b) {
        set_error("admission refused: the NNI batch needs " + std::to_string(need) + " bytes");
        return IQGPU_ERR_OOM;
    }
    CKN(cudaMalloc(&b.ab, (size_t)ncand * 2 * 4));
    CKN(cudaMalloc(&b.theta, (size_t)ncand * B * e->Ppad * 4));
    CKN(cudaMalloc(&b.bscale, (size_t)ncand * e->Ppad * 8));
    CKN(cudaMalloc(&b.red, (size_t)ncand * tiles * kRedSlots * 8));
    CKN(cudaMalloc(&b.out, (size_t)ncand * 2 * 8));
    CKN(cudaMalloc(&b.start, (size_t)ncand * 8));
    CKN(cudaMalloc(&b.st, (size_t)ncand * sizeof(NRState)));
    CKN(cudaMalloc(&b.ticket, (size_t)ncand * 4));
    CKN(cudaMemset(b.ticket, 0, (size_t)ncand * 4));
    CKN(cudaMallocHost(&b.h_out, (size_t)ncand * 2 * 8));
    CKN(cudaMallocHost(&b.h_start, (size_t)ncand * 8));
    CKN(cudaMallocHost(&b.h_ab, (size_t)ncand * 2 * 4));
    b.cap = ncand;
    b.tiles = tiles;
    return IQGPU_OK;
}

extern "C" int iqgpu_nni_batch(iqgpu_engine *e, const iqgpu_nni_candidate *cand, int32_t ncand, int32_t max_nr_step,
                               double min_bl, double max_bl, double *lnl, double *central_len) {
    if (!e || !cand || !lnl || !central_len || ncand < 1 || max_nr_step < 1 || !(min_bl > 0.0) ||
        !(max_bl > min_bl)) {
        set_error("bad argument");
        return IQGPU_ERR_ARG;
    }
    if (e->asc_n > 0 || e->nmix > 1 || e->nonrev) {
        set_error("+ASC, mixture and non-reversible engines: evaluate NNI candidates with the per-branch entry points");
        return IQGPU_ERR_ARG;
    }
    iqgpu_config cfg;
    iqgpu_get_config(e, &cfg);
    if (cfg.precision == IQGPU_F64) {
        set_error("the NNI batch runs on the mixed-precision engine");
        return IQGPU_ERR_STATE;
    }
    if (2 * ncand > cfg.max_ops) {
        set_error("2*ncand must not exceed the engine's max_ops");
        return IQGPU_ERR_ARG;
    }
    // 1. both new partials of every candidate in one traversal launch
    std::vector<iqgpu_op> ops((size_t)2 * ncand);
    for (int k = 0; k < ncand; k++) {
        const iqgpu_nni_candidate &c = cand[k];
        if (c.scratch[0] < 0 || c.scratch[1] < 0 || c.scratch[0] == c.scratch[1]) {
            set_error("candidate " + std::to_string(k) + " needs two distinct scratch slots");
            return IQGPU_ERR_ARG;
        }
        ops[2 * k] = iqgpu_op{c.scratch[0], {c.sub[0], c.sub[1]}, 0, {c.len[0], c.len[1]}};
        ops[2 * k + 1] = iqgpu_op{c.scratch[1], {c.sub[2], c.sub[3]}, 0, {c.len[2], c.len[3]}};
    }
    int rc = iqgpu_compute_partials(e, ops.data(), 2 * ncand);
    if (rc) return rc;

    std::lock_guard<std::mutex> lock(g_nni_mu);
    NniBuffers &b = g_nni[e];
    if ((rc = nni_reserve(e, b, ncand))) return rc;
    for (int k = 0; k < ncand; k++) {
        b.h_ab[2 * k] = cand[k].scratch[0];
        b.h_ab[2 * k + 1] = cand[k].scratch[1];
        b.h_start[k] = cand[k].central;
    }
    cudaStream_t st = e->st;
    CKN(cudaMemcpyAsync(b.ab, b.h_ab, (size_t)ncand * 8, cudaMemcpyHostToDevice, st));
    CKN(cudaMemcpyAsync(b.start, b.h_start, (size_t)ncand * 8, cudaMemcpyHostToDevice, st));

    // 2. theta + Newton-Raphson + final lnL: one graph per batch shape
    NniDev D;
    D.ab = b.ab;
    D.theta = b.theta;
    D.bscale = b.bscale;
    D.st = b.st;
    D.red = b.red;
    D.ticket = b.ticket;
    D.out = b.out;
    D.min_bl = min_bl;
    D.max_bl = max_bl;
    D.max_nr_step = max_nr_step;
    D.tiles = b.tiles;
    MixParams P = mix_params(e, 0);
    if (!b.exec || b.g_ncand != ncand || b.g_steps != max_nr_step || b.g_min != min_bl || b.g_max != max_bl) {
        if (b.exec) {
            cudaGraphExecDestroy(b.exec);
            b.exec = nullptr;
        }
        cudaGraph_t g;
        CKN(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        dim3 grid(b.tiles, ncand);
        k_nni_theta<<<grid, kTPB, 0, st>>>(P, D);
        k_nni_init<<<(ncand + 127) / 128, 128, 0, st>>>(D, b.start, ncand);
        for (int it = 0; it <= max_nr_step; it++) {
            k_nni_derv<<<grid, kTPB, 0, st>>>(P, D);
            k_nni_step<<<(ncand + 127) / 128, 128, 0, st>>>(D, ncand);
        }
        k_nni_lnl<<<grid, kTPB, 0, st>>>(P, D);
        cudaError_t cap = cudaStreamEndCapture(st, &g);
        if (cap != cudaSuccess) return cuda_fail(cap, "capture NNI graph");
        cudaError_t ierr = cudaGraphInstantiate(&b.exec, g, 0);
        cudaGraphDestroy(g);
        if (ierr != cudaSuccess) return cuda_fail(ierr, "instantiate NNI graph");
        b.g_ncand = ncand;
        b.g_steps = max_nr_step;
        b.g_min = min_bl;
        b.g_max = max_bl;
    }
    CKN(cudaGraphLaunch(b.exec, st));
    CKN(cudaMemcpyAsync(b.h_out, b.out, (size_t)ncand * 16, cudaMemcpyDeviceToHost, st));
    CKN(cudaStreamSynchronize(st));
    bool failed = false;
    for (int k = 0; k < ncand; k++) {
        lnl[k] = b.h_out[2 * k];
        central_len[k] = b.h_out[2 * k + 1];
        failed |= !std::isfinite(lnl[k]);
    }
    if (failed) {
        set_error("Newton-Raphson failed for at least one candidate (lnl = NaN)");
        return IQGPU_ERR_NEWTON;
    }
    return IQGPU_OK;
}
