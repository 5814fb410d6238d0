// C ABI of the likelihood engine: lifetime, inputs and the kernel-level entry
// points that stand in for PhyloTree's kernel function pointers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "engine.cuh"

namespace iqg {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int cuda_fail(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return IQGPU_OK;
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return IQGPU_ERR_CUDA;
}

static long long round_up(long long v, long long g) { return (v + g - 1) / g * g; }

struct Sizes {
    long long Ppad, part, scale, states, ops, opmats, theta, red, tcb, flow, cmax, pairs, total, op_stride;
};

static int check_config(const iqgpu_config *c) {
    if (!c) { set_error("null config"); return IQGPU_ERR_ARG; }
    if (c->nptn <= 0 || c->nstates < 2 || c->nstates > kMaxStates || c->ncat < 1 || c->ncat > kMaxCat ||
        c->ntaxa < 3 || c->state_unknown < c->nstates || c->state_unknown > 255 || c->nslots < 1 ||
        c->max_ops < 1) {
        set_error("config out of range (nptn>0, 2<=nstates<=64, 1<=ncat<=16, ntaxa>=3, "
                  "nstates<=state_unknown<=255, nslots>=1, max_ops>=1)");
        return IQGPU_ERR_ARG;
    }
    if (c->precision != IQGPU_F64 && c->precision != IQGPU_F32 && c->precision != IQGPU_TF32X3 &&
        c->precision != IQGPU_BF16) {
        set_error("precision not supported by this build of the engine (F64, F32, TF32X3, BF16)");
        return IQGPU_ERR_ARG;
    }
    return IQGPU_OK;
}

// The reference's kernel choice (PhyloTree::setLikelihoodKernel,
// tree/phylotreesse.cpp:95-96): SAFE scaling when asked for (-safe), when the
// tree has params->numseq_safe_scaling (2000) taxa or more, and whenever the
// model has other than 4 or 20 states. IQGPU_FLAG_SAFE_AS_GIVEN takes cfg.safe
// as it is.
static iqgpu_config normalized(const iqgpu_config *c) {
    iqgpu_config r = *c;
    if (!(c->flags & IQGPU_FLAG_SAFE_AS_GIVEN) &&
        (c->ntaxa >= kSafeScalingTaxa || (c->nstates != 4 && c->nstates != 20)))
        r.safe = 1;
    r.safe = r.safe ? 1 : 0;
    return r;
}

static bool is_mixed(const iqgpu_config *c) { return c->precision != IQGPU_F64; }
// tensor-core contraction (split TF32 or BF16): 20- and 61-state models (any
// 16 <= n <= 64); smaller state spaces stay on the FP32 CUDA-core kernels
static bool uses_tc(const iqgpu_config *c) {
    return (c->precision == IQGPU_TF32X3 || c->precision == IQGPU_BF16) && c->nstates >= 16 && c->nstates <= 64;
}
static long long tcb_stride(const iqgpu_config *c) {
    const int npad = (c->nstates + 3) / 4 * 4;
    return 2LL * c->ncat * 2 * tc_np(npad) * tc_kp(npad);
}

static Sizes sizes(const iqgpu_config *c) {
    Sizes s;
    const long long n = c->nstates, C = c->ncat, B = n * C, S = c->state_unknown;
    const long long npad = round_up(n, 4);
    s.Ppad = round_up(c->nptn, kTPB);
    s.states = (long long)c->ntaxa * s.Ppad;
    s.ops = (long long)(c->max_ops + 1) * (long long)sizeof(OpDev);
    if (is_mixed(c)) {
        // FP32 partials + int32 exponents; op blocks hold FP32 P(t) and leaf tables,
        // plus one block for the evaluated branch and the FP32 copy of U^-1
        s.part = (long long)c->nslots * s.Ppad * (C * npad * 4 + 4);
        s.scale = 0;
        s.op_stride = round_up(2 * C * n * npad + 2 * (S + 1) * C * npad, 4);
        s.opmats = ((long long)(c->max_ops + 1) * s.op_stride + C * n * npad) * 4;  // + U^-1 of each class
        s.theta = B * s.Ppad * 4 + 2 * s.Ppad * (long long)sizeof(double) +
                  (n >= 16 ? C * (2 * n * n + 2 * (S + 1) * n) * 4 : 0) +  // + the hi/lo split of U^-1 and tips
                  (C - 1) * (n + 2 * n * n + (S + 2) * n) * 8 +             // + the other classes' model arrays
                  (3 * n + 4 * n * n + (S + 1) * n) * 8 + 3 * C * n * npad * 8;  // + non-reversible model data
    } else {
        s.part = (long long)c->nslots * B * s.Ppad * (long long)sizeof(double);
        s.scale = (long long)c->nslots * (c->safe ? C : 1) * s.Ppad;
        s.op_stride = round_up(2 * C * n * n + 2 * (S + 1) * B, 4);
        s.opmats = (long long)c->max_ops * s.op_stride * (long long)sizeof(double);
        s.theta = B * s.Ppad * (long long)sizeof(double) + 2 * s.Ppad * (long long)sizeof(double) +
                  (C - 1) * (n + 2 * n * n + (S + 1) * n) * 8 +  // + the other mixture classes' model arrays
                  (3 * n + 4 * n * n + (S + 1) * n) * 8 + 3 * C * n * npad * 8 +  // + non-reversible model data
                  C * n * 8;                                                     // + branch frequency weights
    }
    s.tcb = uses_tc(c) ? (long long)(c->max_ops + 1) * tcb_stride(c) * 4 : 0;
    // category-split tensor-core levels hold fewer than 4 pairs per resident CTA
    // (<= 4 per SM): nl * Ppad < 16 * SMs * 128 patterns, SMs <= 160; the
    // dataflow schedule runs windows of up to kFlowWindowOps ops
    s.cmax = uses_tc(c) ? std::max(16LL * 160 * 128, (long long)kFlowWindowOps * s.Ppad) * C * 4 : 0;
    s.pairs = uses_tc(c) ? std::max<long long>(kPairCounters, (long long)kFlowWindowOps * (s.Ppad / 128)) : 0;
    s.flow = is_mixed(c) ? (long long)(c->max_ops + 1) * (s.Ppad / 128) * 4 : 0;
    // one partial-sum row per CTA; the smallest pattern tile of any kernel is 4
    // (the FP64 lane kernel: 128 threads, up to 32 lanes per pattern)
    s.red = (s.Ppad / 4) * kRedSlots * (long long)sizeof(double) + 64;
    s.total = s.part + s.scale + s.states + s.ops + s.opmats + s.theta + s.red + s.tcb + s.flow + s.cmax +
              s.pairs * 4 +
              2 * s.Ppad * 8 +
              3 * kMaxStates * 8 +
              (n + 2 * n * n + 2 * C + (S + 1) * n) * 8 + 32 * 256;  // + alignment of ~30 buffers
    return s;
}

}  // namespace iqg

using namespace iqg;

#define CK(call)                                              \
    do {                                                      \
        cudaError_t err__ = (call);                           \
        if (err__ != cudaSuccess) return cuda_fail(err__, #call); \
    } while (0)

extern "C" {

const char *iqgpu_last_error(void) { return g_last_error.c_str(); }

int iqgpu_memory_required(const iqgpu_config *cfg, size_t *bytes) {
    int rc = check_config(cfg);
    if (rc) return rc;
    if (!bytes) { set_error("null output"); return IQGPU_ERR_ARG; }
    const iqgpu_config eff = normalized(cfg);
    *bytes = (size_t)sizes(&eff).total;
    return IQGPU_OK;
}

}  // extern "C"

// Device buffers come from cudaMalloc, or are carved (256-byte aligned) from
// the caller's region when the engine was made with iqgpu_create_in.
template <class T>
static cudaError_t dalloc(iqgpu_engine *e, T **p, long long bytes) {
    if (!e->arena_base) return cudaMalloc(p, (size_t)bytes);
    const size_t off = (e->arena_used + 255) & ~(size_t)255;
    if (off + (size_t)bytes > e->arena_size) return cudaErrorMemoryAllocation;
    *p = reinterpret_cast<T *>(e->arena_base + off);
    e->arena_used = off + (size_t)bytes;
    return cudaSuccess;
}

// Host staging: pinned memory, or plain heap memory in a caller-provided
// region engine (no cudaMallocHost/cudaFreeHost per engine on a serving path)
template <class T>
static cudaError_t halloc(iqgpu_engine *e, T **p, long long bytes) {
    if (!e->arena_base) return cudaMallocHost(p, (size_t)bytes);
    *p = static_cast<T *>(std::malloc((size_t)bytes));
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}

extern "C" {

static void free_engine(iqgpu_engine *e) {
    if (!e) return;
    cudaSetDevice(e->dev);
    void *dev_ptrs[] = {e->d_eval, e->d_evec, e->d_inv, e->d_rates, e->d_props, e->d_tip, e->d_freq,
                        e->d_invar, e->d_states, e->d_part, e->d_scale, e->d_ops, e->d_opmats,
                        e->d_theta, e->d_bscale, e->d_plh, e->d_red_partials, e->d_ticket, e->d_red_out,
                        e->d_part32, e->d_exp, e->d_theta32, e->d_pi, e->d_opmats32, e->d_tcb,
                        e->d_flow_done, e->d_asc, e->d_cmax, e->d_ivhl, e->d_tiphl, e->d_pair_cnt,
                        e->d_nr, e->d_nrmats, e->d_pass_ops, e->d_pass_edge, e->d_pass_len, e->d_pass_res};
    if (e->d_asc_holder) cudaFree(e->d_asc_holder);  // cudaMalloc'd even in a region engine
    if (!e->arena_base) {
        for (void *p : dev_ptrs)
            if (p) cudaFree(p);
        if (e->h_ops) cudaFreeHost(e->h_ops);
        if (e->h_red_out) cudaFreeHost(e->h_red_out);
        if (e->h_pass_res) cudaFreeHost(e->h_pass_res);
        for (char *h : e->h_stage)
            if (h) cudaFreeHost(h);
        if (e->h_asc) cudaFreeHost(e->h_asc);
    } else {
        std::free(e->h_ops);
        std::free(e->h_red_out);
        std::free(e->h_stage[0]);
        std::free(e->h_stage[1]);
        std::free(e->h_asc);
    }
    std::free(e->level_off);
    for (cudaEvent_t ev : e->stage_ev)
        if (ev) cudaEventDestroy(ev);
    if (e->ev_t0) cudaEventDestroy(e->ev_t0);
    if (e->ev_t1) cudaEventDestroy(e->ev_t1);
    if (e->own_st) cudaStreamDestroy(e->own_st);
    delete e;
}

static int create_engine(const iqgpu_config *cfg, void *dev_mem, size_t dev_bytes, iqgpu_engine **out);

int iqgpu_create(const iqgpu_config *cfg, iqgpu_engine **out) { return create_engine(cfg, nullptr, 0, out); }

int iqgpu_create_in(const iqgpu_config *cfg, void *dev_mem, size_t bytes, iqgpu_engine **out) {
    if (!dev_mem || (reinterpret_cast<uintptr_t>(dev_mem) & 255)) {
        set_error("iqgpu_create_in needs a 256-byte aligned device region");
        return IQGPU_ERR_ARG;
    }
    return create_engine(cfg, dev_mem, bytes, out);
}

static int create_engine(const iqgpu_config *cfg_in, void *dev_mem, size_t dev_bytes, iqgpu_engine **out) {
    int rc = check_config(cfg_in);
    if (rc) return rc;
    const iqgpu_config cfg_eff = normalized(cfg_in);
    const iqgpu_config *cfg = &cfg_eff;
    if (!out) { set_error("null output"); return IQGPU_ERR_ARG; }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || cfg->device < 0 || cfg->device >= ndev) {
        cudaGetLastError();
        set_error("no CUDA device with that ordinal");
        return IQGPU_ERR_NODEV;
    }
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, cfg->device));
    if (prop.major != 10 || prop.minor != 3) {
        set_error("the engine is built for sm_103a (GB300); device is sm_" + std::to_string(prop.major) +
                  std::to_string(prop.minor));
        return IQGPU_ERR_NODEV;
    }
    CK(cudaSetDevice(cfg->device));
    Sizes s = sizes(cfg);
    if (dev_mem) {
        if ((size_t)s.total > dev_bytes) {
            set_error("admission refused: engine needs " + std::to_string(s.total) + " bytes, region holds " +
                      std::to_string(dev_bytes));
            return IQGPU_ERR_OOM;
        }
    } else {
        size_t free_b = 0, total_b = 0;
        CK(cudaMemGetInfo(&free_b, &total_b));
        if ((size_t)s.total > free_b) {
            set_error("admission refused: engine needs " + std::to_string(s.total) + " bytes, " +
                      std::to_string(free_b) + " free");
            return IQGPU_ERR_OOM;
        }
    }
    iqgpu_engine *e = new iqgpu_engine();
    std::memset(e, 0, sizeof(*e));
    e->arena_base = static_cast<char *>(dev_mem);
    e->arena_size = dev_bytes;
    e->arena_used = 0;
    e->cfg = *cfg;
    e->dev = cfg->device;
    e->n = cfg->nstates;
    e->C = cfg->ncat;
    e->B = e->n * e->C;
    e->S = cfg->state_unknown;
    e->P = cfg->nptn;
    e->Ppad = s.Ppad;
    e->nblk = (int)(s.Ppad / kTPB);
    if (cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, cfg->device) != cudaSuccess || e->sms < 1)
        e->sms = 1;
    e->op_stride = s.op_stride;
    e->level_off = static_cast<int *>(std::malloc(sizeof(int) * ((size_t)cfg->max_ops + 2)));
    if (!e->level_off) {
        delete e;
        set_error("host allocation failed");
        return IQGPU_ERR_OOM;
    }
    auto fail = [&](cudaError_t err, const char *what) {
        int r = cuda_fail(err, what);
        if (err == cudaErrorMemoryAllocation) r = IQGPU_ERR_OOM;
        free_engine(e);
        return r;
    };
#define CKE(call)                                 \
    do {                                          \
        cudaError_t err__ = (call);               \
        if (err__ != cudaSuccess) return fail(err__, #call); \
    } while (0)
    CKE(cudaStreamCreateWithFlags(&e->own_st, cudaStreamNonBlocking));
    e->st = e->own_st;
    CKE(cudaEventCreate(&e->ev_t0));
    CKE(cudaEventCreate(&e->ev_t1));
    const long long n = e->n, C = e->C, B = e->B, S = e->S;
    // model arrays per mixture class: up to ncat classes
    const long long K = C;
    e->nmix = 1;
    e->cpc = (int)C;
    CKE(dalloc(e, &e->d_eval, K * n * 8));
    CKE(dalloc(e, &e->d_evec, K * n * n * 8));
    CKE(dalloc(e, &e->d_inv, K * n * n * 8));
    CKE(dalloc(e, &e->d_rates, C * 8));
    CKE(dalloc(e, &e->d_props, C * 8));
    CKE(dalloc(e, &e->d_tip, (S + 1) * K * n * 8));
    CKE(dalloc(e, &e->d_freq, e->Ppad * 8));
    CKE(dalloc(e, &e->d_invar, e->Ppad * 8));
    CKE(dalloc(e, &e->d_states, s.states));
    CKE(dalloc(e, &e->d_ops, s.ops));
    e->npad = (int)round_up(n, 4);
    e->bp = C * e->npad;
    if (is_mixed(cfg)) {
        e->op_stride32 = s.op_stride;
        CKE(dalloc(e, &e->d_part32, (long long)cfg->nslots * e->Ppad * e->bp * 4));
        CKE(dalloc(e, &e->d_exp, (long long)cfg->nslots * e->Ppad * 4));
        CKE(dalloc(e, &e->d_opmats32, s.opmats));
        CKE(dalloc(e, &e->d_theta32, B * e->Ppad * 4));
        CKE(dalloc(e, &e->d_pi, K * n * 8));
        if (n >= 16) {
            CKE(dalloc(e, &e->d_ivhl, 2 * K * n * n * 4));
            CKE(dalloc(e, &e->d_tiphl, 2 * (S + 1) * K * n * 4));
        }
        // padding states of every slot stay zero: finite inputs for the float4 matvecs
        CKE(cudaMemsetAsync(e->d_part32, 0, (long long)cfg->nslots * e->Ppad * e->bp * 4, e->st));
        CKE(cudaMemsetAsync(e->d_exp, 0, (long long)cfg->nslots * e->Ppad * 4, e->st));
        CKE(cudaMemsetAsync(e->d_opmats32, 0, s.opmats, e->st));
        CKE(dalloc(e, &e->d_flow_done, s.flow));
        CKE(cudaMemsetAsync(e->d_flow_done, 0, s.flow, e->st));
        if (uses_tc(cfg)) {
            e->tc = true;
            e->tcb_stride = tcb_stride(cfg);
            CKE(dalloc(e, &e->d_tcb, s.tcb));
            CKE(dalloc(e, &e->d_cmax, s.cmax));
            e->cmax_bytes = (size_t)s.cmax;
            CKE(dalloc(e, &e->d_pair_cnt, s.pairs * 4));
            CKE(cudaMemsetAsync(e->d_pair_cnt, 0, s.pairs * 4, e->st));
            e->pair_cap = s.pairs;
        }
    } else {
        CKE(dalloc(e, &e->d_part, s.part));
        CKE(dalloc(e, &e->d_scale, s.scale));
        CKE(dalloc(e, &e->d_opmats, s.opmats));
        CKE(cudaMemsetAsync(e->d_scale, 0, s.scale, e->st));
    }
    CKE(dalloc(e, &e->d_theta, is_mixed(cfg) ? 8 : B * e->Ppad * 8));
    CKE(dalloc(e, &e->d_bscale, e->Ppad * 8));
    CKE(dalloc(e, &e->d_plh, e->Ppad * 8));
    CKE(dalloc(e, &e->d_red_partials, (size_t)s.red));  // one row per CTA of the smallest pattern tile
    CKE(dalloc(e, &e->d_ticket, 64));  // ticket at byte 0, status word at 32, flow ticket at 48, state check at 56
    e->d_status = reinterpret_cast<int *>(reinterpret_cast<char *>(e->d_ticket) + 32);
    e->d_flow_ticket = reinterpret_cast<unsigned *>(reinterpret_cast<char *>(e->d_ticket) + 48);
    CKE(dalloc(e, &e->d_red_out, kRedSlots * 8));
    CKE(dalloc(e, &e->d_asc, 3 * kMaxStates * 8));
    // non-reversible model data ([3][C][n][npad] branch matrices: FP32 on the mixed path, FP64 [3][C][n][n] on FP64)
    CKE(dalloc(e, &e->d_nr, (3 * e->n + 4LL * e->n * e->n + (long long)(S + 1) * e->n) * 8));
    CKE(dalloc(e, &e->d_nrmats, 3LL * e->C * e->n * e->npad * 8));
    if (!is_mixed(cfg)) CKE(dalloc(e, &e->d_pi, e->n * 8));  // branch weights of non-reversible models
    CKE(halloc(e, &e->h_ops, s.ops));
    CKE(halloc(e, &e->h_red_out, kRedSlots * 8 + 16));
    CKE(halloc(e, &e->h_asc, 3 * kMaxStates * 8));
    // setter staging: the largest single setter payload (pattern weights, or
    // the model arrays) per half
    // (+ the FP32 arrays the mixed setters build: U^-1 padded, its hi/lo split, the tip vectors' hi/lo)
    e->stage_cap = (size_t)std::max<long long>(2 * e->Ppad * 8, (n + 2 * n * n + 2 * C + (S + 2) * n) * 8 + 1024 +
                                                                    (2 * n * n + n * (n + 3) + 2 * (S + 1) * n) * 4 +
                                                                    4 * 256);
    CKE(halloc(e, &e->h_stage[0], (long long)e->stage_cap));
    CKE(halloc(e, &e->h_stage[1], (long long)e->stage_cap));
    CKE(cudaEventCreateWithFlags(&e->stage_ev[0], cudaEventDisableTiming));
    CKE(cudaEventCreateWithFlags(&e->stage_ev[1], cudaEventDisableTiming));
    CKE(cudaEventRecord(e->stage_ev[0], e->st));
    CKE(cudaEventRecord(e->stage_ev[1], e->st));
    CKE(cudaMemsetAsync(e->d_ticket, 0, 64, e->st));
    CKE(cudaMemsetAsync(e->d_freq, 0, e->Ppad * 8, e->st));
    CKE(cudaMemsetAsync(e->d_invar, 0, e->Ppad * 8, e->st));
    CKE(cudaMemsetAsync(e->d_states, (int)S, s.states, e->st));
    CKE(cudaStreamSynchronize(e->st));
#undef CKE
    *out = e;
    return IQGPU_OK;
}

int iqgpu_destroy(iqgpu_engine *e) {
    if (!e) return IQGPU_OK;
    cudaSetDevice(e->dev);
    cudaStreamSynchronize(e->st);
    nni_release(e);
    rell_release(e);
    free_engine(e);
    return IQGPU_OK;
}

int iqgpu_get_config(const iqgpu_engine *e, iqgpu_config *out) {
    if (!e || !out) { set_error("null argument"); return IQGPU_ERR_ARG; }
    *out = e->cfg;
    return IQGPU_OK;
}

// FP64 values as FP32 pairs hi = fl(v), lo = fl(v - hi) ([hi x count][lo x count]),
// the split the double-float precompute multiplies with

static void check_unit_tips(iqgpu_engine *e) {
    e->unit_tips = e->have_model && e->have_tips;
    for (int s = 0; s < e->n && e->unit_tips; s++)
        for (int i = 0; i < e->n; i++)
            if (e->h_tipv[s * e->n + i] != e->h_inv[i * e->n + s]) { e->unit_tips = false; break; }
}

// Setter uploads: the caller's arrays are copied into a staging half and
// sent from there, in stream order, so a setter returns before its copy runs
// and the caller may overwrite or free its buffer at once (pinned or not).
static cudaError_t stage_begin(iqgpu_engine *e) {
    e->stage_cur ^= 1;
    e->stage_used = 0;
    e->stage_direct = false;
    return cudaEventSynchronize(e->stage_ev[e->stage_cur]);  // the half's previous copies have run
}
static bool page_locked(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // pageable memory on older runtimes reports an error: clear it
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}
static cudaError_t stage_copy(iqgpu_engine *e, void *dst, const void *src, size_t bytes) {
    const size_t off = (e->stage_used + 255) & ~(size_t)255;
    if (off + bytes > e->stage_cap) {  // larger than a half: copy through the driver, then wait for it
        cudaError_t err = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, e->st);
        return err != cudaSuccess ? err : cudaStreamSynchronize(e->st);
    }
    if (bytes >= 16384 && page_locked(src)) {
        // page-locked caller buffer: copied from where it is, and stage_end waits
        // for it before the setter returns (no host copy of large arrays)
        e->stage_direct = true;
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, e->st);
    }
    char *h = e->h_stage[e->stage_cur] + off;
    std::memcpy(h, src, bytes);
    e->stage_used = off + bytes;
    return cudaMemcpyAsync(dst, h, bytes, cudaMemcpyHostToDevice, e->st);
}
// An array built on the host (FP32 conversions of the caller's data) goes
// out from the staging half too: page-locked, so the copy is queued without
// the wait a pageable copy would take.
static float *stage_floats(iqgpu_engine *e, size_t count) {
    const size_t off = (e->stage_used + 255) & ~(size_t)255;
    if (off + count * 4 > e->stage_cap) return nullptr;
    e->stage_used = off + count * 4;
    return reinterpret_cast<float *>(e->h_stage[e->stage_cur] + off);
}
static cudaError_t stage_send(iqgpu_engine *e, float *dst, const std::vector<float> &tmp, float *h, size_t count) {
    if (!h) {  // beyond the half: in stream order from the temporary, which must outlive the copy
        cudaError_t err = cudaMemcpyAsync(dst, tmp.data(), count * 4, cudaMemcpyHostToDevice, e->st);
        return err != cudaSuccess ? err : cudaStreamSynchronize(e->st);
    }
    return cudaMemcpyAsync(dst, h, count * 4, cudaMemcpyHostToDevice, e->st);
}
// hi = (float)v, lo = (float)(v - hi): the double-float operand of the mixed precompute
static cudaError_t upload_hilo(iqgpu_engine *e, float *dst, const double *v, size_t count) {
    std::vector<float> tmp;
    float *h = stage_floats(e, 2 * count);
    if (!h) {
        tmp.resize(2 * count);
        h = nullptr;
    }
    float *o = h ? h : tmp.data();
    for (size_t i = 0; i < count; i++) {
        o[i] = (float)v[i];
        o[count + i] = (float)(v[i] - (double)o[i]);
    }
    return stage_send(e, dst, tmp, h, 2 * count);
}

static cudaError_t stage_end(iqgpu_engine *e) {
    cudaError_t err = cudaEventRecord(e->stage_ev[e->stage_cur], e->st);
    if (err == cudaSuccess && e->stage_direct) err = cudaEventSynchronize(e->stage_ev[e->stage_cur]);
    return err;
}

int iqgpu_set_model(iqgpu_engine *e, const double *eval, const double *evec, const double *inv_evec,
                    const double *rates, const double *props) {
    if (!e || !eval || !evec || !inv_evec || !rates || !props) { set_error("null argument"); return IQGPU_ERR_ARG; }
    CK(cudaSetDevice(e->dev));
    const size_t n = e->n, C = e->C;
    CK(stage_begin(e));
    CK(stage_copy(e, e->d_eval, eval, n * 8));
    CK(stage_copy(e, e->d_evec, evec, n * n * 8));
    CK(stage_copy(e, e->d_inv, inv_evec, n * n * 8));
    CK(stage_copy(e, e->d_rates, rates, C * 8));
    CK(stage_copy(e, e->d_props, props, C * 8));
    if (is_mixed(&e->cfg)) {
        // FP32 copy of U^-1, rows padded to npad, after the op matrix blocks
        const size_t cnt = (size_t)n * e->npad;
        std::vector<float> tmp;
        float *h = stage_floats(e, cnt);
        if (!h) tmp.resize(cnt);
        float *o = h ? h : tmp.data();
        for (size_t i = 0; i < n; i++)
            for (size_t j = 0; j < (size_t)e->npad; j++) o[i * e->npad + j] = j < n ? (float)inv_evec[i * n + j] : 0.f;
        float *dst = e->d_opmats32 + (long long)(e->cfg.max_ops + 1) * e->op_stride32;
        CK(stage_send(e, dst, tmp, h, cnt));
        if (e->d_ivhl) CK(upload_hilo(e, e->d_ivhl, inv_evec, n * n));
    }
    CK(stage_end(e));
    std::memcpy(e->h_eval, eval, n * 8);
    std::memcpy(e->h_rates, rates, C * 8);
    std::memcpy(e->h_props, props, C * 8);
    std::memcpy(e->h_evec, evec, n * n * 8);
    std::memcpy(e->h_inv, inv_evec, n * n * 8);
    e->have_model = true;
    e->theta_valid = false;
    if (e->nonrev) {  // back to a reversible model: its tip vectors must be set again
        e->nonrev = false;
        e->have_tips = false;
    }
    if (e->nmix != 1) {  // back to one class: the class-indexed tip vectors must be set again
        e->nmix = 1;
        e->cpc = e->C;
        e->have_tips = false;
    }
    check_unit_tips(e);
    return IQGPU_OK;
}

int iqgpu_set_mixture(iqgpu_engine *e, int32_t nmix, const double *eval, const double *evec, const double *inv_evec,
                      const double *rates, const double *props, const double *tip_lh, const double *state_freq) {
    if (!e || !eval || !evec || !inv_evec || !rates || !props || !tip_lh || !state_freq) {
        set_error("null argument");
        return IQGPU_ERR_ARG;
    }
    if (nmix < 1 || nmix > e->C || e->C % nmix != 0) {
        set_error("mixture: need 1 <= nmix <= ncat with ncat a multiple of nmix");
        return IQGPU_ERR_ARG;
    }
    CK(cudaSetDevice(e->dev));
    CK(cudaStreamSynchronize(e->st));
    const size_t n = e->n, C = e->C, K = (size_t)nmix, S1 = (size_t)e->S + 1;
    CK(cudaMemcpy(e->d_eval, eval, K * n * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e->d_evec, evec, K * n * n * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e->d_inv, inv_evec, K * n * n * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e->d_rates, rates, C * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e->d_props, props, C * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e->d_tip, tip_lh, S1 * K * n * 8, cudaMemcpyHostToDevice));
    const bool mixed = is_mixed(&e->cfg);
    if (mixed) CK(cudaMemcpy(e->d_pi, state_freq, K * n * 8, cudaMemcpyHostToDevice));
    if (mixed) {  // FP32 copies of every class's U^-1, after the op matrix blocks
        std::vector<float> inv32(K * n * e->npad, 0.f);
        for (size_t m = 0; m < K; m++)
            for (size_t i = 0; i < n; i++)
                for (size_t j = 0; j < n; j++) inv32[(m * n + i) * e->npad + j] = (float)inv_evec[(m * n + i) * n + j];
        float *dst = e->d_opmats32 + (long long)(e->cfg.max_ops + 1) * e->op_stride32;
        CK(cudaMemcpy(dst, inv32.data(), inv32.size() * 4, cudaMemcpyHostToDevice));
    }
    if (mixed && e->d_ivhl) {
        CK(stage_begin(e));
        for (size_t m = 0; m < K; m++) CK(upload_hilo(e, e->d_ivhl + m * 2 * n * n, inv_evec + m * n * n, n * n));
        CK(upload_hilo(e, e->d_tiphl, tip_lh, S1 * K * n));
        CK(stage_end(e));
    }
    // leaf-table shortcut: every class's unambiguous tip vectors are columns of its U^-1
    bool unit = true;
    for (size_t m = 0; m < K && unit; m++)
        for (size_t st = 0; st < n && unit; st++)
            for (size_t i = 0; i < n; i++)
                if (tip_lh[(st * K + m) * n + i] != inv_evec[(m * n + i) * n + st]) { unit = false; break; }
    std::memcpy(e->h_rates, rates, C * 8);
    std::memcpy(e->h_props, props, C * 8);
    e->nmix = nmix;
    e->cpc = (int)(C / K);
    e->nonrev = false;
    e->unit_tips = unit;
    e->have_model = e->have_tips = e->have_pi = true;
    e->theta_valid = false;
    return IQGPU_OK;
}

int iqgpu_set_model_nonrev(iqgpu_engine *e, const double *ceval_re, const double *ceval_im, const double *cevec_re,
                           const double *cevec_im, const double *cinv_re, const double *cinv_im,
                           const double *rates, const double *props, const double *tip_vec,
                           const double *root_freq) {
    if (!e || !ceval_re || !ceval_im || !cevec_re || !cevec_im || !cinv_re || !cinv_im || !rates || !props ||
        !tip_vec || !root_freq) {
        set_error("null argument");
        return IQGPU_ERR_ARG;
    }
    if (e->asc_n > 0) { set_error("+ASC is not available with non-reversible models"); return IQGPU_ERR_ARG; }
    CK(cudaSetDevice(e->dev));
    CK(cudaStreamSynchronize(e->st));
    const size_t n = e->n, nn = n * n, C = e->C, S1 = (size_t)e->S + 1;
    // [ceval re, im][cevec re, im][cinv re, im][root freq][tip vectors]
    std::vector<double> nr(3 * n + 4 * nn + S1 * n);
    double *q = nr.data();
    std::memcpy(q, ceval_re, n * 8); q += n;
    std::memcpy(q, ceval_im, n * 8); q += n;
    std::memcpy(q, cevec_re, nn * 8); q += nn;
    std::memcpy(q, cevec_im, nn * 8); q += nn;
    std::memcpy(q, cinv_re, nn * 8); q += nn;
    std::memcpy(q, cinv_im, nn * 8); q += nn;
    std::memcpy(q, root_freq, n * 8); q += n;
    std::memcpy(q, tip_vec, S1 * n * 8);
    CK(cudaMemcpy(e->d_nr, nr.data(), nr.size() * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e->d_rates, rates, C * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e->d_props, props, C * 8, cudaMemcpyHostToDevice));
    if (!is_mixed(&e->cfg)) {  // FP64: standard-basis partials, the traversal's dad transform is the identity
        std::vector<double> eye(nn, 0.0);
        for (size_t i = 0; i < n; i++) eye[i * n + i] = 1.0;
        CK(cudaMemcpy(e->d_inv, eye.data(), nn * 8, cudaMemcpyHostToDevice));
    }
    std::memcpy(e->h_rates, rates, C * 8);
    std::memcpy(e->h_props, props, C * 8);
    e->nonrev = true;
    e->nmix = 1;
    e->cpc = (int)C;
    e->unit_tips = false;
    e->have_model = e->have_tips = true;
    e->theta_valid = false;
    return IQGPU_OK;
}

int iqgpu_set_state_freq(iqgpu_engine *e, const double *state_freq) {
    if (!e || !state_freq) { set_error("null argument"); return IQGPU_ERR_ARG; }
    // the eigen-space FP64 path folds pi into U^-1; its non-reversible kernels weigh the branch by these
    CK(cudaSetDevice(e->dev));
    CK(stage_begin(e));
    CK(stage_copy(e, e->d_pi, state_freq, (size_t)e->n * 8));
    CK(stage_end(e));
    e->have_pi = true;
    return IQGPU_OK;
}

int iqgpu_set_tip_partials(iqgpu_engine *e, const double *tip_lh) {
    if (!e || !tip_lh) { set_error("null argument"); return IQGPU_ERR_ARG; }
    if (e->nonrev) {
        set_error("a non-reversible model takes its tip vectors with iqgpu_set_model_nonrev");
        return IQGPU_ERR_STATE;
    }
    CK(cudaSetDevice(e->dev));
    CK(stage_begin(e));
    CK(stage_copy(e, e->d_tip, tip_lh, (size_t)(e->S + 1) * e->n * 8));
    if (e->d_tiphl) CK(upload_hilo(e, e->d_tiphl, tip_lh, (size_t)(e->S + 1) * e->n));
    CK(stage_end(e));
    std::memcpy(e->h_tipv, tip_lh, (size_t)e->n * e->n * 8);
    e->have_tips = true;
    check_unit_tips(e);
    return IQGPU_OK;
}

int iqgpu_set_patterns(iqgpu_engine *e, const double *ptn_freq, const double *ptn_invar) {
    if (!e || !ptn_freq) { set_error("null argument"); return IQGPU_ERR_ARG; }
    CK(cudaSetDevice(e->dev));
    CK(stage_begin(e));
    CK(stage_copy(e, e->d_freq, ptn_freq, (size_t)e->P * 8));
    if (ptn_invar) CK(stage_copy(e, e->d_invar, ptn_invar, (size_t)e->P * 8));
    else CK(cudaMemsetAsync(e->d_invar, 0, (size_t)e->Ppad * 8, e->st));
    CK(stage_end(e));
    e->have_patterns = true;
    return IQGPU_OK;
}

// Sets *bad when any byte of the uploaded tip-state rows is above S (the
// padding columns hold S): 16 bytes per thread, grid-stride.
__global__ void k_check_states(const uint4 *__restrict__ st, long long n16, unsigned S, int *bad) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (long long)gridDim.x * blockDim.x) {
        const uint4 v = st[i];
        const unsigned w[4] = {v.x, v.y, v.z, v.w};
        unsigned over = 0;
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int b = 0; b < 4; b++) over |= ((w[j] >> (8 * b)) & 0xffu) > S;
        if (over) {
            atomicOr(bad, 1);
            return;
        }
    }
}

int iqgpu_set_tip_states(iqgpu_engine *e, const uint8_t *states) {
    if (!e || !states) { set_error("null argument"); return IQGPU_ERR_ARG; }
    CK(cudaSetDevice(e->dev));
    e->have_states = false;
    // stream-ordered: after any traversal still reading the previous states
    CK(cudaMemcpy2DAsync(e->d_states, (size_t)e->Ppad, states, (size_t)e->P, (size_t)e->P, (size_t)e->cfg.ntaxa,
                         cudaMemcpyHostToDevice, e->st));
    // the range check runs on the uploaded copy (a byte loop over the host
    // array would cost more than the whole likelihood evaluation)
    int *bad = reinterpret_cast<int *>(reinterpret_cast<char *>(e->d_ticket) + 56);
    CK(cudaMemsetAsync(bad, 0, 4, e->st));
    const long long n16 = (long long)e->cfg.ntaxa * e->Ppad / 16;
    k_check_states<<<(unsigned)std::min<long long>((n16 + 255) / 256, 4 * 152), 256, 0, e->st>>>(
        reinterpret_cast<const uint4 *>(e->d_states), n16, (unsigned)e->S, bad);
    e->launches++;
    CK(cudaGetLastError());
    int h_bad = 0;
    CK(cudaMemcpyAsync(&h_bad, bad, 4, cudaMemcpyDeviceToHost, e->st));
    CK(cudaStreamSynchronize(e->st));
    if (h_bad) {
        set_error("tip state above STATE_UNKNOWN");
        return IQGPU_ERR_ARG;
    }
    e->have_states = true;
    return IQGPU_OK;
}

static int ready(iqgpu_engine *e) {
    if (!e) { set_error("null engine"); return IQGPU_ERR_ARG; }
    if (!e->have_model || !e->have_tips || !e->have_patterns || !e->have_states) {
        set_error("model, tip partials, patterns and tip states must be set first");
        return IQGPU_ERR_STATE;
    }
    if (is_mixed(&e->cfg) && !e->have_pi) {
        set_error("the mixed-precision path needs the state frequencies (iqgpu_set_state_freq)");
        return IQGPU_ERR_STATE;
    }
    return IQGPU_OK;
}

static int check_ref(iqgpu_engine *e, int32_t r) {
    if (r >= 0) return r < e->cfg.nslots ? IQGPU_OK : IQGPU_ERR_ARG;
    return (-1 - r) < e->cfg.ntaxa ? IQGPU_OK : IQGPU_ERR_ARG;
}

// Validate a traversal, stage it in pinned memory and send it to the device.
// The mixed path evaluates a branch with FP32 transition matrices, so a
// branch evaluation appends one entry (index nops) whose child 0 is the far
// end b of the branch with the branch length.
// The checks every op list passes before it reaches the device.
static int check_ops(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops) {
    bool in_group = false;  // inside the records of a multifurcating node
    for (int k = 0; k < nops; k++) {
        const iqgpu_op &o = ops[k];
        const bool more = (o.flags & IQGPU_OP_MORE) != 0;
        // an absent second child closes a multifurcating node with an odd child count
        const bool absent1 = o.child[1] == IQGPU_NO_CHILD && in_group && !more;
        if (o.dad_slot < 0 || o.dad_slot >= e->cfg.nslots || check_ref(e, o.child[0]) ||
            (!absent1 && check_ref(e, o.child[1])) || o.child[0] == o.dad_slot || o.child[1] == o.dad_slot ||
            !(o.len[0] >= 0.0) || !(o.len[1] >= 0.0)) {
            set_error("bad traversal entry " + std::to_string(k));
            return IQGPU_ERR_ARG;
        }
        if (in_group && o.dad_slot != ops[k - 1].dad_slot) {
            set_error("traversal entry " + std::to_string(k) +
                      ": the records of a multifurcating node must share their dad slot");
            return IQGPU_ERR_ARG;
        }
        if ((more || in_group) && e->nonrev) {
            set_error("multifurcating nodes (IQGPU_OP_MORE) run with reversible models");
            return IQGPU_ERR_ARG;
        }
        const int dir = o.flags & ~IQGPU_OP_MORE;
        if (dir & ~(IQGPU_OP_TRANSPOSE0 | IQGPU_OP_TRANSPOSE1 | IQGPU_OP_ROOTLEAF0 | IQGPU_OP_ROOTLEAF1) ||
            (dir && !e->nonrev) || ((dir & IQGPU_OP_ROOTLEAF0) && o.child[0] >= 0) ||
            ((dir & IQGPU_OP_ROOTLEAF1) && o.child[1] >= 0)) {
            set_error("bad flags in traversal entry " + std::to_string(k) +
                      " (non-reversible models only; root-leaf flags on tip children only)");
            return IQGPU_ERR_ARG;
        }
        in_group = more;
    }
    if (in_group) {
        set_error("the last traversal entry is flagged IQGPU_OP_MORE");
        return IQGPU_ERR_ARG;
    }
    return IQGPU_OK;
}

static int upload_ops(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops, bool branch = false, int32_t b = 0,
                      double len = 0.0, bool stage_only = false) {
    if (nops < 0 || nops > e->cfg.max_ops || (nops > 0 && !ops)) {
        set_error("traversal length out of range");
        return IQGPU_ERR_ARG;
    }
    const bool extra = branch && is_mixed(&e->cfg);
    if (nops == 0 && !extra) return IQGPU_OK;
    // the previous upload must have left the staging buffer
    CK(cudaStreamSynchronize(e->st));
    int rc = check_ops(e, ops, nops);
    if (rc) return rc;
    e->has_multi = false;
    for (int k = 0; k < nops && !e->has_multi; k++) e->has_multi = (ops[k].flags & IQGPU_OP_MORE) != 0;
    // Mixed engines take the ops in tree-level order (a valid post-order: every
    // child is produced in a lower level), so that a level-synchronous launch
    // can run each level's independent ops together.
    std::vector<int> order(nops), level(nops, 1);
    for (int k = 0; k < nops; k++) order[k] = k;
    e->nlevels = 0;
    if (is_mixed(&e->cfg) && nops > 0) {
        std::vector<int> producer_level(e->cfg.nslots, 0);  // level of the op writing each slot in this list
        int maxl = 0;
        for (int k = 0, g0 = 0; k < nops; k++) {
            int l = 1;
            for (int j = 0; j < 2; j++)
                if (ops[k].child[j] >= 0) l = std::max(l, producer_level[ops[k].child[j]] + 1);
            level[k] = l;
            if (k > g0) l = std::max(l, level[k - 1]);  // the records of a multifurcating node share one level
            for (int j = g0; j <= k; j++) level[j] = l;
            if (!(ops[k].flags & IQGPU_OP_MORE)) {
                producer_level[ops[k].dad_slot] = l;
                g0 = k + 1;
            }
            maxl = std::max(maxl, l);
        }
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return level[x] < level[y]; });
        int cur = 0;
        for (int i = 0; i < nops; i++) {
            while (cur < level[order[i]]) e->level_off[cur++] = i;
        }
        e->level_off[cur] = nops;
        e->nlevels = maxl;  // level l (1-based) spans [level_off[l-1], level_off[l])
    }
    // producer of each child within the uploaded list (dataflow schedule)
    std::vector<int> writer(is_mixed(&e->cfg) ? e->cfg.nslots : 0, -1);
    for (int i = 0; i < nops; i++) {
        const int k = order[i];
        const iqgpu_op &o = ops[k];
        OpDev &d = e->h_ops[i];
        d.dad_slot = o.dad_slot;
        d.child[0] = o.child[0];
        d.child[1] = o.child[1];
        d.prod0 = (!writer.empty() && o.child[0] >= 0) ? writer[o.child[0]] : -1;
        d.len[0] = o.len[0];
        d.len[1] = o.len[1];
        d.mat_off = (long long)i * e->op_stride;
        d.prod1 = (!writer.empty() && o.child[1] >= 0) ? writer[o.child[1]] : -1;
        d.flags = o.flags;
        if (!writer.empty()) writer[o.dad_slot] = i;
    }
    int total = nops;
    if (extra) {
        OpDev &d = e->h_ops[nops];
        d.dad_slot = -1;
        d.child[0] = d.child[1] = b;
        d.prod0 = -1;
        d.len[0] = d.len[1] = len;
        d.mat_off = (long long)nops * e->op_stride;
        d.prod1 = -1;
        d.flags = 0;
        total++;
    }
    CK(cudaMemcpyAsync(e->d_ops, e->h_ops, sizeof(OpDev) * total, cudaMemcpyHostToDevice, e->st));
    return stage_only ? IQGPU_OK : launch_op_info(e, nops, extra);
}

}  // extern "C"

namespace iqg {
// Per-op P(t) / echild and leaf tables for the uploaded list (+ the branch
// block when `branch`), and the tensor-core B operands.
int launch_op_info(iqgpu_engine *e, int nops, bool branch) {
    const int total = nops + (branch ? 1 : 0);
    if (!is_mixed(&e->cfg)) return launch_partial_info_f64(e, total);
    int rc = launch_partial_info_mixed(e, total);
    if (rc == IQGPU_OK && e->tc) rc = launch_tc_prep(e, nops);
    return rc;
}

int stage_ops(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops, bool branch, int32_t b, double len) {
    return upload_ops(e, ops, nops, branch, b, len, true);
}
}  // namespace iqg

namespace iqg {
// the engines iqgpu_newton_branch serves
bool newton_on_device(const iqgpu_engine *e) {
    return e && !is_mixed(&e->cfg) && !e->nonrev && e->asc_n == 0 &&
           (long long)e->P * e->n * e->C <= IQGPU_NEWTON_MAX_ENTRIES;
}
}  // namespace iqg

extern "C" {

// Fold the last timed traversal into the running total.
static int settle_timing(iqgpu_engine *e) {
    if (!e->timing_pending) return IQGPU_OK;
    CK(cudaEventSynchronize(e->ev_t1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e->ev_t0, e->ev_t1));
    e->timing_ms += ms;
    e->timing_launches++;
    e->timing_pending = false;
    return IQGPU_OK;
}

static int traverse(iqgpu_engine *e, int nops, int epi, int32_t a, int32_t b, double len) {
    int rc;
    if (e->timing) {
        if ((rc = settle_timing(e))) return rc;
        CK(cudaEventRecord(e->ev_t0, e->st));
    }
    rc = is_mixed(&e->cfg) ? launch_traverse_mixed(e, nops, epi, a, b, len)
                           : launch_traverse_f64(e, nops, epi, a, b, len);
    if (rc) return rc;
    if (e->timing) {
        CK(cudaEventRecord(e->ev_t1, e->st));
        e->timing_pending = true;
    }
    return IQGPU_OK;
}

// A kernel that gave up a bounded wait leaves a nonzero status word.
static int check_status(iqgpu_engine *e) {
    int *h_status = reinterpret_cast<int *>(e->h_red_out + kRedSlots);
    CK(cudaMemcpyAsync(h_status, e->d_status, 4, cudaMemcpyDeviceToHost, e->st));
    CK(cudaStreamSynchronize(e->st));
    if (*h_status != 0) {
        CK(cudaMemsetAsync(e->d_status, 0, 4, e->st));
        if (e->d_pair_cnt) CK(cudaMemsetAsync(e->d_pair_cnt, 0, (size_t)e->pair_cap * 4, e->st));  // partial arrivals
        set_error("a device-side wait gave up (TMA copy not completed); results of that launch are invalid");
        return IQGPU_ERR_TIMEOUT;
    }
    return IQGPU_OK;
}

static int fetch_result(iqgpu_engine *e) {
    CK(cudaMemcpyAsync(e->h_red_out, e->d_red_out, kRedSlots * 8, cudaMemcpyDeviceToHost, e->st));
    CK(cudaStreamSynchronize(e->st));
    int rc = settle_timing(e);
    if (rc) return rc;
    return is_mixed(&e->cfg) ? check_status(e) : IQGPU_OK;
}

int iqgpu_compute_partials(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops) {
    int rc = ready(e);
    if (rc) return rc;
    CK(cudaSetDevice(e->dev));
    if ((rc = upload_ops(e, ops, nops))) return rc;
    return traverse(e, nops, EPI_NONE, 0, 0, 0.0);
}

// +ASC (Lewis) on a tree lnL whose per-pattern lnL is in d_plh: P_const =
// sum of the unobserved constant patterns' likelihoods (exp of their pattern
// lnL, which carries their scaling), lnL -= nsite * log(1 - P_const)
// (tree/phylokernelnew.h:3198-3222 and 3405-3420).
// +ASC Holder (tree/phylokernelnew.h:3175-3196, 2580-2617): per observed
// pattern p the unobserved patterns' likelihoods add up to P_p (block s of
// the appended patterns, entry p); the pattern lnL drops by log(1 - P_p) and
// the tree lnL by sum_p freq_p log(1 - P_p); the derivatives gain
// sum_p freq_p d1_p / (1 - P_p) and sum_p freq_p (d2_p / (1 - P_p) + (d1_p /
// (1 - P_p))^2). One CTA, a fixed order of additions: deterministic.
constexpr int kHolderThreads = 1024;
__device__ double holder_block_sum(double v, double *sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = kHolderThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kHolderThreads) k_asc_holder_lnl(double *plh, const double *freq, int nobs,
                                                                   int nstates, double *out) {
    __shared__ double sh[kHolderThreads];
    double acc = 0.0, bad = 0.0;
    for (int p = threadIdx.x; p < nobs; p += kHolderThreads) {
        double c = 0.0;
        for (int s = 0; s < nstates; s++) c += exp(plh[nobs + (long long)s * nobs + p]);
        if (!(c < 1.0 && c >= 0.0)) bad += 1.0;
        const double corr = log(1.0 - c);
        plh[p] -= corr;
        acc += freq[p] * corr;
    }
    acc = holder_block_sum(acc, sh);
    bad = holder_block_sum(bad, sh);
    if (threadIdx.x == 0) {
        out[0] = acc;
        out[1] = bad;
    }
}

__global__ void __launch_bounds__(kHolderThreads) k_asc_holder_derv(const double *t, const double *freq, int nobs,
                                                                    int nstates, double *out) {
    __shared__ double sh[kHolderThreads];
    double sdf = 0.0, sddf = 0.0;
    for (int p = threadIdx.x; p < nobs; p += kHolderThreads) {
        double c = 0.0, d1 = 0.0, d2 = 0.0;
        for (int s = 0; s < nstates; s++) {
            const double *o = t + 3 * ((long long)s * nobs + p);
            c += o[0];
            d1 += o[1];
            d2 += o[2];
        }
        const double pv = 1.0 - c, df_frac = d1 / pv, ddf_frac = d2 / pv;
        sdf += freq[p] * df_frac;
        sddf += freq[p] * (ddf_frac + df_frac * df_frac);
    }
    sdf = holder_block_sum(sdf, sh);
    sddf = holder_block_sum(sddf, sh);
    if (threadIdx.x == 0) {
        out[0] = sdf;
        out[1] = sddf;
    }
}

// out[v] = sum_i f(src[i * stride + v]) for v < nval, f = exp or the identity,
// one CTA in a fixed order (the Lewis correction over any number of patterns)
__global__ void __launch_bounds__(kHolderThreads) k_asc_sum(const double *src, int count, int stride, int nval,
                                                            int expv, double *out) {
    __shared__ double sh[kHolderThreads];
    for (int v = 0; v < nval; v++) {
        double acc = 0.0;
        for (int i = threadIdx.x; i < count; i += kHolderThreads) {
            const double x = src[(long long)i * stride + v];
            acc += expv ? exp(x) : x;
        }
        acc = holder_block_sum(acc, sh);
        if (threadIdx.x == 0) out[v] = acc;
    }
}

static int asc_lewis_sums(iqgpu_engine *e, bool derv, double *r) {
    double *out = e->d_asc_holder ? e->d_asc_holder + (e->asc_cap - 4) : e->d_asc + 3 * kMaxStates - 3;
    const double *src = derv ? (e->d_asc_holder ? e->d_asc_holder : e->d_asc) : e->d_plh + (e->P - e->asc_n);
    k_asc_sum<<<1, kHolderThreads, 0, e->st>>>(src, e->asc_n, derv ? 3 : 1, derv ? 3 : 1, derv ? 0 : 1, out);
    e->launches++;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(e->h_asc, out, (derv ? 3 : 1) * 8, cudaMemcpyDeviceToHost, e->st));
    CK(cudaStreamSynchronize(e->st));
    for (int v = 0; v < (derv ? 3 : 1); v++) r[v] = e->h_asc[v];
    return IQGPU_OK;
}

static int asc_holder_sums(iqgpu_engine *e, bool derv, double *r0, double *r1) {
    double *out = e->d_asc_holder + 3LL * e->asc_n;
    if (derv)
        k_asc_holder_derv<<<1, kHolderThreads, 0, e->st>>>(e->d_asc_holder, e->d_freq, e->asc_nobs, e->n, out);
    else
        k_asc_holder_lnl<<<1, kHolderThreads, 0, e->st>>>(e->d_plh, e->d_freq, e->asc_nobs, e->n, out);
    e->launches++;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(e->h_asc, out, 16, cudaMemcpyDeviceToHost, e->st));
    CK(cudaStreamSynchronize(e->st));
    *r0 = e->h_asc[0];
    *r1 = e->h_asc[1];
    return IQGPU_OK;
}

static int asc_lnl(iqgpu_engine *e, double *lnl) {
    if (e->asc_n <= 0) return IQGPU_OK;
    if (e->asc_holder) {
        double corr = 0.0, bad = 0.0;
        int rc = asc_holder_sums(e, false, &corr, &bad);
        if (rc) return rc;
        if (bad != 0.0) {
            set_error("+ASC (Holder): an observed pattern's unobserved patterns have probability outside [0, 1)");
            return IQGPU_ERR_NONFINITE;
        }
        e->asc_lc = 0.0;  // the observed patterns' lnL were corrected on the device
        *lnl -= corr;
        return IQGPU_OK;
    }
    double pc = 0.0;
    int rc = asc_lewis_sums(e, false, &pc);
    if (rc) return rc;
    if (!(pc < 1.0 && pc >= 0.0)) {
        set_error("+ASC: the unobserved constant patterns' probability is outside [0, 1)");
        return IQGPU_ERR_NONFINITE;
    }
    e->asc_lc = std::log(1.0 - pc);
    *lnl -= e->asc_nsite * e->asc_lc;
    return IQGPU_OK;
}

static int lnl_common(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops, int32_t a, int32_t b, double len,
                      double *lnl) {
    int rc = ready(e);
    if (rc) return rc;
    if (!lnl) { set_error("null output"); return IQGPU_ERR_ARG; }
    if (a < 0) std::swap(a, b);
    if (a < 0 || check_ref(e, a) || check_ref(e, b) || a == b || !(len >= 0.0)) {
        set_error("bad branch: need an internal partial, distinct ends and len >= 0");
        return IQGPU_ERR_ARG;
    }
    CK(cudaSetDevice(e->dev));
    if (e->nonrev && !is_mixed(&e->cfg)) {  // FP64 non-reversible: traversal, then the branch kernel on both ends
        if ((rc = upload_ops(e, ops, nops))) return rc;
        if ((rc = traverse(e, nops, EPI_NONE, a, b, len))) return rc;
        e->theta_valid = true;
        e->theta_a = a;
        e->theta_b = b;
        if ((rc = launch_branch_nonrev64(e, len, false))) return rc;
    } else {
        if ((rc = upload_ops(e, ops, nops, true, b, len))) return rc;
        if ((rc = traverse(e, nops, EPI_LNL, a, b, len))) return rc;
    }
    if ((rc = fetch_result(e))) return rc;
    const double *r = e->h_red_out;
    *lnl = std::isfinite(r[0]) ? r[0] : r[1];
    return asc_lnl(e, lnl);
}

int iqgpu_branch_lnl(iqgpu_engine *e, int32_t a, int32_t b, double len, double *lnl) {
    return lnl_common(e, nullptr, 0, a, b, len, lnl);
}

int iqgpu_compute_likelihood(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops, int32_t a, int32_t b,
                             double len, double *lnl) {
    return lnl_common(e, ops, nops, a, b, len, lnl);
}

int iqgpu_likelihood_derv(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops, int32_t a, int32_t b, double len,
                          int32_t theta_computed, double *df, double *ddf) {
    int rc = ready(e);
    if (rc) return rc;
    if (!df || !ddf) { set_error("null output"); return IQGPU_ERR_ARG; }
    if (a < 0) std::swap(a, b);
    if (a < 0 || check_ref(e, a) || check_ref(e, b) || a == b || !(len >= 0.0)) {
        set_error("bad branch");
        return IQGPU_ERR_ARG;
    }
    CK(cudaSetDevice(e->dev));
    if (!theta_computed || !e->theta_valid || e->theta_a != a || e->theta_b != b) {
        if (theta_computed && (!e->theta_valid || e->theta_a != a || e->theta_b != b)) {
            set_error("theta_computed set but the buffer holds another branch");
            return IQGPU_ERR_STATE;
        }
        if ((rc = upload_ops(e, ops, nops))) return rc;
        // non-reversible: no eigen-space theta; the derivative kernel reads the two ends
        if ((rc = traverse(e, nops, e->nonrev ? EPI_NONE : EPI_THETA, a, b, len))) return rc;
        e->theta_valid = true;
        e->theta_a = a;
        e->theta_b = b;
    }
    rc = e->nonrev ? (is_mixed(&e->cfg) ? launch_branch_nonrev(e, len, true) : launch_branch_nonrev64(e, len, true))
                   : is_mixed(&e->cfg) ? launch_derv_mixed(e, len) : launch_derv_f64(e, len);
    if (rc) return rc;
    if ((rc = fetch_result(e))) return rc;
    *df = e->h_red_out[0];
    *ddf = e->h_red_out[1];
    if (!std::isfinite(*df) && !e->cfg.safe && !is_mixed(&e->cfg)) {
        set_error("Numerical underflow (lh-derivative); the SAFE kernel avoids this");
        return IQGPU_ERR_NONFINITE;
    }
    if (e->asc_n > 0 && e->asc_holder) {
        double sdf = 0.0, sddf = 0.0;
        if ((rc = asc_holder_sums(e, true, &sdf, &sddf))) return rc;
        *df += sdf;
        *ddf += sddf;
    } else if (e->asc_n > 0) {  // Lewis +ASC (tree/phylokernelnew.h:2620-2628)
        double s3[3];
        if ((rc = asc_lewis_sums(e, true, s3))) return rc;
        const double lh = s3[0], d1 = s3[1], d2 = s3[2];
        const double pv = 1.0 - lh, df_frac = d1 / pv, ddf_frac = d2 / pv;
        *df += e->asc_nsite * df_frac;
        *ddf += e->asc_nsite * (ddf_frac + df_frac * df_frac);
    }
    if (!std::isfinite(*df)) *df = *ddf = 0.0;
    return IQGPU_OK;
}

int iqgpu_newton_supported(iqgpu_engine *e, int32_t *supported) {
    if (!e || !supported) { set_error("null argument"); return IQGPU_ERR_ARG; }
    *supported = iqg::newton_on_device(e) ? 1 : 0;
    return IQGPU_OK;
}

int iqgpu_newton_branch(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops, int32_t a, int32_t b,
                        int32_t theta_computed, double x1, double xguess, double x2, double xacc,
                        int32_t max_nr_step, double *optx, double *d2l, double *last_len, int32_t *steps) {
    int rc = ready(e);
    if (rc) return rc;
    if (!optx) { set_error("null output"); return IQGPU_ERR_ARG; }
    if (!iqg::newton_on_device(e)) {
        set_error("device Newton-Raphson: reversible FP64 engines without +ASC and at most "
                  "IQGPU_NEWTON_MAX_ENTRIES theta entries");
        return IQGPU_ERR_ARG;
    }
    if (!std::isfinite(x1) || !std::isfinite(x2) || !std::isfinite(xguess) || !std::isfinite(xacc) || x1 < 0.0) {
        set_error("bad Newton-Raphson bounds");
        return IQGPU_ERR_ARG;
    }
    if (a < 0) std::swap(a, b);
    if (a < 0 || check_ref(e, a) || check_ref(e, b) || a == b) {
        set_error("bad branch");
        return IQGPU_ERR_ARG;
    }
    CK(cudaSetDevice(e->dev));
    if (!theta_computed || !e->theta_valid || e->theta_a != a || e->theta_b != b) {
        if (theta_computed && (!e->theta_valid || e->theta_a != a || e->theta_b != b)) {
            set_error("theta_computed set but the buffer holds another branch");
            return IQGPU_ERR_STATE;
        }
        if ((rc = upload_ops(e, ops, nops))) return rc;
        const double len0 = xguess < x1 ? x1 : (xguess > x2 ? x2 : xguess);
        if ((rc = traverse(e, nops, EPI_THETA, a, b, len0))) return rc;
        e->theta_valid = true;
        e->theta_a = a;
        e->theta_b = b;
    }
    if ((rc = launch_newton_f64(e, x1, xguess, x2, xacc, max_nr_step, e->d_red_out))) return rc;
    if ((rc = fetch_result(e))) return rc;
    const double *r = e->h_red_out;  // {optx, status + 16 * steps, d2l, last length}
    const int status = (int)r[1] & 15;
    if (steps) *steps = (int32_t)(r[1] / 16.0);
    if (d2l) *d2l = r[2];
    if (last_len) *last_len = r[3];
    switch (status) {
    case 0: *optx = r[0]; return IQGPU_OK;
    case 1: set_error("Numerical underflow (lh-derivative); the SAFE kernel avoids this"); return IQGPU_ERR_NONFINITE;
    case 2: set_error("Wrong computeFuncDerv"); return IQGPU_ERR_NEWTON;
    default: set_error("Maximum number of iterations exceeded in minimizeNewton"); return IQGPU_ERR_NEWTON;
    }
}

}  // extern "C"

namespace iqg {
// engines whose tree driver runs whole optimisation passes on the device
bool pass_served(const iqgpu_engine *e) { return newton_on_device(e) && !e->arena_base; }

template <class T>
static cudaError_t grow_dev(T **p, long long &cap, long long need) {
    if (need <= cap) return cudaSuccess;
    if (*p) cudaFree(*p);
    *p = nullptr;
    cap = 0;
    const long long n = std::max(need, 64LL);
    cudaError_t err = cudaMalloc(p, (size_t)n * sizeof(T));
    if (err == cudaSuccess) cap = n;
    return err;
}

// One optimizeAllBranches pass (tree/phylotree.cpp:2698-2774) with every
// branch's minimizeNewton (utils/optimization.cpp:422-499) on the device and
// one host wait for the whole pass. Branch j rebuilds its stale partials,
// ops[off[j], off[j+1]), with each record's lengths read from the pass's
// device copy of the branch lengths (edges[2k], edges[2k+1]: the edge of
// each child, -1 for none), forms theta on refs ab[2j] (internal) and
// ab[2j+1], and k_newton_f64 solves it from the length of edge bedge[j],
// writing the optimum back there before the next branch's records are staged.
// res[4j..4j+3] = {optimum, status + 16 * steps, d2l, last evaluated length}
// as iqgpu_newton_branch reports them; a branch whose solve failed keeps its
// length, and the caller decides what to keep.
int run_pass(iqgpu_engine *e, const iqgpu_op *ops, const int32_t *edges, const int32_t *off, const int32_t *ab,
             const int32_t *bedge, int nb, const double *lengths, int nedge, double x1, double x2, double xacc,
             int max_steps, double *res) {
    int rc = ready(e);
    if (rc) return rc;
    if (!pass_served(e)) {
        set_error("device optimisation pass: engines served by iqgpu_newton_branch, not in a caller's region");
        return IQGPU_ERR_ARG;
    }
    if (nb <= 0 || nedge <= 0 || !edges || !off || !ab || !bedge || !lengths || !res || off[0] != 0) {
        set_error("bad optimisation pass");
        return IQGPU_ERR_ARG;
    }
    if (!std::isfinite(x1) || !std::isfinite(x2) || !std::isfinite(xacc) || x1 < 0.0) {
        set_error("bad Newton-Raphson bounds");
        return IQGPU_ERR_ARG;
    }
    for (int j = 0; j < nb; j++) {
        const int n = off[j + 1] - off[j];
        if (n < 0 || n > e->cfg.max_ops || (n > 0 && !ops)) {
            set_error("traversal length out of range");
            return IQGPU_ERR_ARG;
        }
        if ((rc = check_ops(e, ops + off[j], n))) return rc;
        const int a = ab[2 * j], b = ab[2 * j + 1];
        if (a < 0 || check_ref(e, a) || check_ref(e, b) || a == b || bedge[j] < 0 || bedge[j] >= nedge) {
            set_error("bad branch " + std::to_string(j));
            return IQGPU_ERR_ARG;
        }
    }
    const int total = off[nb];
    for (int k = 0; k < 2 * total; k++)
        if (edges[k] < -1 || edges[k] >= nedge) {
            set_error("bad edge of traversal entry " + std::to_string(k / 2));
            return IQGPU_ERR_ARG;
        }
    for (int k = 0; k < nedge; k++)
        if (!(lengths[k] >= 0.0) || !std::isfinite(lengths[k])) {
            set_error("bad branch length");
            return IQGPU_ERR_ARG;
        }
    CK(cudaSetDevice(e->dev));
    e->theta_valid = false;
    CK(grow_dev(&e->d_pass_ops, e->pass_ops_cap, std::max(total, 1)));
    CK(grow_dev(&e->d_pass_edge, e->pass_edge_cap, 2LL * std::max(total, 1)));
    CK(grow_dev(&e->d_pass_len, e->pass_len_cap, nedge));
    if (e->pass_res_cap < 4LL * nb) {
        CK(cudaStreamSynchronize(e->st));  // the previous pass's read-back has landed
        if (e->h_pass_res) cudaFreeHost(e->h_pass_res);
        e->h_pass_res = nullptr;
        CK(grow_dev(&e->d_pass_res, e->pass_res_cap, 4LL * nb));
        CK(cudaMallocHost(&e->h_pass_res, (size_t)e->pass_res_cap * sizeof(double)));
    }
    // each branch's records index their matrices from 0, as one uploaded list
    std::vector<OpDev> h((size_t)std::max(total, 1));
    for (int j = 0; j < nb; j++)
        for (int k = off[j]; k < off[j + 1]; k++) {
            const iqgpu_op &o = ops[k];
            OpDev &d = h[k];
            d.dad_slot = o.dad_slot;
            d.child[0] = o.child[0];
            d.child[1] = o.child[1];
            d.prod0 = d.prod1 = -1;
            d.len[0] = d.len[1] = 0.0;  // staged from the pass's lengths
            d.mat_off = (long long)(k - off[j]) * e->op_stride;
            d.flags = o.flags;
        }
    // pageable sources: each copy has read its source when the call returns
    CK(cudaMemcpyAsync(e->d_pass_ops, h.data(), sizeof(OpDev) * total, cudaMemcpyHostToDevice, e->st));
    CK(cudaMemcpyAsync(e->d_pass_edge, edges, sizeof(int32_t) * 2 * total, cudaMemcpyHostToDevice, e->st));
    CK(cudaMemcpyAsync(e->d_pass_len, lengths, sizeof(double) * nedge, cudaMemcpyHostToDevice, e->st));
    for (int j = 0; j < nb; j++) {
        const int n = off[j + 1] - off[j];
        const int a = ab[2 * j], b = ab[2 * j + 1];
        e->has_multi = false;
        for (int k = off[j]; k < off[j + 1] && !e->has_multi; k++) e->has_multi = (ops[k].flags & IQGPU_OP_MORE) != 0;
        if (n > 0 && (rc = launch_partial_info_f64(e, n, e->d_pass_ops + off[j], e->d_pass_edge + 2 * off[j],
                                                   e->d_pass_len)))
            return rc;
        if ((rc = traverse(e, n, EPI_THETA, a, b, 0.0))) return rc;
        double *len = e->d_pass_len + bedge[j];
        if ((rc = launch_newton_f64(e, x1, 0.0, x2, xacc, max_steps, e->d_pass_res + 4 * j, len, len))) return rc;
    }
    e->theta_valid = true;
    e->theta_a = ab[2 * nb - 2];
    e->theta_b = ab[2 * nb - 1];
    CK(cudaMemcpyAsync(e->h_pass_res, e->d_pass_res, sizeof(double) * 4 * nb, cudaMemcpyDeviceToHost, e->st));
    CK(cudaStreamSynchronize(e->st));
    if ((rc = settle_timing(e))) return rc;
    std::memcpy(res, e->h_pass_res, sizeof(double) * 4 * nb);
    return IQGPU_OK;
}
}  // namespace iqg

extern "C" {

int iqgpu_lnl_from_buffer(iqgpu_engine *e, double len, double *lnl) {
    int rc = ready(e);
    if (rc) return rc;
    if (!lnl) { set_error("null output"); return IQGPU_ERR_ARG; }
    if (!e->theta_valid) { set_error("no theta buffer: call iqgpu_likelihood_derv first"); return IQGPU_ERR_STATE; }
    CK(cudaSetDevice(e->dev));
    rc = e->nonrev ? (is_mixed(&e->cfg) ? launch_branch_nonrev(e, len, false) : launch_branch_nonrev64(e, len, false))
                   : is_mixed(&e->cfg) ? launch_from_buffer_mixed(e, len) : launch_from_buffer_f64(e, len);
    if (rc) return rc;
    if ((rc = fetch_result(e))) return rc;
    const double *r = e->h_red_out;
    if (!std::isfinite(r[0]) && !e->cfg.safe && !is_mixed(&e->cfg)) {
        set_error("Numerical underflow (lh-from-buffer); the SAFE kernel avoids this");
        return IQGPU_ERR_NONFINITE;
    }
    *lnl = std::isfinite(r[0]) ? r[0] : r[1];
    return asc_lnl(e, lnl);
}

int iqgpu_get_pattern_lh(iqgpu_engine *e, double *out) {
    if (!e || !out) { set_error("null argument"); return IQGPU_ERR_ARG; }
    CK(cudaSetDevice(e->dev));
    CK(cudaMemcpyAsync(out, e->d_plh, (size_t)e->P * 8, cudaMemcpyDeviceToHost, e->st));
    CK(cudaStreamSynchronize(e->st));
    if (e->asc_n > 0)  // the observed patterns' lnL carry the +ASC term of the latest lnL
        for (long long p = 0; p < e->P - e->asc_n; p++) out[p] -= e->asc_lc;
    return IQGPU_OK;
}

int iqgpu_set_asc(iqgpu_engine *e, int32_t nconst, double nsite) {
    if (e && e->nonrev && nconst > 0) {
        set_error("+ASC is not available with non-reversible models");
        return IQGPU_ERR_ARG;
    }
    if (!e || nconst < 0 || nconst >= e->P || !(nsite >= 0.0)) {
        set_error("+ASC: need 0 <= nconst < patterns and nsite >= 0");
        return IQGPU_ERR_ARG;
    }
    // more unobserved patterns than the fixed export buffer takes (ASC_INFORMATIVE): a larger one
    // (an existing buffer, from Holder's correction, is used whenever present, so it must fit too)
    if ((3LL * nconst > 3LL * kMaxStates - 3 || e->d_asc_holder) && 3LL * nconst + 4 > e->asc_cap) {
        CK(cudaSetDevice(e->dev));
        CK(cudaStreamSynchronize(e->st));
        if (e->d_asc_holder) CK(cudaFree(e->d_asc_holder));
        e->d_asc_holder = nullptr;
        e->asc_cap = 0;
        CK(cudaMalloc(&e->d_asc_holder, (3LL * nconst + 4) * 8));
        e->asc_cap = 3LL * nconst + 4;
    }
    e->asc_n = nconst;
    e->asc_nsite = nsite;
    e->asc_lc = 0.0;
    e->asc_holder = false;
    return IQGPU_OK;
}

int iqgpu_set_asc_holder(iqgpu_engine *e, int32_t nobs) {
    if (!e || nobs <= 0 || (long long)nobs * (e->n + 1) != e->P) {
        set_error("+ASC (Holder): need nobs > 0 observed patterns followed by nstates * nobs unobserved ones");
        return IQGPU_ERR_ARG;
    }
    if (e->nonrev) { set_error("+ASC is not available with non-reversible models"); return IQGPU_ERR_ARG; }
    CK(cudaSetDevice(e->dev));
    CK(cudaStreamSynchronize(e->st));
    if (e->d_asc_holder) CK(cudaFree(e->d_asc_holder));
    e->d_asc_holder = nullptr;
    e->asc_cap = 0;
    CK(cudaMalloc(&e->d_asc_holder, (3LL * e->n * nobs + 4) * 8));
    e->asc_cap = 3LL * e->n * nobs + 4;
    e->asc_holder = true;
    e->asc_nobs = nobs;
    e->asc_n = e->n * nobs;
    e->asc_nsite = 0.0;
    e->asc_lc = 0.0;
    return IQGPU_OK;
}

int iqgpu_get_partial(iqgpu_engine *e, int32_t slot, double *partial, uint8_t *scale) {
    if (!e || slot < 0 || slot >= e->cfg.nslots) { set_error("bad slot"); return IQGPU_ERR_ARG; }
    CK(cudaSetDevice(e->dev));
    CK(cudaStreamSynchronize(e->st));
    const long long B = e->B, P = e->P, Pp = e->Ppad;
    if (is_mixed(&e->cfg)) {
        // standard-basis values as stored (true value = stored * 2^exponent)
        if (partial) {
            std::vector<float> tmp((size_t)(Pp * e->bp));
            CK(cudaMemcpy(tmp.data(), e->d_part32 + (size_t)slot * Pp * e->bp, tmp.size() * 4, cudaMemcpyDeviceToHost));
            for (long long p = 0; p < P; p++)
                for (int c = 0; c < e->C; c++)
                    for (int x = 0; x < e->n; x++)
                        partial[p * B + c * e->n + x] = tmp[(size_t)mixed_index(p, c, x, e->npad, e->C)];
        }
        if (scale) std::memset(scale, 0, (size_t)P);
        return IQGPU_OK;
    }
    if (partial) {
        std::vector<double> tmp((size_t)(B * Pp));
        CK(cudaMemcpy(tmp.data(), e->d_part + (size_t)slot * B * Pp, (size_t)(B * Pp) * 8, cudaMemcpyDeviceToHost));
        for (long long p = 0; p < P; p++)
            for (long long r = 0; r < B; r++) partial[p * B + r] = tmp[(size_t)(r * Pp + p)];
    }
    if (scale) {
        const long long rows = e->cfg.safe ? e->C : 1;
        std::vector<uint8_t> tmp((size_t)(rows * Pp));
        CK(cudaMemcpy(tmp.data(), e->d_scale + (size_t)slot * rows * Pp, (size_t)(rows * Pp), cudaMemcpyDeviceToHost));
        for (long long p = 0; p < P; p++)
            for (long long c = 0; c < rows; c++) scale[p * rows + c] = tmp[(size_t)(c * Pp + p)];
    }
    return IQGPU_OK;
}

int iqgpu_get_exponent(iqgpu_engine *e, int32_t slot, int32_t *exponent) {
    if (!e || !exponent || slot < 0 || slot >= e->cfg.nslots) { set_error("bad argument"); return IQGPU_ERR_ARG; }
    if (!is_mixed(&e->cfg)) {
        set_error("the FP64 path keeps uint8 scale counts, not exponents");
        return IQGPU_ERR_STATE;
    }
    CK(cudaSetDevice(e->dev));
    CK(cudaStreamSynchronize(e->st));
    CK(cudaMemcpy(exponent, e->d_exp + (size_t)slot * e->Ppad, (size_t)e->P * 4, cudaMemcpyDeviceToHost));
    return IQGPU_OK;
}

int iqgpu_sync(iqgpu_engine *e) {
    if (!e) { set_error("null engine"); return IQGPU_ERR_ARG; }
    CK(cudaSetDevice(e->dev));
    CK(cudaStreamSynchronize(e->st));
    int rc = settle_timing(e);
    if (rc) return rc;
    return is_mixed(&e->cfg) ? check_status(e) : IQGPU_OK;
}

int iqgpu_set_stream(iqgpu_engine *e, void *cuda_stream) {
    if (!e) { set_error("null engine"); return IQGPU_ERR_ARG; }
    CK(cudaSetDevice(e->dev));
    CK(cudaStreamSynchronize(e->st));
    int rc = settle_timing(e);
    if (rc) return rc;
    e->st = cuda_stream ? (cudaStream_t)cuda_stream : e->own_st;
    return IQGPU_OK;
}

int iqgpu_set_timing(iqgpu_engine *e, int32_t enable) {
    if (!e) { set_error("null engine"); return IQGPU_ERR_ARG; }
    CK(cudaSetDevice(e->dev));
    CK(cudaStreamSynchronize(e->st));
    int rc = settle_timing(e);
    if (rc) return rc;
    e->timing = enable != 0;
    e->timing_ms = 0.0;
    e->timing_launches = 0;
    return IQGPU_OK;
}

int iqgpu_set_tile(iqgpu_engine *e, int32_t patterns_per_cta) {
    if (!e || !(patterns_per_cta == 0 || patterns_per_cta == 32 || patterns_per_cta == 64 ||
                patterns_per_cta == 128 || ((patterns_per_cta == 1 || patterns_per_cta == 2) && e->n == 4))) {
        set_error("tile must be 0, 32, 64 or 128 patterns (4-state models: 1 = one thread per pattern, "
                  "2 = two patterns per thread on the level schedule)");
        return IQGPU_ERR_ARG;
    }
    e->tile = patterns_per_cta;
    return IQGPU_OK;
}

int iqgpu_set_schedule(iqgpu_engine *e, int32_t schedule) {
    if (!e || schedule < 0 || schedule > 9) { set_error("schedule must be 0 .. 9"); return IQGPU_ERR_ARG; }
    e->level_sync = schedule == 1 || schedule >= 3;
    e->flow = schedule == 2;
    e->tc_ws = schedule == 3 || schedule >= 5;
    e->tc_tm = schedule == 4;
    e->tc_split = schedule == 5 || schedule == 6;
    e->tc_flow = schedule == 6;
    e->tc_flow_whole = schedule == 7;
    e->tc_ring = schedule == 8 || schedule == 9;
    e->tc_ring_all = schedule == 9;
    return IQGPU_OK;
}

int iqgpu_set_wait_limit(iqgpu_engine *e, uint32_t polls) {
    if (!e) { set_error("null engine"); return IQGPU_ERR_ARG; }
    e->wait_polls = polls;
    return IQGPU_OK;
}

int iqgpu_set_stages(iqgpu_engine *e, int32_t stages) {
    if (!e || !(stages == 0 || (stages >= 2 && stages <= 4))) {
        set_error("stages must be 0, 2, 3 or 4");
        return IQGPU_ERR_ARG;
    }
    e->tc_stages = stages;
    return IQGPU_OK;
}

int iqgpu_set_kpieces(iqgpu_engine *e, int32_t pieces) {
    if (!e || pieces < 0 || pieces > 4 || pieces == 3) {
        set_error("pieces must be 0, 1, 2 or 4");
        return IQGPU_ERR_ARG;
    }
    e->tc_kpieces = pieces;
    return IQGPU_OK;
}

int iqgpu_get_launches(iqgpu_engine *e, int64_t *launches) {
    if (!e || !launches) { set_error("null argument"); return IQGPU_ERR_ARG; }
    *launches = e->launches;
    return IQGPU_OK;
}

int iqgpu_get_timing(iqgpu_engine *e, double *total_ms, int64_t *launches) {
    if (!e || !total_ms || !launches) { set_error("null argument"); return IQGPU_ERR_ARG; }
    int rc = settle_timing(e);
    if (rc) return rc;
    *total_ms = e->timing_ms;
    *launches = e->timing_launches;
    return IQGPU_OK;
}

}  // extern "C"
