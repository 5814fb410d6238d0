// Internal definitions shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/iqgpu.h"

namespace iqg {

// 2^-256 scaling threshold and its log (tree/phylotree.h:74-80).
constexpr int kScaleExp = 256;
constexpr double kScaleThreshold = 8.636168555094444625386e-78;
constexpr double kLogScaleThreshold = -177.4456782233459932741;
constexpr double kTwoPow256 = 1.157920892373161954235709850086879078532699846656405640394575840079131296399e77;

constexpr int kTPB = 128;        // threads (= patterns) per CTA in the pattern-tile kernels
constexpr int kMaxStates = 64;
constexpr int kPairCounters = 8192;  // (op, tile) pairs of one category-split tensor-core level
constexpr int kFlowWindowOps = 32;   // ops of one dataflow tensor-core launch (pair counters and maxima)
constexpr int kMaxCat = 16;
// params->numseq_safe_scaling default (utils/tools.cpp:1262): from this many
// taxa on, the reference switches to SAFE scaling
constexpr int kSafeScalingTaxa = 2000;

// Device copy of one traversal entry plus the offset of its per-op matrices.
struct OpDev {
    int32_t dad_slot;
    int32_t child[2];
    int32_t prod0;      // mixed engines: index (in the uploaded list) of the op writing child 0, or -1
    double len[2];
    long long mat_off;  // doubles into Engine::d_opmats
    int32_t prod1;      // as prod0, for child 1
    int32_t flags;      // IQGPU_OP_* (non-reversible models): transpose / root leaf per child
};

// Deterministic grid reduction: each CTA writes its partial sums, the last
// CTA (by ticket) adds them in CTA order.
struct Reduce {
    double *partials;    // [gridDim.x][kRedSlots]
    unsigned *ticket;    // zero between launches
    double *out;         // [kRedSlots]
};
constexpr int kRedSlots = 4;

struct TravParams {
    int n, ncat, state_unknown, nops, nptn;
    long long ldp;             // padded pattern count (row stride of a partial)
    long long slot_stride;     // elements per slot
    long long scale_stride;    // bytes per slot of scale counts
    long long op_stride;       // doubles per op in opmats
    const OpDev *ops;
    const double *opmats;
    const double *inv_evec;    // n*n
    const double *eval, *rates, *props;
    const double *tip_lh;      // (S+1)*nmix*n
    int nmix, cpc;             // mixture classes; category c belongs to class c / cpc
    const double *freq, *invar;
    const uint8_t *states;     // ntaxa*ldp
    double *partials;
    uint8_t *scale;
    // epilogue
    int32_t a, b;              // branch partials (a internal)
    double len;
    double *pattern_lh;        // LNL
    double *theta;             // THETA
    double *buffer_scale;      // THETA
    Reduce red;
    int cat_split;             // 1: this launch's CTA (x, y) computes category y only (SAFE op walks)
};

enum Epilogue { EPI_NONE = 0, EPI_LNL = 1, EPI_THETA = 2 };

}  // namespace iqg

struct iqgpu_engine {
    iqgpu_config cfg;
    int n, C, B, S;
    long long P, Ppad;
    int nblk;
    int dev;
    cudaStream_t st;
    // model
    double *d_eval, *d_evec, *d_inv, *d_rates, *d_props, *d_tip;
    double h_eval[iqg::kMaxStates], h_rates[iqg::kMaxCat], h_props[iqg::kMaxCat];
    bool have_model, have_tips, have_patterns, have_states;
    double *d_freq, *d_invar;
    uint8_t *d_states;
    // FP64 partials
    double *d_part;
    uint8_t *d_scale;
    // ops
    iqg::OpDev *d_ops, *h_ops;
    double *d_opmats;
    long long op_stride;
    // theta / results
    double *d_theta, *d_bscale, *d_plh;
    double *d_red_partials;
    unsigned *d_ticket;
    double *d_red_out, *h_red_out;
    // +ASC (Lewis): the last asc_n patterns are the unobserved constant
    // patterns; d_asc/h_asc hold their (lh, df, ddf) from the derivative
    // kernels, asc_lc the log(1 - P_const) of the latest lnL
    int asc_n;
    double asc_nsite, asc_lc;
    double *d_asc, *h_asc;
    // +ASC Holder (missing data): asc_n = n * asc_nobs unobserved patterns,
    // block s holding state s at every taxon each observed pattern has data
    // for; d_asc_holder (cudaMalloc) takes their (lh, df, ddf) and two sums
    bool asc_holder;
    int asc_nobs;
    double *d_asc_holder;  // also the export buffer of Lewis corrections with more than n patterns
    long long asc_cap;     // doubles in d_asc_holder
    bool theta_valid;
    int32_t theta_a, theta_b;
    // mixed-precision (FP32 standard-basis) state
    int npad;                 // n rounded up to 4
    long long bp;             // floats per pattern block = C * npad
    float *d_part32;          // [nslots][Ppad/8][C][npad/4][8][4]
    int32_t *d_exp;           // [nslots][Ppad] power-of-two exponent per pattern
    float *d_theta32;         // [B][Ppad] eigen-space theta
    double *d_pi, *d_tipstd;  // state frequencies, standard-basis tip vectors
    float *d_opmats32;
    long long op_stride32;    // floats per op
    double h_evec[iqg::kMaxStates * iqg::kMaxStates];
    // host copies of U^-1 and of the eigen-space tip vectors: unit_tips is set
    // when every unambiguous state's tip vector is exactly column s of U^-1,
    // so its leaf-table row equals column s of P(t)
    double h_inv[iqg::kMaxStates * iqg::kMaxStates];
    double h_tipv[iqg::kMaxStates * iqg::kMaxStates];  // rows of the n unambiguous states
    bool unit_tips;
    // non-reversible model (mixed engines): complex eigen system of Q, root
    // frequencies and standard-basis tip vectors in d_nr ([ceval re, im][cevec
    // re, im][cinv re, im][root freq][tip vectors (S+1) x n]); d_nrmats holds
    // prop * P, P', P'' of the evaluated branch ([3][C][n][npad] FP32)
    bool nonrev;
    double *d_nr;
    float *d_nrmats;
    bool have_pi, tipstd_ready;
    int tile;                 // patterns per CTA of the mixed traversal (0 = default)
    bool level_sync;          // mixed traversal schedule: one launch per tree level
    int *level_off;           // [max_ops + 2] first op of each level (ops are uploaded level-sorted)
    int nlevels;
    int *d_status;            // device status word (bounded waits that gave up)
    bool flow;                // dataflow schedule (4-state one-thread-per-pattern kernel)
    unsigned *d_flow_done;    // [max_ops][Ppad/128] nonzero once each (op, tile) item finished
    unsigned *d_flow_ticket;  // next item to hand out
    // tensor-core contraction (precision IQGPU_TF32X3, 16 <= n <= 64)
    bool tc;
    float *d_tcb;             // per op: [child 2][C][hi, lo][NP*KP] P(t) in core-matrix order
    long long tcb_stride;     // floats per op
    alignas(64) unsigned char tc_tmap[128];  // CUtensorMap over the partial slots (operand A tiles)
    bool tc_tmap_ready;
    int tc_tmap_kqs;          // box height (core matrices) the tensor map was encoded with
    int tc_stages;            // shared-memory ring depth of the tensor-core kernel (0 = default)
    int tc_kpieces;           // K pieces per stage (0/1 = whole K, 2 = halves)
    bool tc_ws;               // level schedule on the warp-specialised tensor-core kernel
    bool tc_tm;               // level schedule on the A-in-tensor-memory kernel (20 states, split TF32)
    bool tc_split;            // category-split items on narrow levels for <= 32 padded states too (schedule 5)
    bool tc_flow;             // dataflow schedule on the warp-specialised tensor-core kernel (schedule 6)
    bool tc_flow_whole;       // as tc_flow, with whole (op, tile) items (schedule 7)
    bool tc_ring;             // level schedule on the deep-ring kernel (20 states, split TF32; schedules 8, 9)
    bool tc_ring_all;         // ... with the one-op levels on it too, per tile in one launch (schedule 9)
    bool has_multi;           // the uploaded op list holds multifurcating records (IQGPU_OP_MORE)
    int sms;                  // multiprocessors of the engine's device
    float *d_ivhl, *d_tiphl;  // mixed, 16+ states: U^-1 and the eigen-space tip vectors as FP32 hi/lo pairs
    int nmix, cpc;            // mixture classes; categories per class (category c belongs to class c / cpc)
    float *d_cmax;            // category-split levels: per (op, category, pattern) maxima
    size_t cmax_bytes;
    unsigned *d_pair_cnt;     // category-split levels: arrivals per (op, tile) pair, re-armed to 0
    long long pair_cap;       // counters in d_pair_cnt
    // caller-provided device memory (iqgpu_create_in): buffers are carved from it
    char *arena_base;
    size_t arena_size, arena_used;
    // host inputs of the setters go through engine-owned staging (pinned unless
    // the engine lives in a caller's region): two halves used in turn, a half
    // refilled only after the copies that read it last have run (its event)
    char *h_stage[2];
    size_t stage_cap, stage_used;
    int stage_cur;
    bool stage_direct;        // a copy of this setter reads the caller's page-locked buffer directly
    cudaEvent_t stage_ev[2];
    // limit of the waits on other CTAs' progress (0 = the built-in ~seconds)
    unsigned wait_polls;
    // stream ownership and kernel timing
    cudaStream_t own_st;
    cudaEvent_t ev_t0, ev_t1;
    bool timing, timing_pending;
    double timing_ms;
    long long timing_launches;
    long long launches;       // kernel launches this engine has issued (throughput accounting)
    // device-resident branch-optimisation pass (allocated on first use): every
    // branch's op records, the edge each record's lengths come from, the
    // branch lengths the Newton solves update, and the per-branch results
    iqg::OpDev *d_pass_ops;
    int32_t *d_pass_edge;
    double *d_pass_len, *d_pass_res, *h_pass_res;
    long long pass_ops_cap, pass_edge_cap, pass_len_cap, pass_res_cap;
};

namespace iqg {
// Programmatic dependent launch: a kernel started by pdl_launch may be
// scheduled while the previous kernel of its stream is still running, and
// calls pdl_wait() before it reads anything that kernel (or one before it)
// writes; pdl_trigger() lets the next such kernel be scheduled. Both are
// no-ops for a kernel launched the ordinary way.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... K, typename... A>
static cudaError_t pdl_launch(void (*kern)(K...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<A &&>(args)...);
}

}  // namespace iqg

namespace iqg {
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

// FP64 kernel launchers (kernels_f64.cu)
// src/edge/len: the records of one branch of a device optimisation pass,
// staged into the engine's op list with their lengths from device memory
int launch_partial_info_f64(iqgpu_engine *e, int nops, const OpDev *src = nullptr, const int32_t *edge = nullptr,
                            const double *len = nullptr);
int launch_traverse_f64(iqgpu_engine *e, int nops, int epi, int32_t a, int32_t b, double len);
int launch_derv_f64(iqgpu_engine *e, double len);
int launch_newton_f64(iqgpu_engine *e, double x1, double xguess, double x2, double xacc, int max_steps,
                      double *out_dev, const double *xg_dev = nullptr, double *len_out = nullptr);
int launch_from_buffer_f64(iqgpu_engine *e, double len);

// mixed-precision launchers (kernels_mixed.cu); op index nops holds the
// transition matrices of the evaluated branch when epi != EPI_NONE
int launch_partial_info_mixed(iqgpu_engine *e, int nops_with_branch);
int launch_traverse_mixed(iqgpu_engine *e, int nops, int epi, int32_t a, int32_t b, double len);
int launch_derv_mixed(iqgpu_engine *e, double len);
int launch_from_buffer_mixed(iqgpu_engine *e, double len);
// non-reversible models: branch lnL (derv false) or lnL and derivatives
// (derv true) from the partials of the branch ends theta_a / theta_b
int launch_branch_nonrev(iqgpu_engine *e, double len, bool derv);
int launch_branch_nonrev64(iqgpu_engine *e, double len, bool derv);  // the same on FP64 engines

// tensor-core pattern-node update (traverse_tc.cu)
int tc_np(int npad);  // N of the MMA: npad padded to 32 or 64
int tc_kp(int npad);  // K of the MMA: npad padded to the TF32 K step
int tc_ksplit(const iqgpu_engine *e);  // K pieces per (category, side) stage
int launch_tc_prep(iqgpu_engine *e, int nops);

// op lists: host validation, level ordering and upload (stage_ops), and the
// per-op precompute launches for an uploaded list (launch_op_info)
int stage_ops(iqgpu_engine *e, const iqgpu_op *ops, int32_t nops, bool branch, int32_t b, double len);
int launch_op_info(iqgpu_engine *e, int nops, bool branch);

// side buffers of the batched entry points, released with the engine
void nni_release(iqgpu_engine *e);
void rell_release(iqgpu_engine *e);

// element offset of (pattern p, category c, state y) in a mixed-precision slot
__host__ __device__ inline long long mixed_index(long long p, int c, int y, int npad, int C) {
    return (p >> 3) * (8LL * C * npad) + (long long)(c * (npad >> 2) + (y >> 2)) * 32 + (p & 7) * 4 + (y & 3);
}
}  // namespace iqg
