// Partitioned likelihood in one launch: a group of engines (one per partition,
// each with its own model, patterns, buffers and stream) whose evaluations are
// captured once into a CUDA graph and replayed with one cudaGraphLaunch.
//
// Reference: PhyloSuperTree::computeLikelihood (tree/phylosupertree.cpp:701-723)
// evaluates every partition's PhyloTree from an OpenMP loop and sums the
// partition lnLs. Here the partitions' kernels run on forked streams inside
// one graph, so small partitions fill the GPU together, and a replay costs one
// launch instead of 3+ launches and a synchronisation per partition. The
// graph reads each partition's op list (with its branch lengths) from device
// memory at replay time: re-staging the lists (iqgpu_group_set_lengths) and
// replaying evaluates new branch lengths without a new capture.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "engine.cuh"

struct iqgpu_group {
    std::vector<iqgpu_engine *> eng;
    std::vector<std::vector<iqgpu_op>> ops;
    std::vector<int32_t> a, b;
    std::vector<double> len;
    cudaStream_t st = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int dev = 0;
};

namespace iqg {

static void release_graph(iqgpu_group *g) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    g->exec = nullptr;
    g->graph = nullptr;
}

static int stage_all(iqgpu_group *g) {
    for (size_t i = 0; i < g->eng.size(); i++) {
        int rc = stage_ops(g->eng[i], g->ops[i].data(), (int32_t)g->ops[i].size(), true, g->b[i], g->len[i]);
        if (rc) return rc;
    }
    for (iqgpu_engine *e : g->eng) {
        cudaError_t err = cudaStreamSynchronize(e->st);
        if (err != cudaSuccess) return cuda_fail(err, "group staging");
    }
    return IQGPU_OK;
}

// One partition's evaluation on its own stream: per-op precompute, the
// traversal with the branch-lnL epilogue, and the copies of its sums and
// status word to pinned host memory.
static int enqueue_one(iqgpu_group *g, size_t i) {
    iqgpu_engine *e = g->eng[i];
    const int nops = (int)g->ops[i].size();
    const bool mixed = e->cfg.precision != IQGPU_F64;
    int rc = launch_op_info(e, nops, mixed);
    if (rc) return rc;
    rc = mixed ? launch_traverse_mixed(e, nops, EPI_LNL, g->a[i], g->b[i], g->len[i])
               : launch_traverse_f64(e, nops, EPI_LNL, g->a[i], g->b[i], g->len[i]);
    if (rc) return rc;
    cudaError_t err = cudaMemcpyAsync(e->h_red_out, e->d_red_out, kRedSlots * 8, cudaMemcpyDeviceToHost, e->st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(e->h_red_out + kRedSlots, e->d_status, 4, cudaMemcpyDeviceToHost, e->st);
    return cuda_fail(err, "group result copy");
}

static int capture(iqgpu_group *g) {
    release_graph(g);
    std::vector<bool> timing(g->eng.size());
    for (size_t i = 0; i < g->eng.size(); i++) {  // kernel timing events are not part of a graph
        timing[i] = g->eng[i]->timing;
        g->eng[i]->timing = false;
    }
    cudaError_t err = cudaStreamBeginCapture(g->st, cudaStreamCaptureModeThreadLocal);
    int rc = cuda_fail(err, "group capture begin");
    if (!rc) rc = cuda_fail(cudaEventRecord(g->fork, g->st), "group fork");
    for (size_t i = 0; i < g->eng.size() && !rc; i++) {
        rc = cuda_fail(cudaStreamWaitEvent(g->eng[i]->st, g->fork, 0), "group fork wait");
        if (!rc) rc = enqueue_one(g, i);
        if (!rc) rc = cuda_fail(cudaEventRecord(g->join[i], g->eng[i]->st), "group join");
        if (!rc) rc = cuda_fail(cudaStreamWaitEvent(g->st, g->join[i], 0), "group join wait");
    }
    cudaGraph_t graph = nullptr;
    err = cudaStreamEndCapture(g->st, &graph);  // always end the capture, also after an error
    if (!rc) rc = cuda_fail(err, "group capture end");
    if (!rc) {
        g->graph = graph;
        rc = cuda_fail(cudaGraphInstantiate(&g->exec, g->graph, 0), "group graph instantiate");
    } else if (graph) {
        cudaGraphDestroy(graph);
    }
    for (size_t i = 0; i < g->eng.size(); i++) g->eng[i]->timing = timing[i];
    return rc;
}

}  // namespace iqg

using namespace iqg;

extern "C" {

int iqgpu_group_create(iqgpu_engine *const *engines, int32_t n, iqgpu_group **out) {
    if (!engines || n < 1 || !out) { set_error("group needs >= 1 engine and an output"); return IQGPU_ERR_ARG; }
    *out = nullptr;
    for (int i = 0; i < n; i++) {
        if (!engines[i]) { set_error("null engine in group"); return IQGPU_ERR_ARG; }
        if (engines[i]->dev != engines[0]->dev) { set_error("group engines must share a device"); return IQGPU_ERR_ARG; }
        if (engines[i]->asc_n > 0 || engines[i]->nonrev) {
            set_error("+ASC and non-reversible engines cannot join a group");
            return IQGPU_ERR_ARG;
        }
        for (int j = 0; j < i; j++)
            if (engines[j] == engines[i]) { set_error("an engine appears twice in the group"); return IQGPU_ERR_ARG; }
    }
    iqgpu_group *g = new iqgpu_group();
    g->eng.assign(engines, engines + n);
    g->dev = engines[0]->dev;
    g->ops.resize(n);
    g->a.assign(n, 0);
    g->b.assign(n, 0);
    g->len.assign(n, 0.0);
    g->join.assign(n, nullptr);
    int rc = cuda_fail(cudaSetDevice(g->dev), "group device");
    if (!rc) rc = cuda_fail(cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking), "group stream");
    if (!rc) rc = cuda_fail(cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming), "group event");
    for (int i = 0; i < n && !rc; i++)
        rc = cuda_fail(cudaEventCreateWithFlags(&g->join[i], cudaEventDisableTiming), "group event");
    if (rc) {
        iqgpu_group_destroy(g);
        return rc;
    }
    *out = g;
    return IQGPU_OK;
}

int iqgpu_group_prepare(iqgpu_group *g, const iqgpu_op *const *ops, const int32_t *nops, const int32_t *a,
                        const int32_t *b, const double *len) {
    if (!g || !ops || !nops || !a || !b || !len) { set_error("null argument"); return IQGPU_ERR_ARG; }
    int rc = cuda_fail(cudaSetDevice(g->dev), "group device");
    if (rc) return rc;
    for (size_t i = 0; i < g->eng.size(); i++) {
        int32_t ai = a[i], bi = b[i];
        if (ai < 0) std::swap(ai, bi);
        if (ai < 0 || ai == bi || !(len[i] >= 0.0) || nops[i] < 0 || (nops[i] > 0 && !ops[i])) {
            set_error("bad branch or op list for group member " + std::to_string(i));
            return IQGPU_ERR_ARG;
        }
        g->ops[i].assign(ops[i], ops[i] + nops[i]);
        g->a[i] = ai;
        g->b[i] = bi;
        g->len[i] = len[i];
    }
    if ((rc = stage_all(g))) return rc;
    return capture(g);
}

int iqgpu_group_set_lengths(iqgpu_group *g, const iqgpu_op *const *ops, const double *len) {
    if (!g || !g->exec || !ops || !len) { set_error("group not prepared, or null argument"); return IQGPU_ERR_ARG; }
    int rc = cuda_fail(cudaSetDevice(g->dev), "group device");
    if (rc) return rc;
    for (size_t i = 0; i < g->eng.size(); i++) {
        for (size_t k = 0; k < g->ops[i].size(); k++) {
            const iqgpu_op &o = ops[i][k];
            if (o.dad_slot != g->ops[i][k].dad_slot || o.child[0] != g->ops[i][k].child[0] ||
                o.child[1] != g->ops[i][k].child[1]) {
                set_error("set_lengths may change branch lengths only; prepare the group again for new traversals");
                return IQGPU_ERR_ARG;
            }
            g->ops[i][k] = o;
        }
        g->len[i] = len[i];
    }
    // the captured epilogue carries the evaluated branch's length: a new length needs a new capture
    if ((rc = stage_all(g))) return rc;
    return capture(g);
}

int iqgpu_group_lnl(iqgpu_group *g, double *per_part, double *total) {
    if (!g || !g->exec) { set_error("group not prepared"); return IQGPU_ERR_STATE; }
    int rc = cuda_fail(cudaSetDevice(g->dev), "group device");
    if (!rc) rc = cuda_fail(cudaGraphLaunch(g->exec, g->st), "group launch");
    if (!rc) rc = cuda_fail(cudaStreamSynchronize(g->st), "group sync");
    if (rc) return rc;
    double sum = 0.0;
    for (size_t i = 0; i < g->eng.size(); i++) {
        iqgpu_engine *e = g->eng[i];
        const int *status = reinterpret_cast<const int *>(e->h_red_out + kRedSlots);
        if (*status != 0) {
            cudaMemsetAsync(e->d_status, 0, 4, e->st);
            cudaStreamSynchronize(e->st);
            set_error("a device-side wait gave up in group member " + std::to_string(i));
            return IQGPU_ERR_TIMEOUT;
        }
        const double v = std::isfinite(e->h_red_out[0]) ? e->h_red_out[0] : e->h_red_out[1];
        if (per_part) per_part[i] = v;
        sum += v;
    }
    if (total) *total = sum;
    return IQGPU_OK;
}

int iqgpu_group_destroy(iqgpu_group *g) {
    if (!g) return IQGPU_OK;
    cudaSetDevice(g->dev);
    if (g->st) cudaStreamSynchronize(g->st);
    release_graph(g);
    for (cudaEvent_t ev : g->join)
        if (ev) cudaEventDestroy(ev);
    if (g->fork) cudaEventDestroy(g->fork);
    if (g->st) cudaStreamDestroy(g->st);
    delete g;
    return IQGPU_OK;
}

}  // extern "C"
