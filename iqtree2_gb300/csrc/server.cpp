// Serving loop: continuous batching of likelihood + branch-optimisation jobs.
//
// The server owns one HBM arena (allocated once). A scheduler thread admits
// queued jobs in arrival order whenever a worker slot is free and the job's
// engine footprint (iqgpu_memory_required) fits in the arena's free space;
// a job larger than the whole arena is refused at once. Each admitted job
// gets its own engine carved from the arena (iqgpu_create_in: no cudaMalloc
// or cudaFree on the serving path, so admitting or retiring a job never
// synchronises the device) and its own CUDA stream, and runs the PhyloTree
// drivers (computeLikelihood, then optimizeAllBranches) on a worker thread.
// Jobs that arrive while others run are admitted as soon as memory and a slot
// free up, and their kernels overlap on the device with the running jobs'.
// Every reduction in the engine is deterministic, so a job's result does not
// depend on what else is running.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/iqgpu.h"

namespace iqg {
void set_error(const std::string &msg);
}

namespace {

// first-fit allocator over the arena with coalescing of free neighbours
struct Arena {
    char *base = nullptr;
    size_t total = 0;
    std::map<size_t, size_t> free;  // offset -> size

    bool alloc(size_t bytes, size_t *off) {
        bytes = (bytes + 255) & ~(size_t)255;
        for (auto it = free.begin(); it != free.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes, at = it->first + bytes;
                free.erase(it);
                if (rest) free[at] = rest;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = (bytes + 255) & ~(size_t)255;
        auto it = free.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free.erase(nx);
        }
        if (it != free.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free.erase(it);
            }
        }
    }
};

struct Job {
    int64_t id = 0;
    iqgpu_config cfg{};
    int32_t opt_iterations = 0;
    double tolerance = 1e-3;
    std::vector<double> eval, evec, inv, rates, props, pi, tip, freq, lengths, out_lengths;
    std::vector<uint8_t> states;
    std::vector<int32_t> edges;
    size_t bytes = 0, off = 0;
    iqgpu_job_result res{};
    bool done = false;
    std::thread worker;
};

double now_s(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct iqgpu_server {
    iqgpu_server_config cfg{};
    Arena arena;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Job *> queue;
    std::map<int64_t, std::unique_ptr<Job>> jobs;
    int active = 0;
    int64_t next_id = 1;
    bool stop = false;
    iqgpu_server_stats stats{};
    uint64_t bytes_in_use = 0;
    std::chrono::steady_clock::time_point t0;
    std::thread scheduler;
};

namespace {

void run_job(iqgpu_server *s, Job *j) {
    cudaSetDevice(s->cfg.device);
    iqgpu_engine *e = nullptr;
    iqgpu_tree *t = nullptr;
    double lnl0 = 0.0, lnl = 0.0;
    int rc = iqgpu_create_in(&j->cfg, s->arena.base + j->off, j->bytes, &e);
    if (!rc) rc = iqgpu_set_model(e, j->eval.data(), j->evec.data(), j->inv.data(), j->rates.data(), j->props.data());
    if (!rc) rc = iqgpu_set_state_freq(e, j->pi.data());
    if (!rc) rc = iqgpu_set_tip_partials(e, j->tip.data());
    if (!rc) rc = iqgpu_set_patterns(e, j->freq.data(), nullptr);
    if (!rc) rc = iqgpu_set_tip_states(e, j->states.data());
    if (!rc) rc = iqgpu_tree_create(e, j->edges.data(), j->lengths.data(), &t);
    if (!rc) rc = iqgpu_tree_compute_likelihood(t, &lnl0, nullptr);
    lnl = lnl0;
    if (!rc && j->opt_iterations > 0) rc = iqgpu_tree_optimize_all_branches(t, j->opt_iterations, j->tolerance, 100, &lnl);
    if (!rc) {
        j->out_lengths.resize(j->lengths.size());
        rc = iqgpu_tree_get_lengths(t, j->out_lengths.data());
    }
    if (rc) std::snprintf(j->res.error, sizeof(j->res.error), "%s", iqgpu_last_error());
    if (t) iqgpu_tree_destroy(t);
    if (e) iqgpu_destroy(e);
    std::lock_guard<std::mutex> lk(s->mu);
    s->arena.release(j->off, j->bytes);
    s->bytes_in_use -= j->bytes;
    s->active--;
    s->stats.completed++;
    j->res.status = rc;
    j->res.lnl_initial = lnl0;
    j->res.lnl = lnl;
    j->res.t_end = now_s(s->t0);
    j->done = true;
    s->cv.notify_all();
}

void schedule(iqgpu_server *s) {
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        s->cv.wait(lk, [&] { return s->stop || (!s->queue.empty() && s->active < s->cfg.max_active); });
        if (s->queue.empty()) {
            if (s->stop) break;
            continue;
        }
        Job *j = s->queue.front();
        if (j->bytes > s->arena.total) {  // can never fit: refuse now
            s->queue.pop_front();
            s->stats.refused++;
            j->res.status = IQGPU_ERR_OOM;
            std::snprintf(j->res.error, sizeof(j->res.error), "admission refused: job needs %zu bytes, arena holds %zu",
                          j->bytes, s->arena.total);
            j->res.t_start = j->res.t_end = now_s(s->t0);
            j->done = true;
            s->cv.notify_all();
            continue;
        }
        size_t off = 0;
        if (!s->arena.alloc(j->bytes, &off)) {  // wait for a running job to return memory
            s->cv.wait(lk);
            continue;
        }
        s->queue.pop_front();
        j->off = off;
        s->active++;
        s->stats.admitted++;
        s->bytes_in_use += j->bytes;
        if (s->active > s->stats.peak_active) s->stats.peak_active = s->active;
        if (s->bytes_in_use > s->stats.peak_bytes) s->stats.peak_bytes = s->bytes_in_use;
        j->res.t_start = now_s(s->t0);
        j->worker = std::thread(run_job, s, j);
    }
}

}  // namespace

extern "C" {

int iqgpu_server_create(const iqgpu_server_config *cfg, iqgpu_server **out) {
    if (!cfg || !out || cfg->max_active < 1) {
        iqg::set_error("bad server configuration");
        return IQGPU_ERR_ARG;
    }
    *out = nullptr;
    if (cudaSetDevice(cfg->device) != cudaSuccess) {
        cudaGetLastError();
        iqg::set_error("no CUDA device with that ordinal");
        return IQGPU_ERR_NODEV;
    }
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        iqg::set_error("cudaMemGetInfo failed");
        return IQGPU_ERR_CUDA;
    }
    size_t budget = cfg->memory_budget ? (size_t)cfg->memory_budget : free_b / 10 * 9;
    if (budget > free_b) budget = free_b / 10 * 9;
    auto *s = new iqgpu_server();
    s->cfg = *cfg;
    void *base = nullptr;
    if (cudaMalloc(&base, budget) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        iqg::set_error("could not reserve the serving arena");
        return IQGPU_ERR_OOM;
    }
    s->arena.base = static_cast<char *>(base);
    s->arena.total = budget;
    s->arena.free[0] = budget;
    s->stats.arena_bytes = budget;
    s->t0 = std::chrono::steady_clock::now();
    s->scheduler = std::thread(schedule, s);
    *out = s;
    return IQGPU_OK;
}

int iqgpu_server_submit(iqgpu_server *s, const iqgpu_job *job, int32_t precision, int64_t *id) {
    if (!s || !job || !id || !job->eval || !job->evec || !job->inv_evec || !job->rates || !job->props ||
        !job->state_freq || !job->tip_lh || !job->ptn_freq || !job->tip_states || !job->edges || !job->lengths) {
        iqg::set_error("null job field");
        return IQGPU_ERR_ARG;
    }
    auto j = std::make_unique<Job>();
    const int n = job->nstates, C = job->ncat, T = job->ntaxa, P = job->nptn, S = job->state_unknown;
    iqgpu_config &c = j->cfg;
    c.nptn = P;
    c.nstates = n;
    c.ncat = C;
    c.ntaxa = T;
    c.state_unknown = S;
    c.nslots = 3 * (T - 2);
    c.safe = 0;
    c.precision = precision;
    c.device = s->cfg.device;
    c.max_ops = 2 * T;
    c.flags = 0;
    size_t bytes = 0;
    int rc = iqgpu_memory_required(&c, &bytes);
    if (rc) return rc;
    if (bytes > s->arena.total / 2) {
        // slot recycling: as many partial slots as half the arena holds, at
        // least the ones pinned along a root path (larger subtrees first)
        iqgpu_config c1 = c;
        size_t b1 = 0, b2 = 0;
        c1.nslots = 1;
        if ((rc = iqgpu_memory_required(&c1, &b1))) return rc;
        c1.nslots = 2;
        if ((rc = iqgpu_memory_required(&c1, &b2))) return rc;
        const size_t per = b2 - b1, base = b1 - per, target = s->arena.total / 2;
        int lg = 1;
        while ((1 << lg) < T) lg++;
        const long long fit = target > base ? (long long)((target - base) / per) : 0;
        if (fit >= 2 * lg + 4) {
            c.nslots = (int32_t)std::min<long long>(fit, c.nslots);
            if ((rc = iqgpu_memory_required(&c, &bytes))) return rc;
        }
    }
    j->bytes = bytes;
    j->res.slots = c.nslots;
    j->opt_iterations = job->opt_iterations;
    j->tolerance = job->tolerance > 0 ? job->tolerance : 1e-3;
    j->eval.assign(job->eval, job->eval + n);
    j->evec.assign(job->evec, job->evec + (size_t)n * n);
    j->inv.assign(job->inv_evec, job->inv_evec + (size_t)n * n);
    j->rates.assign(job->rates, job->rates + C);
    j->props.assign(job->props, job->props + C);
    j->pi.assign(job->state_freq, job->state_freq + n);
    j->tip.assign(job->tip_lh, job->tip_lh + (size_t)(S + 1) * n);
    j->freq.assign(job->ptn_freq, job->ptn_freq + P);
    j->states.assign(job->tip_states, job->tip_states + (size_t)T * P);
    j->edges.assign(job->edges, job->edges + 2 * (2 * T - 3));
    j->lengths.assign(job->lengths, job->lengths + (2 * T - 3));
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
        iqg::set_error("server is shutting down");
        return IQGPU_ERR_STATE;
    }
    j->id = s->next_id++;
    j->res.id = j->id;
    j->res.bytes = (int64_t)bytes;
    j->res.t_submit = now_s(s->t0);
    *id = j->id;
    s->queue.push_back(j.get());
    s->jobs[j->id] = std::move(j);
    s->stats.submitted++;
    s->cv.notify_all();
    return IQGPU_OK;
}

int iqgpu_server_wait(iqgpu_server *s, int64_t id, iqgpu_job_result *out, double *lengths) {
    if (!s || !out) {
        iqg::set_error("null argument");
        return IQGPU_ERR_ARG;
    }
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) {
        iqg::set_error("unknown job id");
        return IQGPU_ERR_ARG;
    }
    Job *j = it->second.get();
    s->cv.wait(lk, [&] { return j->done; });
    *out = j->res;
    if (lengths && !j->out_lengths.empty()) std::memcpy(lengths, j->out_lengths.data(), j->out_lengths.size() * 8);
    std::thread w = std::move(j->worker);
    lk.unlock();
    if (w.joinable()) w.join();
    return IQGPU_OK;
}

int iqgpu_server_get_stats(iqgpu_server *s, iqgpu_server_stats *out) {
    if (!s || !out) {
        iqg::set_error("null argument");
        return IQGPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    return IQGPU_OK;
}

int iqgpu_server_destroy(iqgpu_server *s) {
    if (!s) return IQGPU_OK;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        s->cv.wait(lk, [&] { return s->queue.empty() && s->active == 0; });  // finish admitted work
        s->stop = true;
        s->cv.notify_all();
    }
    if (s->scheduler.joinable()) s->scheduler.join();
    for (auto &kv : s->jobs)
        if (kv.second->worker.joinable()) kv.second->worker.join();
    cudaSetDevice(s->cfg.device);
    cudaFree(s->arena.base);
    delete s;
    return IQGPU_OK;
}

}  // extern "C"
