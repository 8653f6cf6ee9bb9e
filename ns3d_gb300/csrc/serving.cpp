// serving.cpp -- many permeability solves on one GPU: a batch call and a
// continuous-batching server.
//
// Every solve owns a solver instance (its geometry, fields and Krylov state
// resident in HBM until it converges) and its own CUDA stream, so the kernels
// of concurrent solves overlap on the device.  The server admits queued
// requests as soon as a slot is free and the device reports enough free
// memory for the request's estimated footprint; finished solves release
// their memory at once (stream-ordered, into the library's pool, without
// synchronizing the device) and the next requests are admitted -- continuous
// batching, not a queue in front of one solver.  Results do not depend on
// what else runs: every kernel uses a fixed reduction order, so a solve gives
// bit-identical fields alone and in the mix.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <string>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ns3d_capi.h"

namespace ns3d {
size_t pool_cached_bytes();  // solver.cu: device memory the library pool holds free
}

namespace {

using Clock = std::chrono::steady_clock;

// device bytes of one solve, from the image size: index maps, four systems
// (coefficients, neighbour columns, Krylov workspace) and the fields; the
// mixed path adds its FP32 copies.  A conservative per-cell bound.
size_t estimate_bytes(const ns3d_params &p, int nx, int ny, int nz) {
    const double cells = (double)(nx + 2 * std::max(p.border, 0) + 1) * ny * nz;
    const double per_cell = 4 * 4 + 4 * 200.0 + (p.precision == NS3D_MIXED ? 4 * 72.0 : 0.0);
    return (size_t)(cells * per_cell) + (64u << 20);
}

struct Job {
    int64_t ticket = 0;
    ns3d_params params;
    std::vector<uint8_t> raw;
    const uint8_t *ext = nullptr;  // caller-owned image (ns3d_server_submit_resident), not copied
    int nx = 0, ny = 0, nz = 0;
    size_t bytes = 0;
    int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
    int status = NS3D_OK;
    ns3d_result result;
    std::vector<double> fields[4];
    bool keep_fields = false;
    std::string error;  // ns3d_last_error() of a failed request
    Clock::time_point submitted, started, finished;
};

int run_one(Job &j, ns3d_group *group) {
    ns3d_handle *h = nullptr;
    int rc = ns3d_open(&j.params, j.ext ? j.ext : j.raw.data(), j.nx, j.ny, j.nz, &h);
    if (rc != NS3D_OK) return rc;
    if (group) rc = ns3d_set_group(h, group);
    if (rc == NS3D_OK) rc = ns3d_solve(h);
    if (rc == NS3D_OK) rc = ns3d_get_result(h, &j.result);
    if (rc == NS3D_OK && j.keep_fields) {
        ns3d_sizes s;
        ns3d_get_sizes(h, &s);
        j.fields[0].resize(s.np);
        j.fields[1].resize(s.nu);
        j.fields[2].resize(s.nv);
        j.fields[3].resize(s.nw);
        rc = ns3d_get_fields(h, j.fields[0].data(), j.fields[1].data(), j.fields[2].data(), j.fields[3].data());
    }
    ns3d_close(h);
    return rc;
}

}  // namespace

struct ns3d_server {
    int max_active = 1;
    size_t hbm_budget = 0;  // 0: whatever the device reports free
    int device = 0;
    std::mutex mu;
    std::condition_variable cv, done_cv;
    std::deque<Job *> queue;
    std::map<int64_t, std::unique_ptr<Job>> jobs;
    std::thread scheduler;
    int active = 0, peak_active = 0;
    size_t reserved = 0;
    bool stopping = false;
    int64_t next_ticket = 1;
    std::vector<double> latencies;
    Clock::time_point first_submit, last_finish;
    bool any = false;
    int64_t completed = 0, failed = 0;
    ns3d_group *group = nullptr;  // merged solve sets (ns3d_server_set_merging)

    // device memory available to a new solve: free memory plus what the
    // library pool holds released by finished solves (queried without the
    // server lock: the call can take a while when the device is busy)
    size_t available_bytes() {
        size_t free_b = 0, total_b = 0;
        cudaSetDevice(device);
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 0;
        size_t cached = 0;
        try {
            cached = ns3d::pool_cached_bytes();
        } catch (...) {
        }
        return free_b + cached;
    }

    void schedule_loop() {
        std::unique_lock<std::mutex> lk(mu);
        while (true) {
            cv.wait(lk, [&] { return stopping || (!queue.empty() && active < max_active); });
            if (stopping && queue.empty()) return;
            if (queue.empty() || active >= max_active) continue;
            Job *j = queue.front();
            bool ok;
            if (hbm_budget) {
                ok = reserved + j->bytes <= hbm_budget || active == 0;
            } else {
                lk.unlock();
                const size_t avail = available_bytes();
                lk.lock();
                if (queue.empty() || queue.front() != j || active >= max_active) continue;  // changed meanwhile
                // keep 2 GiB of head room beyond the estimates of running solves
                ok = j->bytes + (2ull << 30) <= avail || active == 0;
            }
            if (!ok) {  // wait for a running solve to release memory
                cv.wait_for(lk, std::chrono::milliseconds(5));
                continue;
            }
            queue.pop_front();
            j->state = 1;
            j->started = Clock::now();
            active++;
            peak_active = std::max(peak_active, active);
            reserved += j->bytes;
            // a worker touches the server only under the lock and until it
            // has decremented `active`; stop waits for active == 0
            std::thread([this, j] { work(j); }).detach();
        }
    }

    void work(Job *j) {
        cudaSetDevice(device);
        int rc = run_one(*j, group);
        if (rc != NS3D_OK) {
            j->error = ns3d_last_error();  // the worker thread's error text
            std::fprintf(stderr, "ns3d server: request %lld failed (%d): %s\n", (long long)j->ticket, rc,
                         j->error.c_str());
        }
        std::lock_guard<std::mutex> lk(mu);
        j->finished = Clock::now();
        j->status = rc;
        j->state = rc == NS3D_OK ? 2 : 3;
        active--;
        reserved -= j->bytes;
        if (rc == NS3D_OK) {
            completed++;
            latencies.push_back(std::chrono::duration<double>(j->finished - j->submitted).count());
        } else {
            failed++;
        }
        last_finish = j->finished;
        cv.notify_all();
        done_cv.notify_all();
    }
};

static double percentile(std::vector<double> v, double q) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    double pos = q * (v.size() - 1);
    size_t lo = (size_t)pos;
    size_t hi = std::min(lo + 1, v.size() - 1);
    return v[lo] + (pos - lo) * (v[hi] - v[lo]);
}

extern "C" {

NS3D_API int ns3d_server_start(int32_t max_active, size_t hbm_budget_bytes, ns3d_server **out) {
    if (!out || max_active <= 0) return NS3D_ERR_ARG;
    ns3d_server *s = new ns3d_server();
    s->max_active = max_active;
    s->hbm_budget = hbm_budget_bytes;
    cudaGetDevice(&s->device);
    s->scheduler = std::thread([s] { s->schedule_loop(); });
    *out = s;
    return NS3D_OK;
}

static int submit(ns3d_server *s, const ns3d_params *p, const uint8_t *raw, int32_t nx, int32_t ny, int32_t nz,
                  int32_t keep_fields, int64_t *ticket, bool copy) {
    if (!s || !p || !raw || !ticket || nx <= 0 || ny <= 0 || nz <= 0) return NS3D_ERR_ARG;
    std::unique_ptr<Job> j(new Job());
    j->params = *p;
    if (copy) j->raw.assign(raw, raw + (size_t)nx * ny * nz);
    else j->ext = raw;
    j->nx = nx;
    j->ny = ny;
    j->nz = nz;
    j->keep_fields = keep_fields != 0;
    j->bytes = estimate_bytes(*p, nx, ny, nz);
    std::memset(&j->result, 0, sizeof j->result);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) return NS3D_ERR_STATE;
    j->ticket = s->next_ticket++;
    j->submitted = Clock::now();
    if (!s->any) {
        s->first_submit = j->submitted;
        s->any = true;
    }
    *ticket = j->ticket;
    s->queue.push_back(j.get());
    s->jobs[j->ticket] = std::move(j);
    s->cv.notify_all();
    return NS3D_OK;
}

NS3D_API int ns3d_server_submit(ns3d_server *s, const ns3d_params *p, const uint8_t *raw, int32_t nx, int32_t ny,
                                int32_t nz, int32_t keep_fields, int64_t *ticket) {
    return submit(s, p, raw, nx, ny, nz, keep_fields, ticket, true);
}

NS3D_API int ns3d_server_submit_resident(ns3d_server *s, const ns3d_params *p, const uint8_t *raw, int32_t nx,
                                         int32_t ny, int32_t nz, int32_t keep_fields, int64_t *ticket) {
    return submit(s, p, raw, nx, ny, nz, keep_fields, ticket, false);
}

/* state: 0 queued, 1 running, 2 done, 3 failed */
NS3D_API int ns3d_server_poll(ns3d_server *s, int64_t ticket, int32_t *state, ns3d_result *result) {
    if (!s || !state) return NS3D_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return NS3D_ERR_ARG;
    *state = it->second->state;
    if (result && it->second->state == 2) *result = it->second->result;
    return it->second->state == 3 ? it->second->status : NS3D_OK;
}

NS3D_API int ns3d_server_wait(ns3d_server *s, int64_t ticket, ns3d_result *result, double *latency_s) {
    if (!s) return NS3D_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return NS3D_ERR_ARG;
    Job *j = it->second.get();
    s->done_cv.wait(lk, [&] { return j->state >= 2; });
    if (result) *result = j->result;
    if (latency_s) *latency_s = std::chrono::duration<double>(j->finished - j->submitted).count();
    return j->state == 2 ? NS3D_OK : j->status;
}

NS3D_API int ns3d_server_fields(ns3d_server *s, int64_t ticket, double *p, double *u, double *v, double *w) {
    if (!s) return NS3D_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end() || it->second->state != 2 || !it->second->keep_fields) return NS3D_ERR_STATE;
    double *dst[4] = {p, u, v, w};
    for (int k = 0; k < 4; ++k)
        if (dst[k]) std::memcpy(dst[k], it->second->fields[k].data(), it->second->fields[k].size() * sizeof(double));
    return NS3D_OK;
}

NS3D_API int ns3d_server_get_stats(ns3d_server *s, ns3d_server_stats *out) {
    if (!s || !out) return NS3D_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof *out);
    out->completed = s->completed;
    out->failed = s->failed;
    out->queued = (int64_t)s->queue.size();
    out->active = s->active;
    out->peak_active = s->peak_active;
    out->p50_latency_s = percentile(s->latencies, 0.50);
    out->p99_latency_s = percentile(s->latencies, 0.99);
    out->mean_latency_s = s->latencies.empty() ? 0.0
        : std::accumulate(s->latencies.begin(), s->latencies.end(), 0.0) / s->latencies.size();
    double span = s->any ? std::chrono::duration<double>(s->last_finish - s->first_submit).count() : 0.0;
    out->solves_per_s = span > 0 ? s->completed / span : 0.0;
    return NS3D_OK;
}

NS3D_API int ns3d_server_cancel_queued(ns3d_server *s, int64_t *cancelled) {
    if (!s) return NS3D_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    int64_t n = 0;
    for (Job *j : s->queue) {
        j->state = 3;
        j->status = NS3D_ERR_STATE;
        j->finished = Clock::now();
        ++n;
    }
    s->queue.clear();
    if (cancelled) *cancelled = n;
    s->done_cv.notify_all();
    return NS3D_OK;
}

NS3D_API int ns3d_server_stop(ns3d_server *s) {
    if (!s) return NS3D_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        s->cv.notify_all();
    }
    s->scheduler.join();
    {
        // the scheduler returns once the queue is empty; wait for running solves
        std::unique_lock<std::mutex> lk(s->mu);
        s->done_cv.wait(lk, [&] { return s->active == 0; });
    }
    if (s->group) ns3d_group_destroy(s->group);
    delete s;
    return NS3D_OK;
}

NS3D_API int ns3d_server_set_merging(ns3d_server *s, int32_t lanes) {
    if (!s || lanes < 0) return NS3D_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->any) return NS3D_ERR_STATE;  // before the first request only
    if (s->group) {
        ns3d_group_destroy(s->group);
        s->group = nullptr;
    }
    if (lanes > 0) {
        cudaSetDevice(s->device);
        return ns3d_group_create(lanes, &s->group);
    }
    return NS3D_OK;
}

NS3D_API int ns3d_server_group_stats(ns3d_server *s, ns3d_group_stats *out) {
    if (!s || !out) return NS3D_ERR_ARG;
    std::memset(out, 0, sizeof *out);
    return s->group ? ns3d_group_get_stats(s->group, out) : NS3D_OK;
}

static int batch_solve(const ns3d_params *params, const uint8_t *const *raws, const int32_t *dims, int32_t njobs,
                       int32_t max_concurrent, int32_t lanes, ns3d_result *results, int32_t *status,
                       ns3d_group_stats *gstats) {
    if (!params || !raws || !dims || !results || njobs < 0 || max_concurrent <= 0) return NS3D_ERR_ARG;
    ns3d_server *s = nullptr;
    int rc = ns3d_server_start(max_concurrent, 0, &s);
    if (rc != NS3D_OK) return rc;
    if (lanes > 0 && (rc = ns3d_server_set_merging(s, lanes)) != NS3D_OK) {
        ns3d_server_stop(s);
        return rc;
    }
    std::vector<int64_t> tickets((size_t)njobs);
    for (int i = 0; i < njobs; ++i) {
        rc = ns3d_server_submit(s, &params[i], raws[i], dims[3 * i], dims[3 * i + 1], dims[3 * i + 2], 0,
                                &tickets[(size_t)i]);
        if (rc != NS3D_OK) {
            ns3d_server_stop(s);
            return rc;
        }
    }
    int worst = NS3D_OK;
    for (int i = 0; i < njobs; ++i) {
        int r = ns3d_server_wait(s, tickets[(size_t)i], &results[i], nullptr);
        if (status) status[i] = r;
        if (r != NS3D_OK) worst = r;
    }
    if (gstats) ns3d_server_group_stats(s, gstats);
    ns3d_server_stop(s);
    return worst;
}

NS3D_API int ns3d_batch_solve(const ns3d_params *params, const uint8_t *const *raws, const int32_t *dims,
                              int32_t njobs, int32_t max_concurrent, ns3d_result *results, int32_t *status) {
    return batch_solve(params, raws, dims, njobs, max_concurrent, 0, results, status, nullptr);
}

NS3D_API int ns3d_batch_solve_merged(const ns3d_params *params, const uint8_t *const *raws, const int32_t *dims,
                                     int32_t njobs, int32_t max_concurrent, int32_t lanes, ns3d_result *results,
                                     int32_t *status, ns3d_group_stats *stats) {
    if (lanes < 1) return NS3D_ERR_ARG;
    return batch_solve(params, raws, dims, njobs, max_concurrent, lanes, results, status, stats);
}

}  // extern "C"
