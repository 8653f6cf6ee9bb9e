// group.cu -- merged solve sets: the BiCGSTAB work of many concurrent solves
// in one set of persistent kernels (SolveGroup, runtime.h), and its C-ABI.
//
// A member thread queues its set and waits.  A waiting member whose set is
// still queued becomes the leader of a free lane: it waits until a cohort
// of sets is queued (ceil(members / lanes), or window_s passes), takes the
// oldest queued set and the later ones of the same kind in arrival order,
// up to the cohort and the merged capacity (KMAX_MERGED FP64 or
// KMAX_MERGED_M mixed systems), orders the lane's stream after each
// member's stream (an event per set), runs the merged set, copies each
// system's final state back to its member, and orders each member's stream
// after the merged launch (a second event per set).  A lane has one leader
// at a time, so its stream and its sets have a single user.
#include <algorithm>
#include <chrono>
#include <cstring>

#include "runtime.h"

namespace ns3d {

struct SolveGroup::Req {
    int kind = 0;  // 0: FP64; 1 + v: mixed precision, FP32 loop variant v
    const std::vector<SolveItem> *items = nullptr;
    cudaStream_t st = nullptr;
    KState *dst = nullptr;
    std::vector<SolveOutcome> *out = nullptr;
    cudaEvent_t ready = nullptr, fin = nullptr;
    bool taken = false, done = false;
    int err_code = NS3D_OK;
    std::string err;
};

SolveGroup::SolveGroup(int lanes) {
    for (int i = 0; i < std::max(lanes, 1); ++i) {
        std::unique_ptr<Lane> l(new Lane());
        NS3D_CUDA_CHECK(cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking));
        l->set.reset(new KrylovSetMerged());
        l->mset.reset(new MixedSetMerged());
        l->set->share = std::max(lanes, 1);  // the lanes' launches run side by side
        l->mset->share = std::max(lanes, 1);
        lanes_.push_back(std::move(l));
    }
}

SolveGroup::Lane::~Lane() {
    set.reset();  // their buffers are freed on the lane's stream
    mset.reset();
    if (stream) {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
}

SolveGroup::~SolveGroup() = default;

void SolveGroup::join() {
    std::lock_guard<std::mutex> lk(mu_);
    if (closing_) throw ApiError(NS3D_ERR_STATE, "the solve group is being destroyed");
    members_++;
}

void SolveGroup::leave() {
    std::lock_guard<std::mutex> lk(mu_);
    members_--;
    cv_.notify_all();  // a leader waiting for this member stops waiting
}

bool SolveGroup::busy() {
    std::lock_guard<std::mutex> lk(mu_);
    if (members_ > 0 || !pending_.empty()) return true;
    for (auto &l : lanes_)
        if (l->busy) return true;
    return false;
}

bool SolveGroup::close_if_idle() {
    std::lock_guard<std::mutex> lk(mu_);
    if (members_ > 0 || !pending_.empty()) return false;
    for (auto &l : lanes_)
        if (l->busy) return false;
    closing_ = true;
    return true;
}

SolveGroup::Stats SolveGroup::stats() {
    std::lock_guard<std::mutex> lk(mu_);
    return stats_;
}

void SolveGroup::execute(Lane &lane, std::vector<Req *> &batch) {
    const cudaStream_t st = lane.stream;
    auto fail = [&](int code, const std::string &m) {
        // the members' buffers may still be in use by queued work: drain the
        // lane's stream before any member returns with the error
        cudaStreamSynchronize(st);
        for (Req *q : batch) {
            q->err_code = code;
            q->err = m;
        }
    };
    try {
        std::vector<SolveItem> all;
        for (Req *q : batch) {
            NS3D_CUDA_CHECK(cudaStreamWaitEvent(st, q->ready, 0));
            all.insert(all.end(), q->items->begin(), q->items->end());
        }
        std::vector<SolveOutcome> out;
        const int kind = batch.front()->kind;
        if (kind == 0) lane.set->run(all, st, out);
        else lane.mset->run(all, st, out, kind - 1);
        size_t off = 0;
        for (Req *q : batch) {
            const size_t n = q->items->size();
            q->out->assign(out.begin() + off, out.begin() + off + n);
            const KState *src = kind == 0 ? lane.set->device_state((int)off) : lane.mset->device_state((int)off);
            if (q->dst && n)
                NS3D_CUDA_CHECK(
                    cudaMemcpyAsync(q->dst, src, n * sizeof(KState), cudaMemcpyDeviceToDevice, st));
            NS3D_CUDA_CHECK(cudaEventRecord(q->fin, st));
            off += n;
        }
    } catch (const ApiError &e) {
        fail(e.code, e.what());
    } catch (const std::bad_alloc &) {
        fail(NS3D_ERR_OOM, "host allocation failed");
    } catch (const std::exception &e) {
        fail(NS3D_ERR_CUDA, e.what());
    }
}

void SolveGroup::run(const std::vector<SolveItem> &items, cudaStream_t st, KState *state_dst,
                     std::vector<SolveOutcome> &out) {
    Req r;
    r.items = &items;
    r.st = st;
    r.dst = state_dst;
    r.out = &out;
    submit(r);
}

void SolveGroup::run_mixed(const std::vector<SolveItem> &items, cudaStream_t st, KState *state_dst,
                           std::vector<SolveOutcome> &out, int variant) {
    Req r;
    r.kind = 1 + (variant == 1 ? 1 : 0);
    r.items = &items;
    r.st = st;
    r.dst = state_dst;
    r.out = &out;
    submit(r);
}

static int capacity(int kind) { return kind == 0 ? KMAX_MERGED : KMAX_MERGED_M; }

void SolveGroup::submit(Req &r) {
    if ((int)r.items->size() > capacity(r.kind))
        throw ApiError(NS3D_ERR_ARG, "too many systems in one solve set");
    struct Events {  // destroyed on every path (a wait already issued keeps its event alive)
        Req &q;
        ~Events() {
            if (q.ready) cudaEventDestroy(q.ready);
            if (q.fin) cudaEventDestroy(q.fin);
        }
    } events{r};
    NS3D_CUDA_CHECK(cudaEventCreateWithFlags(&r.ready, cudaEventDisableTiming));
    NS3D_CUDA_CHECK(cudaEventCreateWithFlags(&r.fin, cudaEventDisableTiming));
    NS3D_CUDA_CHECK(cudaEventRecord(r.ready, r.st));
    std::unique_lock<std::mutex> lk(mu_);
    pending_.push_back(&r);
    cv_.notify_all();
    while (!r.done) {
        Lane *lane = nullptr;
        if (!r.taken)
            for (auto &l : lanes_)
                if (!l->busy) {
                    lane = l.get();
                    break;
                }
        if (!lane) {  // taken by a leader, or every lane busy
            cv_.wait(lk);
            continue;
        }
        // lead one merged solve on this lane: wait (up to the window) for a
        // cohort, then take the oldest queued set and the later ones of its
        // kind, in arrival order, while they fit the cohort and the set
        lane->busy = true;
        const int cohort = std::max(1, (members_ + lanes() - 1) / lanes());
        const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(window_s);
        cv_.wait_until(lk, deadline, [&] { return (int)pending_.size() >= cohort; });
        if (pending_.empty()) {  // another lane's leader took every queued set (this one's too)
            lane->busy = false;
            cv_.notify_all();
            continue;
        }
        std::vector<Req *> batch;
        batch.reserve(pending_.size());
        int systems = 0;
        const int kind = pending_.front()->kind;
        for (auto it = pending_.begin(); it != pending_.end() && (int)batch.size() < cohort;) {
            Req *q = *it;
            const int n = (int)q->items->size();
            if (q->kind != kind) {
                ++it;
                continue;
            }
            if (!batch.empty() && systems + n > capacity(kind)) break;
            it = pending_.erase(it);
            q->taken = true;
            batch.push_back(q);
            systems += n;
        }
        stats_.launches++;
        stats_.requests += (int64_t)batch.size();
        stats_.systems += systems;
        stats_.max_systems = std::max(stats_.max_systems, systems);
        stats_.max_requests = std::max(stats_.max_requests, (int)batch.size());
        lk.unlock();
        execute(*lane, batch);
        lk.lock();
        for (Req *q : batch) q->done = true;
        lane->busy = false;
        cv_.notify_all();
    }
    lk.unlock();
    if (r.err_code != NS3D_OK) throw ApiError(r.err_code, "merged solve set: " + r.err);
    NS3D_CUDA_CHECK(cudaStreamWaitEvent(r.st, r.fin, 0));
}

}  // namespace ns3d

using namespace ns3d;

struct ns3d_group {
    SolveGroup g;
    explicit ns3d_group(int lanes) : g(lanes) {}
};

extern "C" {

NS3D_API int ns3d_group_create(int32_t lanes, ns3d_group **out) {
    if (!out || lanes < 1 || lanes > 16) return report_error(NS3D_ERR_ARG, "bad argument");
    try {
        *out = new ns3d_group(lanes);
        return NS3D_OK;
    } catch (const CudaError &e) {
        return report_error(NS3D_ERR_CUDA, e.what());
    } catch (const std::exception &e) {
        return report_error(NS3D_ERR_OOM, e.what());
    }
}

NS3D_API int ns3d_group_get_stats(ns3d_group *g, ns3d_group_stats *out) {
    if (!g || !out) return report_error(NS3D_ERR_ARG, "NULL argument");
    const SolveGroup::Stats s = g->g.stats();
    std::memset(out, 0, sizeof *out);
    out->launches = s.launches;
    out->requests = s.requests;
    out->systems = s.systems;
    out->max_systems = s.max_systems;
    out->max_requests = s.max_requests;
    return NS3D_OK;
}

NS3D_API int ns3d_group_destroy(ns3d_group *g) {
    if (g && !g->g.close_if_idle())
        return report_error(NS3D_ERR_STATE, "ns3d_group_destroy: solves of the group are running");
    delete g;
    return NS3D_OK;
}

}  // extern "C"

namespace ns3d {
SolveGroup *group_of(ns3d_group *g) { return g ? &g->g : nullptr; }
}  // namespace ns3d
