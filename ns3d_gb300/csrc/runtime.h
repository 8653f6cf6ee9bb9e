// runtime.h -- device memory ownership and the batched Krylov driver.
#pragma once

#include <cuda_runtime.h>

#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ns3d_capi.h"
#include "device.cuh"
#include "kernels.h"
#include "mixed.h"

namespace ns3d {

struct CudaError : std::runtime_error {
    cudaError_t code;
    CudaError(cudaError_t e, const char *expr, const char *file, int line)
        : std::runtime_error(std::string(cudaGetErrorString(e)) + " in " + expr + " (" + file + ":" +
                             std::to_string(line) + ")"),
          code(e) {}
};

struct ApiError : std::runtime_error {
    int code;
    ApiError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// records the text ns3d_last_error() returns on this thread; returns code
int report_error(int code, const std::string &m);

// owning device buffer
// Device memory of the library: one stream-ordered pool per device, kept
// reserved between solves (no cudaMalloc / cudaFree, which synchronize the
// whole device and would stall every other solve running in the process).
cudaMemPool_t device_pool();
// bytes the pool holds reserved but unused (free for new solves)
size_t pool_cached_bytes();

// Device array allocated on a stream from the library pool and freed on the
// same stream (stream-ordered: it may be released while work that uses it
// is still queued on that stream).
template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t st_ = nullptr;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { release(); }
    void alloc(size_t count, cudaStream_t st) {
        release();
        n = count;
        st_ = st;
        if (count == 0) return;
        cudaError_t e = cudaMallocFromPoolAsync((void **)&p, count * sizeof(T), device_pool(), st);
        if (e != cudaSuccess) {
            p = nullptr;
            n = 0;
            cudaGetLastError();
            throw ApiError(NS3D_ERR_OOM, "device allocation of " + std::to_string(count * sizeof(T)) + " bytes failed");
        }
    }
    void alloc_zero(size_t count, cudaStream_t st) {
        alloc(count, st);
        if (count) NS3D_CUDA_CHECK(cudaMemsetAsync(p, 0, count * sizeof(T), st));
    }
    void release() {
        if (p) cudaFreeAsync(p, st_);
        p = nullptr;
        n = 0;
    }
};

// Host staging array of the small per-solve state copies.  Pageable memory:
// a device-to-host copy into it returns once the copy is done, and freeing
// it does not synchronize the device (cudaFreeHost would).
template <class T>
struct HBuf {
    std::vector<T> v;
    T *p = nullptr;
    size_t n = 0;
    void alloc(size_t count) {
        v.assign(count, T());
        p = count ? v.data() : nullptr;
        n = count;
    }
};

inline int pad_rows(int n) { return ((n + CH - 1) / CH) * CH; }

// one linear system (momentum component or pressure) and its Krylov workspace
// Device arrays of the multilevel hierarchy of one system (MIXED_MG)
struct MGHostLevel {
    int n = 0, npad = 0;
    DBuf<int> nbr, agg, mstart, members;
    DBuf<float> coef, invdiag, x, b, t;
};
struct MGHost {
    int nlev = 0;
    MGHostLevel lev[MG_MAX + 1];
};

struct DevSys {
    int n = 0, npad = 0, nchunks = 0, d0 = 0;
    int cell_ny = 0, cell_nz = 0;  // extents of the map behind `cell` (cell = (i ny + j) nz + k)
    std::unique_ptr<MGHost> mg;    // built on first MIXED_MG use
    DBuf<int> cell;
    DBuf<double> coef;
    DBuf<int> nbr;
    DBuf<double> rhs, rowsum, invdiag;
    DBuf<double> r, r0, p, v, y, s, z, t, part;
    // FP32 copy of the system and the FP32 Krylov vectors (mixed precision),
    // allocated on first use
    DBuf<float> coef32, invdiag32, fx, fr, fr0, fp, fv, fy, fs, fz, ft, fp2, fv2;
    void allocate(int rows, int first_extent, cudaStream_t st);
    void allocate_f32(cudaStream_t st);
    SysView view() const {
        SysView sv;
        sv.n = n;
        sv.npad = npad;
        sv.nchunks = nchunks;
        sv.cell = cell.p;
        sv.coef = coef.p;
        sv.nbr = nbr.p;
        sv.rhs = rhs.p;
        sv.rowsum = rowsum.p;
        sv.invdiag = invdiag.p;
        return sv;
    }
    size_t device_bytes() const;
};

struct SolveItem {
    DevSys *sys;
    double *x;        // guess in, solution out (npad doubles)
    const double *b;  // right-hand side (npad doubles)
    double tol;
    int maxit;
    bool mg = false;  // merged mixed sets: the system's own set chose the multilevel preconditioner
};

struct SolveOutcome {
    int iters = 0, info = 0, work = 0;
    double error = 0;
    bool valid = false;
};

// A CUDA stream destroyed after the buffers that are freed on it: declare it
// before them in a class (members are destroyed in reverse order).
struct OwnedStream {
    cudaStream_t s = nullptr;
    ~OwnedStream() {
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
};

// A set of up to CAP systems solved together by the BiCGSTAB loop kernel
// (KrylovSet: one solver instance's systems; KrylovSetMerged: the systems of
// many concurrent solves, see SolveGroup).
template <int CAP>
class KrylovSetT {
  public:
    void run(const std::vector<SolveItem> &items, cudaStream_t st, std::vector<SolveOutcome> &out);
    const KState *device_state(int i) const { return st_.p + i; }
    // allocates the per-system state of `items` (and records them) without
    // solving: a merged run copies the final states here
    void prepare(const std::vector<SolveItem> &items, cudaStream_t st) { configure(items, st); }
    KState *state_buffer() { return st_.p; }
    long launches() const { return launches_; }
    void reset_launch_count() { launches_ = 0; }

    // timing of the loop kernel: phases K1..K5 (index 0..4, block 0's view
    // between grid barriers, global timer) and whole launches (index 5,
    // CUDA events); rows = row-iterations
    struct Profile {
        int64_t launches[6] = {0, 0, 0, 0, 0, 0};
        double ms[6] = {0, 0, 0, 0, 0, 0};
        int64_t rows[6] = {0, 0, 0, 0, 0, 0};
    };
    bool profiling = false;
    Profile prof;
    int share = 1;  // a merged set's loop launches take 1/share of the SMs
    ~KrylovSetT();

  private:
    void configure(const std::vector<SolveItem> &items, cudaStream_t st);
    cudaEvent_t ev_[2] = {nullptr, nullptr};
    KSetArgT<CAP> set_;  // passed to every kernel by value
    DBuf<KState> st_;
    HBuf<KState> h_st_, h_up_;
    DBuf<GridBar> bar_;
    DBuf<LoopProf> prof_;
    HBuf<int> h_err_;
    int nsys_ = 0, total_chunks_ = 0;
    long launches_ = 0;
};
using KrylovSet = KrylovSetT<KMAX>;
using KrylovSetMerged = KrylovSetT<KMAX_MERGED>;


struct DCState;

#ifndef NS3D_MIXED_INNER_TOL
#define NS3D_MIXED_INNER_TOL 1e-4
#endif
#ifndef NS3D_MIXED_INNER_CAP
#define NS3D_MIXED_INNER_CAP 400
#endif

// A set of systems solved by FP32 BiCGSTAB inside FP64 defect correction.
// The FP32 copy of each matrix is refreshed from the FP64 one at every run.
// MixedSet: one solver instance's systems; MixedSetMerged: the systems of
// many concurrent solves (SolveGroup), each with the preconditioner and FP32
// loop variant its own set chose.
template <int CAP>
class MixedSetT {
  public:
    // variant: -1 from the set's own rows, 0 five-phase, 1 fused FP32 loop
    void run(const std::vector<SolveItem> &items, cudaStream_t st, std::vector<SolveOutcome> &out,
             int variant = -1);
    const KState *inner_state(int i) const { return st_.p + i; }
    // FP64 outcome of system i, mirrored into a KState (iter, info) for the
    // velocity post-processing kernel
    const KState *device_state(int i) const { return out_st_.p + i; }
    // set-up without solving (FP32 buffers, hierarchy, state buffers): a
    // merged run solves these items and leaves the outcome states here
    void prepare(const std::vector<SolveItem> &items, cudaStream_t st) { configure(items, st); }
    KState *out_state_buffer() { return out_st_.p; }
    bool uses_mg(int i) const { return set_.sys[i].mg.nlev > 0; }
    int variant() const;  // the FP32 loop variant this set runs (0 five-phase, 1 fused)
    bool use_mg = false;                          // multilevel preconditioner for single-system sets
    double inner_rel_tol = NS3D_MIXED_INNER_TOL;  // floor of the per-round FP32 reduction target
    int inner_cap = NS3D_MIXED_INNER_CAP;         // FP32 iterations per round at most
    int share = 1;                                // a merged set's loop launches take 1/share of the SMs
    ~MixedSetT();

  private:
    void configure(const std::vector<SolveItem> &items, cudaStream_t st);
    cudaEvent_t ev_[2] = {nullptr, nullptr};  // around the FP32 loop launch (merged sets: autotuner timing)
    DBuf<KState> st_, out_st_;
    DBuf<DCState> dc_;
    HBuf<KState> h_st_, h_out_;
    HBuf<DCState> h_dc_;
    std::vector<const double *> key_;
    MSetArgT<CAP> set_;  // passed to every kernel by value
    DBuf<GridBar> bar_;
    HBuf<int> h_err_;
    int nsys_ = 0, total_chunks_ = 0;
};
using MixedSet = MixedSetT<KMAX>;
using MixedSetMerged = MixedSetT<KMAX_MERGED_M>;

// The BiCGSTAB work of many concurrent solver instances merged into shared
// persistent kernels: each member's solve sets (its momentum components,
// its pressure system; FP64, or FP32 inside FP64 defect correction) are
// queued here, and a member (the leader of a lane) gathers queued sets of
// one kind -- FP64, or mixed precision with one FP32 loop variant -- up to
// KMAX_MERGED (FP64) or KMAX_MERGED_M (mixed) systems, and solves them
// together on the lane's stream: every launch covers the ragged list of all
// their 1024-row chunks.  The members are split into cohorts, one per lane
// (at most ceil(members / lanes) sets per merged solve); a leader waits for
// a full cohort up to a short window (members run their outer iterations in
// near lockstep), so launches stay full, while the lanes run side by side:
// one cohort's solves overlap another's assembly and host work.  Each
// system keeps its own scalars, reduction order and preconditioner, so a
// solve gives the same bits alone and merged.
class SolveGroup {
  public:
    explicit SolveGroup(int lanes = 1);
    ~SolveGroup();
    // a solve of a member starts / ends (the leader waits for members only)
    void join();
    void leave();
    // Solves the FP64 set `items` (whose inputs are ready on `st`) with
    // whatever else the members queue meanwhile.  On return `out` holds the
    // outcomes, the final state of item i is in state_dst[i] (device), and
    // work queued on `st` afterwards runs after the merged launches.
    void run(const std::vector<SolveItem> &items, cudaStream_t st, KState *state_dst,
             std::vector<SolveOutcome> &out);
    // The same for a mixed-precision set (its items carry their
    // preconditioner choice; variant: the set's FP32 loop variant); the
    // outcome state of item i (MixedSet::device_state) lands in state_dst[i].
    void run_mixed(const std::vector<SolveItem> &items, cudaStream_t st, KState *state_dst,
                   std::vector<SolveOutcome> &out, int variant);
    struct Stats {
        int64_t launches = 0, requests = 0, systems = 0;
        int max_systems = 0, max_requests = 0;
    };
    Stats stats();
    double window_s = 2e-3;  // longest wait of a leader for the other members

    int lanes() const { return (int)lanes_.size(); }
    // a member is solving or a set is queued or being solved
    bool busy();
    // Marks the group closed if it is idle (under the group's lock, so no
    // solve can join between the check and the mark) and returns true;
    // false while it is busy.  join() of a closed group throws
    // NS3D_ERR_STATE.  Threads that still hold the group after it is
    // destroyed are the caller's to prevent.
    bool close_if_idle();

  private:
    struct Req;
    struct Lane {  // a stream and the merged sets solved on it
        cudaStream_t stream = nullptr;
        std::unique_ptr<KrylovSetMerged> set;
        std::unique_ptr<MixedSetMerged> mset;
        bool busy = false;
        ~Lane();  // frees the sets' buffers on the stream, then the stream
    };
    void submit(Req &r);
    void execute(Lane &lane, std::vector<Req *> &batch);
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<Req *> pending_;
    int members_ = 0;
    bool closing_ = false;  // set by close_if_idle: the group is being destroyed
    Stats stats_;
    std::vector<std::unique_ptr<Lane>> lanes_;
};
// the solve group behind a C-ABI group handle (NULL for NULL)
SolveGroup *group_of(ns3d_group *g);

}  // namespace ns3d
