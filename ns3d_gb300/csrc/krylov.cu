// krylov.cu -- batched Jacobi-preconditioned BiCGSTAB on the device.
//
// Replaces Eigen::BiCGSTAB<SparseMatrix<double,RowMajor>> with the default
// DiagonalPreconditioner (src/NSBase.h:97-100), called through
// solveWithGuess at src/NSBase.cxx:1799,1825,1852,2343,2393,2397.  The
// algorithm is the published right-preconditioned BiCGSTAB
// (van der Vorst 1992) with the behaviour the reference depends on:
// convergence when |r|^2 <= tol^2 |b|^2, iterations() counting completed
// iterations, error() = |r|/|b|, restart with a fresh shadow residual when
// |rho| < eps^2 |r0|^2 (the counter restarts on the first restart), and the
// zero right-hand side rule (x = 0, Success, iterations() = max).
//
// A solve set holds up to KMAX independent systems (the three momentum
// components, or the pressure system).  Their rows are processed as one list
// of 1024-row chunks; the set is passed to every kernel by value
// (__grid_constant__), so a block finds its system and the system's arrays
// in constant memory.  One BiCGSTAB iteration has five phases:
//   K1 p = r + beta (p - w v); y = D^-1 p
//   K2 v = A y, <r0,v>                      -> alpha
//   K3 s = r - alpha v; z = D^-1 s
//   K4 t = A z, <t,t>, <t,s>                -> w
//   K5 x += alpha y + w z; r = s - w t, <r0,r>, <r,r> -> convergence, beta
// All iterations of a solve run in one persistent cooperative launch
// (k_kr_loop), the phases separated by bounded grid barriers (loop.cuh).
// The set-up (r = b - A x, norms) and the restart after |rho| breakdown are
// separate launches whose last block to finish (one atomic counter per
// system) combines the partials, so they wait on no other block.
#include <atomic>
#include <cfloat>
#include <cstring>

#include "device.cuh"
#include "kernels.h"
#include "loop.cuh"

namespace ns3d {

struct Row4 {  // a thread's RPL rows
    double v[RPL];
};

// A thread's rows are r0 + m*LANES, m < RPL (coalesced across the warp).
__device__ __forceinline__ Row4 ld4(const double *p) {
    Row4 r;
#pragma unroll
    for (int m = 0; m < RPL; ++m) r.v[m] = p[m * LANES];
    return r;
}
__device__ __forceinline__ void st4(double *p, const Row4 &r) {
#pragma unroll
    for (int m = 0; m < RPL; ++m) p[m * LANES] = r.v[m];
}

// One row of y = A x: fma chain in ascending column order from 0 (the order
// of row_ordered in device.cuh).  Every gather is issued unconditionally (a
// missing neighbour reads the row's own element) so the loads of a row do
// not wait on each other; only the fused multiply-adds are predicated.  The
// two rare orders (W directly before the row, E directly after it) are taken
// only by warps that contain such a row.
// The neighbour columns come from `nb` (nb[k * stride], k = slot - 1): the
// system's table in global memory, or a chunk's copy in shared memory.
template <class Stride>
__device__ __forceinline__ double spmv_row_nb(const KSys &S, int row, const double *__restrict__ x, const int *nb,
                                              Stride stride) {
    const size_t np = (size_t)S.npad;
    const double *cf = S.coef + row;
    const int nW = nb[0 * stride], nE = nb[1 * stride], nS = nb[2 * stride], nN = nb[3 * stride],
              nB = nb[4 * stride], nT = nb[5 * stride];
    const double xP = x[row];
    const double xW = x[nW >= 0 ? nW : row], xE = x[nE >= 0 ? nE : row], xS = x[nS >= 0 ? nS : row];
    const double xN = x[nN >= 0 ? nN : row], xB = x[nB >= 0 ? nB : row], xT = x[nT >= 0 ? nT : row];
    const double cP = ro(cf), cW = ro(cf + 1 * np), cE = ro(cf + 2 * np), cS = ro(cf + 3 * np),
                 cN = ro(cf + 4 * np), cB = ro(cf + 5 * np), cT = ro(cf + 6 * np);
    const bool wlate = nW >= 0 && nW == row - 1;
    const bool eearly = nE >= 0 && nE == row + 1;
    double acc = 0.0;
    if (__any_sync(0xffffffffu, wlate || eearly)) {
        if (!wlate && nW >= 0) acc = __fma_rn(cW, xW, acc);
        if (nS >= 0) acc = __fma_rn(cS, xS, acc);
        if (nB >= 0) acc = __fma_rn(cB, xB, acc);
        if (wlate) acc = __fma_rn(cW, xW, acc);
        acc = __fma_rn(cP, xP, acc);
        if (eearly) acc = __fma_rn(cE, xE, acc);
        if (nT >= 0) acc = __fma_rn(cT, xT, acc);
        if (nN >= 0) acc = __fma_rn(cN, xN, acc);
        if (!eearly && nE >= 0) acc = __fma_rn(cE, xE, acc);
    } else {
        if (nW >= 0) acc = __fma_rn(cW, xW, acc);
        if (nS >= 0) acc = __fma_rn(cS, xS, acc);
        if (nB >= 0) acc = __fma_rn(cB, xB, acc);
        acc = __fma_rn(cP, xP, acc);
        if (nT >= 0) acc = __fma_rn(cT, xT, acc);
        if (nN >= 0) acc = __fma_rn(cN, xN, acc);
        if (nE >= 0) acc = __fma_rn(cE, xE, acc);
    }
    return acc;
}

__device__ __forceinline__ double spmv_row(const KSys &S, int row, const double *__restrict__ x) {
    return spmv_row_nb(S, row, x, S.nbr + row, (size_t)S.npad);
}

// y = A x for the thread's rows (rows >= n give garbage that callers mask)
__device__ __forceinline__ Row4 spmv4(const KSys &S, int r0, const double *__restrict__ x) {
    Row4 out;
#pragma unroll
    for (int m = 0; m < RPL; ++m) out.v[m] = spmv_row(S, r0 + m * LANES, x);
    return out;
}

// system owning global chunk c (chunk_begin ascending, first system begins
// at 0; a system without rows shares its chunk_begin with the next one, and
// both forms pick the last system whose first chunk is <= c)
template <int CAP>
__device__ __forceinline__ int sys_of_chunk(const KSetArgT<CAP> &A, int c) {
    if constexpr (CAP <= KMAX) {
        int s = 0;
#pragma unroll
        for (int q = 1; q < CAP; ++q)
            if (q < A.nsys && c >= A.sys[q].chunk_begin) s = q;
        return s;
    } else {
        int lo = 0, hi = A.nsys - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (c >= A.sys[mid].chunk_begin) lo = mid;
            else hi = mid - 1;
        }
        return lo;
    }
}

// the done/paused flags change only between kernels (or after the last
// chunk of the system arrived), so every thread of a block reads the same
__device__ __forceinline__ bool sys_active(const KSys &S) {
    return (__ldcg(&S.st->done) | __ldcg(&S.st->paused)) == 0;
}

__device__ __forceinline__ bool arrive_last(KState *st, unsigned int total, int *sh) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int prev = atomicAdd(&st->counter, 1u);
        sh[0] = (prev == total - 1) ? 1 : 0;
    }
    __syncthreads();
    bool last = sh[0] != 0;
    if (last) __threadfence();
    return last;
}

__device__ __forceinline__ void finish_loop(KState *st) {
    // loop exit: error() and info() as Eigen reports them
    st->done = 1;
    st->error = sqrt(st->rr / st->rhs_sqnorm);
    st->info = (st->error <= st->tol) ? 0 : 2;
}

#define NS3D_CHUNK_LOOP                                                        \
    for (int c = blockIdx.x; c < A.total_chunks; c += gridDim.x) {            \
        const int sidx = sys_of_chunk(A, c);                                   \
        const KSys &S = A.sys[sidx];                                           \
        const int lc = c - S.chunk_begin;                                      \
        const int r0 = lc * CH + threadIdx.x;

// ---- init: r = b - A x, r0 = r, |r|^2, |b|^2 ---------------------------------
template <int CAP>
__global__ void __launch_bounds__(LANES) k_kr_init(const __grid_constant__ KSetArgT<CAP> A) {
    __shared__ double sm[LANES];
    __shared__ int sh[2];
    NS3D_CHUNK_LOOP
        double arr = 0.0, abb = 0.0;
        {
            const Row4 ax = spmv4(S, r0, S.x);
            const Row4 b = ld4(S.b + r0);
            Row4 r;
#pragma unroll
            for (int m = 0; m < RPL; ++m) {
                r.v[m] = b.v[m] - ax.v[m];
                if (r0 + m * LANES < S.n) {
                    arr = __fma_rn(r.v[m], r.v[m], arr);
                    abb = __fma_rn(b.v[m], b.v[m], abb);
                }
            }
            st4(S.r + r0, r);
            st4(S.r0 + r0, r);
        }
        double trr, tbb;
        block_tree_sum2(arr, abb, sm, trr, tbb);
        if (threadIdx.x == 0) {
            S.part[2 * (size_t)lc + 0] = trr;
            S.part[2 * (size_t)lc + 1] = tbb;
        }
        if (arrive_last(S.st, (unsigned)S.nchunks, sh)) {
            double rr, bb;
            final_partials_sum2(S.part, S.nchunks, sm, rr, bb);
            if (threadIdx.x == 0) {
                KState *st = S.st;
                st->counter = 0;
                st->r0_sqnorm = rr;
                st->rr = rr;
                st->rhs_sqnorm = bb;
                st->iter = 0;
                st->restarts = 0;
                st->paused = 0;
                st->zero_rhs = 0;
                if (bb == 0.0) {
                    st->zero_rhs = 1;
                    st->done = 1;
                    st->iter = st->maxit;
                    st->error = st->tol;
                    st->info = 0;
                } else {
                    st->rho = 1.0;
                    st->alpha = 1.0;
                    st->w = 1.0;
                    st->tol2 = st->tol * st->tol * bb;
                    if (!(rr > st->tol2 && 0 < st->maxit)) {
                        finish_loop(st);
                    } else {
                        // first iteration: rho = <r0, r> equals |r0|^2 bit for bit
                        const double rho_old = st->rho;
                        const double rho = rr;
                        st->beta = (rho / rho_old) * (st->alpha / st->w);
                        st->rho = rho;
                        st->done = 0;
                    }
                }
            }
        }
    }
}

// p = v = 0; x = 0 for a zero right-hand side
template <int CAP>
__global__ void k_kr_init2(const __grid_constant__ KSetArgT<CAP> A) {
    NS3D_CHUNK_LOOP
        Row4 z;
#pragma unroll
        for (int m = 0; m < RPL; ++m) z.v[m] = 0.0;
        st4(S.p + r0, z);
        st4(S.v + r0, z);
        if (__ldcg(&S.st->zero_rhs)) st4(S.x + r0, z);
    }
}

// ---- the BiCGSTAB iteration loop: one persistent cooperative kernel ----------
//
// LOOP_THREADS threads per block form LOOP_GROUPS groups of LANES threads; a
// group processes whole chunks (its lanes own the rows of the fixed
// reduction order) and reduces them with a named barrier.  Every block keeps
// a copy of the per-system scalars in shared memory; after each grid-wide
// barrier every block combines the chunk partials of each system in the
// fixed order itself (group g for systems g, g + LOOP_GROUPS, ...), so all
// copies stay bit-identical without a broadcast.  Partials of the three
// reductions of an iteration go to separate regions of S.part, so a block
// that runs ahead never overwrites partials another block is still
// combining:
//   [0, 2n)  <t,t>, <t,s> pairs     [2n, 4n)  <r0,r>, <r,r> pairs
//   [4n, 5n) <r0,v>
// The loop ends when every system is done, when a system needs a restart
// (the host recomputes its residual and launches the loop again), after
// `max_iters` iterations, or when a grid barrier gives up waiting.

// rows of a chunk in flight per thread in the SpMV phases (register budget)
#ifndef NS3D_SPMV_UNROLL
#define NS3D_SPMV_UNROLL 2
#endif
constexpr int kSpmvUnroll = NS3D_SPMV_UNROLL;

// Resident neighbour tables.  The matrix does not change during a solve, and
// every group of the loop kernel processes the same chunks in every
// iteration, so each group copies the six neighbour-column slabs of its
// first chunk (6 x 1024 int32 = 24 KB) into shared memory once per launch
// and both SpMV phases of every iteration gather through that copy: 48 B
// per row-iteration less memory traffic, and the gathers of x no longer wait
// for an index load from memory.  A group that owns more chunks (systems
// above grid x LOOP_GROUPS chunks) reads the others' tables from memory.
#ifndef NS3D_NBR_SMEM
#define NS3D_NBR_SMEM 1
#endif
constexpr bool kNbrSmem = NS3D_NBR_SMEM != 0;
constexpr size_t kNbrSmemBytes = kNbrSmem ? (size_t)LOOP_GROUPS * 6 * CH * sizeof(int) : 0;

__device__ __forceinline__ bool state_active(const KState &k) { return (k.done | k.paused) == 0; }

template <int CAP>
__global__ void __launch_bounds__(LOOP_THREADS, LOOP_MIN_BLOCKS)
    k_kr_loop(const __grid_constant__ KSetArgT<CAP> A, GridBar *bar, LoopProf *prof, int max_iters) {
    static_assert(CAP <= LOOP_THREADS, "one thread copies each system's state");
    __shared__ KState sst[CAP];
    __shared__ double sm[LOOP_GROUPS][LANES];
    __shared__ int s_ok;
    extern __shared__ int s_nbr_all[];  // [LOOP_GROUPS][6][CH] when kNbrSmem
    const int gi = threadIdx.x / LANES, lane = threadIdx.x % LANES;
    const GroupSync gsync{gi + 1};
    // chunk c belongs to block c % gridDim.x (group (c / gridDim.x) % LOOP_GROUPS):
    // every block, hence every SM, gets the same number of chunks to within one
    const int gstride = gridDim.x * LOOP_GROUPS;
    const int cbegin = blockIdx.x + gridDim.x * gi;
    if (threadIdx.x < A.nsys) sst[threadIdx.x] = *A.sys[threadIdx.x].st;
    if (kNbrSmem && cbegin < A.total_chunks) {  // this group's first chunk, for the whole launch
        int *const s_nbr = s_nbr_all + (size_t)gi * 6 * CH;
        const KSys &S = A.sys[sys_of_chunk(A, cbegin)];
        const int *src = S.nbr + (size_t)(cbegin - S.chunk_begin) * CH;
#pragma unroll
        for (int k = 0; k < 6; ++k)
#pragma unroll
            for (int m = 0; m < RPL; ++m) s_nbr[k * CH + lane + m * LANES] = src[(size_t)k * S.npad + lane + m * LANES];
    }
    unsigned int target = grid_sync_start(bar);  // the counter is zeroed before every launch
    __syncthreads();           // the scalar copies in sst are complete
    // phase times of block 0 (thread 0), kept in shared memory
    __shared__ unsigned long long s_tp[6];
    const bool timing = prof != nullptr && blockIdx.x == 0 && threadIdx.x == 0;
    if (timing) {
        for (int k = 0; k < 5; ++k) s_tp[k] = 0;
        s_tp[5] = global_ns();
    }
    auto mark = [&](int k) {
        if (timing) {
            const unsigned long long t = global_ns();
            s_tp[k] += t - s_tp[5];
            s_tp[5] = t;
        }
    };
    int it = 0;
    bool ok = true;
    for (; it < max_iters; ++it) {
        // K1: p = r + beta (p - w v); y = D^-1 p
        for (int c = cbegin; c < A.total_chunks; c += gstride) {
            const int si = sys_of_chunk(A, c);
            if (!state_active(sst[si])) continue;
            const KSys &S = A.sys[si];
            const int r0 = (c - S.chunk_begin) * CH + lane;
            const double beta = sst[si].beta, w = sst[si].w;
#pragma unroll 4
            for (int m = 0; m < RPL; ++m) {
                const int row = r0 + m * LANES;
                const double p = __fma_rn(beta, __fma_rn(-w, S.v[row], S.p[row]), S.r[row]);
                S.p[row] = p;
                S.y[row] = S.invdiag[row] * p;
            }
        }
        if (!(ok = grid_sync(bar, target, &s_ok))) break;
        mark(0);
        // K2: v = A y, <r0, v>
        for (int c = cbegin; c < A.total_chunks; c += gstride) {
            const int si = sys_of_chunk(A, c);
            if (!state_active(sst[si])) continue;
            const KSys &S = A.sys[si];
            const int lc = c - S.chunk_begin;
            const int r0 = lc * CH + lane;
            double a = 0.0;
            if (kNbrSmem && c == cbegin) {
                // the resident copy: s_nbr_all[(gi * 6 + k) * CH + lane + m * LANES] for slot k, written
                // from threadIdx.x = gi * LANES + lane so the offset stays one register
#pragma unroll kSpmvUnroll
                for (int m = 0; m < RPL; ++m) {
                    const int row = r0 + m * LANES;
                    const double v = spmv_row_nb(S, row, S.y, s_nbr_all + threadIdx.x + (gi * (6 * RPL - 1) + m) * LANES, CH);
                    S.v[row] = v;
                    if (row < S.n) a = __fma_rn(S.r0[row], v, a);
                }
            } else {
#pragma unroll kSpmvUnroll
                for (int m = 0; m < RPL; ++m) {
                    const int row = r0 + m * LANES;
                    const double v = spmv_row(S, row, S.y);
                    S.v[row] = v;
                    if (row < S.n) a = __fma_rn(S.r0[row], v, a);
                }
            }
            const double t = lanes_tree_sum(a, lane, sm[gi], gsync);
            if (lane == 0) S.part[4 * (size_t)S.nchunks + lc] = t;
        }
        if (!(ok = grid_sync(bar, target, &s_ok))) break;
        for (int q = gi; q < A.nsys; q += LOOP_GROUPS) {
            if (!state_active(sst[q])) continue;
            const KSys &S = A.sys[q];
            const double d = lanes_final_sum(S.part + 4 * (size_t)S.nchunks, S.nchunks, 1, lane, sm[gi], gsync);
            if (lane == 0) sst[q].alpha = sst[q].rho / d;
        }
        __syncthreads();
        mark(1);
        // K3: s = r - alpha v; z = D^-1 s
        for (int c = cbegin; c < A.total_chunks; c += gstride) {
            const int si = sys_of_chunk(A, c);
            if (!state_active(sst[si])) continue;
            const KSys &S = A.sys[si];
            const int r0 = (c - S.chunk_begin) * CH + lane;
            const double alpha = sst[si].alpha;
#pragma unroll 4
            for (int m = 0; m < RPL; ++m) {
                const int row = r0 + m * LANES;
                const double sv = __fma_rn(-alpha, S.v[row], S.r[row]);
                S.s[row] = sv;
                S.z[row] = S.invdiag[row] * sv;
            }
        }
        if (!(ok = grid_sync(bar, target, &s_ok))) break;
        mark(2);
        // K4: t = A z, <t, t>, <t, s>
        for (int c = cbegin; c < A.total_chunks; c += gstride) {
            const int si = sys_of_chunk(A, c);
            if (!state_active(sst[si])) continue;
            const KSys &S = A.sys[si];
            const int lc = c - S.chunk_begin;
            const int r0 = lc * CH + lane;
            double att = 0.0, ats = 0.0;
            if (kNbrSmem && c == cbegin) {
#pragma unroll kSpmvUnroll
                for (int m = 0; m < RPL; ++m) {
                    const int row = r0 + m * LANES;
                    const double t = spmv_row_nb(S, row, S.z, s_nbr_all + threadIdx.x + (gi * (6 * RPL - 1) + m) * LANES, CH);
                    S.t[row] = t;
                    if (row < S.n) {
                        att = __fma_rn(t, t, att);
                        ats = __fma_rn(t, S.s[row], ats);
                    }
                }
            } else {
#pragma unroll kSpmvUnroll
                for (int m = 0; m < RPL; ++m) {
                    const int row = r0 + m * LANES;
                    const double t = spmv_row(S, row, S.z);
                    S.t[row] = t;
                    if (row < S.n) {
                        att = __fma_rn(t, t, att);
                        ats = __fma_rn(t, S.s[row], ats);
                    }
                }
            }
            double tt, ts;
            lanes_tree_sum2(att, ats, lane, sm[gi], tt, ts, gsync);
            if (lane == 0) reinterpret_cast<double2 *>(S.part)[lc] = make_double2(tt, ts);
        }
        if (!(ok = grid_sync(bar, target, &s_ok))) break;
        for (int q = gi; q < A.nsys; q += LOOP_GROUPS) {
            if (!state_active(sst[q])) continue;
            const KSys &S = A.sys[q];
            double ftt, fts;
            lanes_final_sum2(S.part, S.nchunks, lane, sm[gi], ftt, fts, gsync);
            if (lane == 0) sst[q].w = (ftt > 0.0) ? fts / ftt : 0.0;
        }
        __syncthreads();
        mark(3);
        // K5: x += alpha y + w z; r = s - w t; <r0, r>, <r, r>
        for (int c = cbegin; c < A.total_chunks; c += gstride) {
            const int si = sys_of_chunk(A, c);
            if (!state_active(sst[si])) continue;
            const KSys &S = A.sys[si];
            const int lc = c - S.chunk_begin;
            const int r0 = lc * CH + lane;
            const double alpha = sst[si].alpha, w = sst[si].w;
            double a0r = 0.0, arr = 0.0;
#pragma unroll 4
            for (int m = 0; m < RPL; ++m) {
                const int row = r0 + m * LANES;
                // rows >= n of x are padding; they receive values computed from zeros
                S.x[row] = __fma_rn(w, S.z[row], __fma_rn(alpha, S.y[row], S.x[row]));
                const double r = __fma_rn(-w, S.t[row], S.s[row]);
                S.r[row] = r;
                if (row < S.n) {
                    a0r = __fma_rn(S.r0[row], r, a0r);
                    arr = __fma_rn(r, r, arr);
                }
            }
            double t0r, trr;
            lanes_tree_sum2(a0r, arr, lane, sm[gi], t0r, trr, gsync);
            if (lane == 0) reinterpret_cast<double2 *>(S.part + 2 * (size_t)S.nchunks)[lc] = make_double2(t0r, trr);
        }
        if (!(ok = grid_sync(bar, target, &s_ok))) break;
        for (int q = gi; q < A.nsys; q += LOOP_GROUPS) {
            if (!state_active(sst[q])) continue;
            const KSys &S = A.sys[q];
            double f0r, frr;
            lanes_final_sum2(S.part + 2 * (size_t)S.nchunks, S.nchunks, lane, sm[gi], f0r, frr, gsync);
            if (lane == 0) {
                KState *st = &sst[q];
                st->rr = frr;
                st->iter += 1;
                st->work += 1;
                if (!(frr > st->tol2 && st->iter < st->maxit)) {
                    finish_loop(st);
                } else {
                    const double eps2 = DBL_EPSILON * DBL_EPSILON;
                    if (fabs(f0r) < eps2 * st->r0_sqnorm) {
                        st->paused = 1;  // the host recomputes r = b - A x and r0
                    } else {
                        st->beta = (f0r / st->rho) * (st->alpha / st->w);
                        st->rho = f0r;
                    }
                }
            }
        }
        __syncthreads();
        mark(4);
        bool any_active = false, any_paused = false;
        if constexpr (CAP <= KMAX) {
            for (int q = 0; q < A.nsys; ++q) {
                any_active = any_active || state_active(sst[q]);
                any_paused = any_paused || (sst[q].paused != 0 && sst[q].done == 0);
            }
        } else {  // the lanes of each warp split the systems
            for (int q = threadIdx.x & 31; q < A.nsys; q += 32) {
                any_active = any_active || state_active(sst[q]);
                any_paused = any_paused || (sst[q].paused != 0 && sst[q].done == 0);
            }
            any_active = __any_sync(0xffffffffu, any_active);
            any_paused = __any_sync(0xffffffffu, any_paused);
        }
        if (!any_active || any_paused) {
            ++it;
            break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < A.nsys) {
        KState k = sst[threadIdx.x];
        k.counter = 0;
        *A.sys[threadIdx.x].st = k;
    }
    if (timing) {
        for (int k = 0; k < 5; ++k) prof->ns[k] += s_tp[k];
        prof->iters += it;
        prof->ok = ok ? 1 : 0;
    }
}

// restart of paused systems: r = b - A x, r0 = r, rho = |r0|^2
template <int CAP>
__global__ void __launch_bounds__(LANES) k_kr_restart(const __grid_constant__ KSetArgT<CAP> A) {
    __shared__ double sm[LANES];
    __shared__ int sh[2];
    NS3D_CHUNK_LOOP
        if (!(__ldcg(&S.st->paused) != 0 && __ldcg(&S.st->done) == 0)) continue;
        const Row4 ax = spmv4(S, r0, S.x);
        const Row4 b = ld4(S.b + r0);
        Row4 r;
        double arr = 0.0;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            r.v[m] = b.v[m] - ax.v[m];
            if (r0 + m * LANES < S.n) arr = __fma_rn(r.v[m], r.v[m], arr);
        }
        st4(S.r + r0, r);
        st4(S.r0 + r0, r);
        const double trr = block_tree_sum(arr, sm);
        if (threadIdx.x == 0) S.part[2 * (size_t)lc] = trr;
        if (arrive_last(S.st, (unsigned)S.nchunks, sh)) {
            const double rr = final_partials_sum(S.part, S.nchunks, 2, sm);
            if (threadIdx.x == 0) {
                KState *st = S.st;
                st->counter = 0;
                st->r0_sqnorm = rr;
                if (st->restarts++ == 0) st->iter = 0;
                st->beta = (rr / st->rho) * (st->alpha / st->w);
                st->rho = rr;
                st->paused = 0;
            }
        }
    }
}

#undef NS3D_CHUNK_LOOP

// y = A x for one system (tests and the residual checks of the drivers)
__global__ void __launch_bounds__(LANES) k_spmv(SysView A, const double *__restrict__ x, double *__restrict__ y) {
    KSys S;
    S.n = A.n;
    S.npad = A.npad;
    S.coef = A.coef;
    S.nbr = A.nbr;
    for (int c = blockIdx.x; c < A.nchunks; c += gridDim.x) {
        const int r0 = c * CH + threadIdx.x;
        st4(y + r0, spmv4(S, r0, x));
    }
}

// Test hook of the bounded grid barrier (ns3d_debug_barrier_timeout): while
// set, every loop-kernel launch's barrier waits for g_bar_bias arrivals that
// never come, for at most g_bar_limit_ns, then the launch ends with its
// error flag set.
static std::atomic<unsigned int> g_bar_bias{0};
static std::atomic<unsigned long long> g_bar_limit_ns{0};

void set_barrier_test(unsigned int bias, unsigned long long limit_ns) {
    g_bar_limit_ns = limit_ns;
    g_bar_bias = bias;
}

cudaError_t reset_grid_bar(GridBar *bar, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(bar, 0, sizeof(GridBar), st);
    const unsigned int bias = g_bar_bias.load();
    if (e != cudaSuccess || bias == 0) return e;
    GridBar h;
    std::memset(&h, 0, sizeof h);
    h.bias = bias;
    h.limit_ns = g_bar_limit_ns.load();
    // pageable source: the copy is staged before the call returns
    return cudaMemcpyAsync(bar, &h, sizeof h, cudaMemcpyHostToDevice, st);
}

static std::atomic<int64_t> g_launches{0};
int64_t launch_count() { return g_launches.load(); }
void count_launches(int64_t n) { g_launches += n; }

static int g_sms = 0;
int device_sm_count() {
    if (g_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 152;
    }
    return g_sms;
}

// one block per chunk up to 32 blocks per SM (the hardware schedules the
// waves); beyond that, blocks walk the chunks grid-stride
static inline int kr_grid(int total_chunks) { return std::max(1, std::min(total_chunks, device_sm_count() * 32)); }

template <int CAP>
void launch_krylov_init(const KSetArgT<CAP> &A, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    count_launches(2);
    k_kr_init<CAP><<<kr_grid(A.total_chunks), LANES, 0, st>>>(A);
    k_kr_init2<CAP><<<kr_grid(A.total_chunks), LANES, 0, st>>>(A);
}

// Blocks of a loop-kernel launch.  Every block must be resident at once
// (cooperative launch).  A solve that runs alone spreads its work units over
// every SM (one block per SM).  While k solves run in the process, a solve
// takes about 1/k of the SMs -- but at least one block per LOOP_GROUPS
// chunks of rows, so that no group holds more than one chunk per phase --
// and the loop kernels of concurrent solves, on their own streams, run side
// by side.
static std::atomic<int> g_active_solves{0};
ActiveSolve::ActiveSolve() { g_active_solves++; }
ActiveSolve::~ActiveSolve() { g_active_solves--; }
int active_solves() { return g_active_solves.load(); }

int loop_grid(int units, int units_per_chunk, int occ) {
    const int slots = device_sm_count() * std::max(occ, 1);
    const int active = std::max(1, g_active_solves.load());
    if (active == 1) return std::max(1, std::min(units, slots));
    // a fair share of the SMs, but never more than one chunk of rows per group
    const int per_block = LOOP_GROUPS * std::max(units_per_chunk, 1);
    const int dense = (units + per_block - 1) / per_block;
    const int fair = std::max(1, slots / active);
    return std::max(1, std::min(std::max(dense, std::min(fair, units)), slots));
}

// A merged set (the systems of many concurrent solves) spreads over its
// share of the SMs: all of them, or 1/share while `share` merged sets run.
template <int CAP>
static int krylov_loop_grid(int total_chunks, int occ, int share) {
    if (CAP > KMAX)
        return std::max(1, std::min(total_chunks, device_sm_count() * std::max(occ, 1) / std::max(share, 1)));
    return loop_grid(total_chunks, 1, occ);
}

template <int CAP>
cudaError_t launch_krylov_loop(const KSetArgT<CAP> &A, GridBar *bar, LoopProf *prof, int max_iters,
                               cudaStream_t st, int share) {
    if (A.total_chunks <= 0 || max_iters <= 0) return cudaSuccess;
    static std::atomic<int> loop_occ{0};
    int occ = loop_occ.load();
    if (occ == 0) {
        cudaError_t e = cudaSuccess;
        if (kNbrSmemBytes > 0)
            e = cudaFuncSetAttribute((const void *)k_kr_loop<CAP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kNbrSmemBytes);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_kr_loop<CAP>, LOOP_THREADS, kNbrSmemBytes);
        if (e != cudaSuccess) return e;
        if (occ <= 0) return cudaErrorLaunchOutOfResources;
        loop_occ = occ;
    }
    const int grid = krylov_loop_grid<CAP>(A.total_chunks, occ, share);
    cudaError_t e = reset_grid_bar(bar, st);
    if (e != cudaSuccess) return e;
    KSetArgT<CAP> a = A;
    void *args[] = {&a, &bar, &prof, &max_iters};
    count_launches(1);
    return cudaLaunchCooperativeKernel((const void *)k_kr_loop<CAP>, grid, LOOP_THREADS, args, kNbrSmemBytes, st);
}

template <int CAP>
void launch_krylov_restart(const KSetArgT<CAP> &A, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    count_launches(1);
    k_kr_restart<CAP><<<kr_grid(A.total_chunks), LANES, 0, st>>>(A);
}

template void launch_krylov_init<KMAX>(const KSetArg &, cudaStream_t);
template void launch_krylov_init<KMAX_MERGED>(const KSetArgMerged &, cudaStream_t);
template cudaError_t launch_krylov_loop<KMAX>(const KSetArg &, GridBar *, LoopProf *, int, cudaStream_t, int);
template cudaError_t launch_krylov_loop<KMAX_MERGED>(const KSetArgMerged &, GridBar *, LoopProf *, int,
                                                     cudaStream_t, int);
template void launch_krylov_restart<KMAX>(const KSetArg &, cudaStream_t);
template void launch_krylov_restart<KMAX_MERGED>(const KSetArgMerged &, cudaStream_t);

void launch_spmv(const SysView &A, const double *x, double *y, cudaStream_t st) {
    if (A.n <= 0) return;
    count_launches(1);
    k_spmv<<<std::max(1, std::min(A.nchunks, device_sm_count() * 6)), LANES, 0, st>>>(A, x, y);
}

}  // namespace ns3d
