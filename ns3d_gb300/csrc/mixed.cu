// mixed.cu -- mixed-precision solves: FP32 BiCGSTAB (FP32 vectors, FP32
// matrix copy, FP32 accumulation in the lanes) wrapped in FP64 defect
// correction.  FP64 stays on the device for the residual r = b - A x, its
// norm, the right-hand-side norm, the Krylov scalars (alpha, beta, omega,
// rho) and the solution update, so the converged solution satisfies the same
// FP64 tolerance test as the plain path (|r|^2 <= tol^2 |b|^2).
//
// One correction round of a set of systems:
//   k_dc_resid   r64 = b - A64 x (FP64), |r64|^2 (and |b|^2 in round 0);
//                last block: convergence test, scale = 1/|r64|, inner target
//   k_m32_init   f = float(r64 * scale); r = r0 = f; d = 0; p = v = 0; |f|^2
//   k_m32_loop   the BiCGSTAB iterations in FP32 on A32 d = f (one
//                persistent cooperative launch per round)
//   k_dc_step    theta minimizing |r64 - theta A64 delta|, delta = double(d) / scale
//   k_dc_update  x += theta delta
// An inner solve stops at its relative target, at the iteration budget, or
// at a breakdown (|rho| tiny, non-finite scalars); the next round restarts
// from the new FP64 residual.  iterations() reports the inner iterations.
#include <atomic>
#include <cfloat>

#include "device.cuh"
#include "kernels.h"
#include "loop.cuh"
#include "mixed.h"

namespace ns3d {

struct RowF4 {  // a thread's RPL rows
    float v[RPL];
};

__device__ __forceinline__ RowF4 ldf4(const float *p) {
    RowF4 r;
#pragma unroll
    for (int m = 0; m < RPL; ++m) r.v[m] = p[m * LANES];
    return r;
}
__device__ __forceinline__ void stf4(float *p, const RowF4 &r) {
#pragma unroll
    for (int m = 0; m < RPL; ++m) p[m * LANES] = r.v[m];
}

// FP32 row product.  A missing entry has a zero coefficient; its gather
// reads the row's own (finite) element, so all seven products are issued
// without branches (FP32 issue is plentiful on GB300).
__device__ __forceinline__ float spmv_f32_row(const MSys &S, int row, const float *__restrict__ x) {
    const size_t np = (size_t)S.npad;
    const int *nb = S.nbr + row;
    const float *cf = S.coef32 + row;
    const int nW = ro(nb + 0 * np), nE = ro(nb + 1 * np), nS = ro(nb + 2 * np), nN = ro(nb + 3 * np),
              nB = ro(nb + 4 * np), nT = ro(nb + 5 * np);
    float acc = ro(cf) * x[row];
    acc = __fmaf_rn(ro(cf + 1 * np), x[nW >= 0 ? nW : row], acc);
    acc = __fmaf_rn(ro(cf + 3 * np), x[nS >= 0 ? nS : row], acc);
    acc = __fmaf_rn(ro(cf + 5 * np), x[nB >= 0 ? nB : row], acc);
    acc = __fmaf_rn(ro(cf + 6 * np), x[nT >= 0 ? nT : row], acc);
    acc = __fmaf_rn(ro(cf + 4 * np), x[nN >= 0 ? nN : row], acc);
    acc = __fmaf_rn(ro(cf + 2 * np), x[nE >= 0 ? nE : row], acc);
    return acc;
}

// spmv_f32_row with the input vector given by a function of the column:
// the loop kernel recomputes y = D^-1 p and z = D^-1 s of neighbouring rows
// instead of waiting for their owners to store them
template <class F>
__device__ __forceinline__ float spmv_f32_fn(const MSys &S, int row, F xf) {
    const size_t np = (size_t)S.npad;
    const int *nb = S.nbr + row;
    const float *cf = S.coef32 + row;
    const int nW = nb[0 * np], nE = nb[1 * np], nS = nb[2 * np], nN = nb[3 * np], nB = nb[4 * np], nT = nb[5 * np];
    float acc = cf[0] * xf(row);
    acc = __fmaf_rn(cf[1 * np], xf(nW >= 0 ? nW : row), acc);
    acc = __fmaf_rn(cf[3 * np], xf(nS >= 0 ? nS : row), acc);
    acc = __fmaf_rn(cf[5 * np], xf(nB >= 0 ? nB : row), acc);
    acc = __fmaf_rn(cf[6 * np], xf(nT >= 0 ? nT : row), acc);
    acc = __fmaf_rn(cf[4 * np], xf(nN >= 0 ? nN : row), acc);
    acc = __fmaf_rn(cf[2 * np], xf(nE >= 0 ? nE : row), acc);
    return acc;
}

__device__ __forceinline__ double spmv_f64_row(const MSys &S, int row, const double *__restrict__ x) {
    const size_t np = (size_t)S.npad;
    const int *nb = S.nbr + row;
    const double *cf = S.coef64 + row;
    return row_ordered(row, nb[0 * np], nb[1 * np], nb[2 * np], nb[3 * np], nb[4 * np], nb[5 * np],
                       [&](double acc, int s, int col) { return __fma_rn(cf[(size_t)s * np], x[col], acc); });
}

// system owning global chunk c (systems in chunk order, first begins at 0;
// the last system whose first chunk is <= c, so a system without rows is
// never chosen)
template <int CAP>
__device__ __forceinline__ int msys_of_chunk(const MSetArgT<CAP> &A, int c) {
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

// Flags change only between kernels (or in the last block of a system, after
// every other block of that system has passed its check), so all threads of a
// block read the same values.  `inner`: the FP32 solve must be running too.
__device__ __forceinline__ bool m_active(const MSys &S, bool inner) {
    bool act = __ldcg(&S.dc->done) == 0;
    if (inner) act = act && __ldcg(&S.st->done) == 0;
    return act;
}

#define NS3D_MCHUNK_LOOP(INNER)                                              \
    for (int c = blockIdx.x; c < A.total_chunks; c += gridDim.x) {           \
        const MSys &S = A.sys[msys_of_chunk(A, c)];                          \
        if (!m_active(S, INNER)) continue;                                    \
        const int lc = c - S.chunk_begin;                                     \
        const int r0 = lc * CH + threadIdx.x;

__device__ __forceinline__ bool m_arrive_last(unsigned int *counter, unsigned int total, int *sh) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int prev = atomicAdd(counter, 1u);
        sh[2] = (prev == total - 1) ? 1 : 0;
    }
    __syncthreads();
    bool last = sh[2] != 0;
    if (last) __threadfence();
    return last;
}

__device__ __forceinline__ bool finite(double x) { return isfinite(x); }

// ---- FP64 residual and outer control -----------------------------------------
template <int CAP>
__global__ void __launch_bounds__(LANES) k_dc_resid(const __grid_constant__ MSetArgT<CAP> A, int first) {
    __shared__ double sm[LANES];
    __shared__ int sh[4];
    NS3D_MCHUNK_LOOP(false)
        double arr = 0.0, abb = 0.0;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            const int row = r0 + m * LANES;
            const double b = S.b64[row];
            const double r = b - spmv_f64_row(S, row, S.x64);
            S.r64[row] = r;
            if (row < S.n) {
                arr = __fma_rn(r, r, arr);
                abb = __fma_rn(b, b, abb);
            }
        }
        double trr, tbb;
        block_tree_sum2(arr, abb, sm, trr, tbb);
        if (threadIdx.x == 0) {
            S.part[2 * (size_t)lc + 0] = trr;
            S.part[2 * (size_t)lc + 1] = tbb;
        }
        if (m_arrive_last(&S.dc->counter, (unsigned)S.nchunks, sh)) {
            double rr, bb;
            final_partials_sum2(S.part, S.nchunks, sm, rr, bb);
            if (threadIdx.x == 0) {
                DCState *dc = S.dc;
                KState *st = S.st;
                dc->counter = 0;
                if (!first) dc->total_iter += st->iter;
                if (first) {
                    dc->bb = bb;
                    dc->tol2 = dc->tol * dc->tol * bb;
                }
                dc->rr = rr;
                if (first && bb == 0.0) {
                    dc->zero_rhs = 1;
                    dc->done = 1;
                    dc->total_iter = dc->maxit;
                    dc->error = dc->tol;
                    dc->info = 0;
                } else if (!finite(rr) || (!first && st->info == 1)) {
                    dc->done = 1;
                    dc->error = sqrt(rr / dc->bb);
                    dc->info = 1;  // NumericalIssue
                } else if (!(rr > dc->tol2 && dc->total_iter < dc->maxit)) {
                    dc->done = 1;
                    dc->error = sqrt(rr / dc->bb);
                    dc->info = (dc->error <= dc->tol) ? 0 : 2;
                } else {
                    dc->scale = 1.0 / sqrt(rr);
                    // reduce the normalized residual to the inner target, but
                    // not (much) further than the outer test needs
                    const double need = 0.5 * sqrt(dc->tol2 / rr);
                    dc->tin = need > dc->tin_min ? need : dc->tin_min;
                    st->done = 0;
                    st->iter = 0;
                    st->info = 0;
                    st->maxit = min(dc->inner_cap, dc->maxit - dc->total_iter);
                }
            }
        }
    }
}

// x64 = 0 for systems with a zero right-hand side (first round)
template <int CAP>
__global__ void k_dc_zero(const __grid_constant__ MSetArgT<CAP> A) {
    for (int c = blockIdx.x; c < A.total_chunks; c += gridDim.x) {
        const MSys &S = A.sys[msys_of_chunk(A, c)];
        if (!__ldcg(&S.dc->zero_rhs)) continue;
        const int r0 = (c - S.chunk_begin) * CH + threadIdx.x;
#pragma unroll
        for (int m = 0; m < RPL; ++m) S.x64[r0 + m * LANES] = 0.0;
    }
}

// ---- FP32 inner solve -------------------------------------------------------
template <int CAP>
__global__ void __launch_bounds__(LANES) k_m32_init(const __grid_constant__ MSetArgT<CAP> A) {
    __shared__ double sm[LANES];
    __shared__ int sh[4];
    NS3D_MCHUNK_LOOP(true)
        const double scale = __ldcg(&S.dc->scale);
        float acc = 0.0f;
        RowF4 f;
        RowF4 zero;
#pragma unroll
        for (int m = 0; m < RPL; ++m) zero.v[m] = 0.0f;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            const int row = r0 + m * LANES;
            f.v[m] = (float)(S.r64[row] * scale);
            if (row < S.n) acc = __fmaf_rn(f.v[m], f.v[m], acc);
        }
        stf4(S.r + r0, f);
        stf4(S.r0 + r0, f);
        stf4(S.x + r0, zero);
        stf4(S.p + r0, zero);
        stf4(S.v + r0, zero);
        const double t = block_tree_sum((double)acc, sm);
        if (threadIdx.x == 0) S.part[2 * (size_t)lc] = t;
        if (m_arrive_last(&S.st->counter, (unsigned)S.nchunks, sh)) {
            const double bb = final_partials_sum(S.part, S.nchunks, 2, sm);
            if (threadIdx.x == 0) {
                KState *st = S.st;
                st->counter = 0;
                st->rhs_sqnorm = bb;
                st->r0_sqnorm = bb;
                st->rr = bb;
                st->tol = __ldcg(&S.dc->tin);
                st->tol2 = st->tol * st->tol * bb;
                st->rho = 1.0;
                st->alpha = 1.0;
                st->w = 1.0;
                if (!(bb > st->tol2 && 0 < st->maxit)) {
                    st->done = 1;
                } else {
                    st->beta = bb;  // (rho/1) * (1/1) with rho = <r0, r> = |r0|^2
                    st->rho = bb;
                }
            }
        }
    }
}

// ---- aggregation multilevel preconditioner (MIXED_MG) -------------------------
struct MGView {
    int n, npad;
    const int *nbr;
    const float *coef, *invdiag;
    float *x, *b, *t;
};

// level k of the hierarchy of S (level 0: the FP32 system, solution x0 of
// right-hand side b0, scratch S.t)
__device__ __forceinline__ MGView mg_level(const MSys &S, int k, const float *b0, float *x0) {
    MGView L;
    if (k == 0) {
        L.n = S.n;
        L.npad = S.npad;
        L.nbr = S.nbr;
        L.coef = S.coef32;
        L.invdiag = S.invdiag32;
        L.x = x0;
        L.b = const_cast<float *>(b0);
        L.t = S.t;
    } else {
        const MGLevel &G = S.mg.lev[k];
        L.n = G.n;
        L.npad = G.npad;
        L.nbr = G.nbr;
        L.coef = G.coef;
        L.invdiag = G.invdiag;
        L.x = G.x;
        L.b = G.b;
        L.t = G.t;
    }
    return L;
}

// row of A x at one level (slot d+1 couples through neighbour d; a missing
// neighbour has a zero coefficient and gathers the row itself)
__device__ __forceinline__ float mg_spmv(const MGView &L, int row, const float *x) {
    const size_t np = (size_t)L.npad;
    const int *nb = L.nbr + row;
    const float *cf = L.coef + row;
    float acc = ro(cf) * x[row];
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        const int c = ro(nb + d * np);
        acc = __fmaf_rn(ro(cf + (d + 1) * np), x[c >= 0 ? c : row], acc);
    }
    return acc;
}

// Jacobi sweeps on the coarsest level by the calling block: x = w D^-1 b,
// then `sweeps` times t = b - A x, x += w D^-1 t
__device__ void mg_coarsest(const MGView &L, float w, int sweeps) {
    for (int r = threadIdx.x; r < L.n; r += blockDim.x) L.x[r] = w * L.invdiag[r] * L.b[r];
    __syncthreads();
    for (int it = 0; it < sweeps; ++it) {
        for (int r = threadIdx.x; r < L.n; r += blockDim.x) L.t[r] = L.b[r] - mg_spmv(L, r, L.x);
        __syncthreads();
        for (int r = threadIdx.x; r < L.n; r += blockDim.x) L.x[r] += w * L.invdiag[r] * L.t[r];
        __syncthreads();
    }
}

// x0 = M^-1 b0: one V-cycle -- a damped Jacobi sweep from zero, the residual
// restricted to the next level (sum over the block), ... , Jacobi sweeps on
// the coarsest level in block 0, then on the way up the correction of the
// coarser level added and one damped Jacobi sweep.  Every thread of the grid
// calls it (grid barriers between the passes); false when a barrier failed.
// The fine level's Jacobi start x0 = w D^-1 b0 is already written by the
// loop phase that computed b0 (p or s), so the V-cycle starts with the
// fine residual.  (Fusing the Jacobi start, residual and restriction into
// one pass per coarse row -- one grid barrier per level instead of three,
// neighbours' starts recomputed -- gave the same values but measured 3-8%
// slower, on the coarse levels as on the fine one.)
__device__ bool mg_apply(const MSys &S, const float *b0, float *x0, GridBar *bar, unsigned int &target,
                         int *s_ok) {
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gth = gridDim.x * blockDim.x;
    const int K = S.mg.nlev;
    const float w = S.mg.omega;
    for (int k = 0; k < K; ++k) {
        const MGView L = mg_level(S, k, b0, x0);
        const MGLevel &C = S.mg.lev[k + 1];
        if (k > 0) {
            for (int r = gtid; r < L.n; r += gth) L.x[r] = w * L.invdiag[r] * L.b[r];
            if (!grid_sync(bar, target, s_ok)) return false;
        }
        for (int r = gtid; r < L.n; r += gth) L.t[r] = L.b[r] - mg_spmv(L, r, L.x);
        if (!grid_sync(bar, target, s_ok)) return false;
        for (int I = gtid; I < C.n; I += gth) {
            float acc = 0.0f;
            for (int q = C.mstart[I]; q < C.mstart[I + 1]; ++q) acc += L.t[C.members[q]];
            C.b[I] = acc;
        }
        if (!grid_sync(bar, target, s_ok)) return false;
    }
    if (blockIdx.x == 0) mg_coarsest(mg_level(S, K, b0, x0), w, S.mg.sweeps);
    if (!grid_sync(bar, target, s_ok)) return false;
    for (int k = K - 1; k >= 0; --k) {
        const MGView L = mg_level(S, k, b0, x0);
        const MGLevel &C = S.mg.lev[k + 1];
        for (int r = gtid; r < L.n; r += gth) L.x[r] += C.x[C.agg[r]];
        if (!grid_sync(bar, target, s_ok)) return false;
        for (int r = gtid; r < L.n; r += gth) L.t[r] = L.b[r] - mg_spmv(L, r, L.x);
        if (!grid_sync(bar, target, s_ok)) return false;
        for (int r = gtid; r < L.n; r += gth) L.x[r] += w * L.invdiag[r] * L.t[r];
        if (!grid_sync(bar, target, s_ok)) return false;
    }
    return true;
}

// the inner solve of a system runs (its outer solve is not done either)
__device__ __forceinline__ bool inner_active(const KState &k, int dc_done) { return !dc_done && !k.done; }

// Calls op(q, r) for the rows r < rows(q) of every system q with part(q):
// the systems' row ranges, concatenated in system order, are cut
// round-robin over the grid's threads (one system alone: thread t takes rows
// t, t + threads, ...).
template <int CAP, class Part, class Rows, class Op>
__device__ __forceinline__ void mg_rows(const MSetArgT<CAP> &A, Part part, Rows rows, Op op) {
    const long gtid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long gth = (long)gridDim.x * blockDim.x;
    long base = 0;
    for (int q = 0; q < A.nsys; ++q) {
        if (!part(q)) continue;
        const int n = rows(q);
        long first = gtid - base;  // smallest r >= 0 with base + r = gtid (mod gth)
        if (first < 0) first += ((-first + gth - 1) / gth) * gth;
        for (long r = first; r < n; r += gth) op(q, (int)r);
        base += n;
    }
}

// mg_apply for every system of a merged set that has a hierarchy and an
// active inner solve (which = 0: y = M^-1 p, 1: z = M^-1 s).  Pass k of the
// way down (or up) runs for the systems with more than k coarse levels, the
// coarsest sweeps of system j in block j mod gridDim.x, so every system
// takes exactly the steps and the arithmetic of mg_apply, with one set of
// grid barriers for all of them.
template <int CAP>
__device__ bool mg_apply_set(const MSetArgT<CAP> &A, const KState *sst, const int *sdc, int which, GridBar *bar,
                             unsigned int &target, int *s_ok) {
    auto on = [&](int q) { return A.sys[q].mg.nlev > 0 && inner_active(sst[q], sdc[q]); };
    auto lvl = [&](int q, int k) {
        const MSys &S = A.sys[q];
        return which == 0 ? mg_level(S, k, S.p, S.y) : mg_level(S, k, S.s, S.z);
    };
    int kmax = 0;
    for (int q = 0; q < A.nsys; ++q)
        if (on(q)) kmax = max(kmax, A.sys[q].mg.nlev);
    for (int k = 0; k < kmax; ++k) {
        auto part = [&](int q) { return on(q) && k < A.sys[q].mg.nlev; };
        if (k > 0) {  // the fine level's start is written by the loop phase
            mg_rows(A, part, [&](int q) { return A.sys[q].mg.lev[k].n; },
                    [&](int q, int r) {
                        const MGView L = lvl(q, k);
                        const float w = A.sys[q].mg.omega;
                        L.x[r] = w * L.invdiag[r] * L.b[r];
                    });
            if (!grid_sync(bar, target, s_ok)) return false;
        }
        mg_rows(A, part, [&](int q) { return k == 0 ? A.sys[q].n : A.sys[q].mg.lev[k].n; },
                [&](int q, int r) {
                    const MGView L = lvl(q, k);
                    L.t[r] = L.b[r] - mg_spmv(L, r, L.x);
                });
        if (!grid_sync(bar, target, s_ok)) return false;
        mg_rows(A, part, [&](int q) { return A.sys[q].mg.lev[k + 1].n; },
                [&](int q, int I) {
                    const MGView L = lvl(q, k);
                    const MGLevel &C = A.sys[q].mg.lev[k + 1];
                    float acc = 0.0f;
                    for (int m = C.mstart[I]; m < C.mstart[I + 1]; ++m) acc += L.t[C.members[m]];
                    C.b[I] = acc;
                });
        if (!grid_sync(bar, target, s_ok)) return false;
    }
    {
        int j = 0;  // index of the system among those preconditioned
        for (int q = 0; q < A.nsys; ++q) {
            if (!on(q)) continue;
            if (j++ % gridDim.x != blockIdx.x) continue;
            mg_coarsest(lvl(q, A.sys[q].mg.nlev), A.sys[q].mg.omega, A.sys[q].mg.sweeps);
        }
        if (!grid_sync(bar, target, s_ok)) return false;
    }
    for (int k = kmax - 1; k >= 0; --k) {
        auto part = [&](int q) { return on(q) && k < A.sys[q].mg.nlev; };
        auto rows = [&](int q) { return k == 0 ? A.sys[q].n : A.sys[q].mg.lev[k].n; };
        mg_rows(A, part, rows, [&](int q, int r) {
            const MGView L = lvl(q, k);
            const MGLevel &C = A.sys[q].mg.lev[k + 1];
            L.x[r] += C.x[C.agg[r]];
        });
        if (!grid_sync(bar, target, s_ok)) return false;
        mg_rows(A, part, rows, [&](int q, int r) {
            const MGView L = lvl(q, k);
            L.t[r] = L.b[r] - mg_spmv(L, r, L.x);
        });
        if (!grid_sync(bar, target, s_ok)) return false;
        mg_rows(A, part, rows, [&](int q, int r) {
            const MGView L = lvl(q, k);
            const float w = A.sys[q].mg.omega;
            L.x[r] += w * L.invdiag[r] * L.t[r];
        });
        if (!grid_sync(bar, target, s_ok)) return false;
    }
    return true;
}

// y = M^-1 p (which = 0) or z = M^-1 s (1) for the multilevel systems of a set
template <int CAP>
__device__ __forceinline__ bool mg_precondition(const MSetArgT<CAP> &A, const KState *sst, const int *sdc,
                                                int which, GridBar *bar, unsigned int &target, int *s_ok) {
    if constexpr (CAP <= KMAX) {  // one solver instance's set: a single system
        const MSys &S = A.sys[0];
        return which == 0 ? mg_apply(S, S.p, S.y, bar, target, s_ok) : mg_apply(S, S.s, S.z, bar, target, s_ok);
    } else {
        return mg_apply_set(A, sst, sdc, which, bar, target, s_ok);
    }
}

// Galerkin operator of a coarse level: per row, the sum of its block's
// diagonal and internal couplings, and per direction the couplings that
// leave the block (in the members' order).
// A block that holds a whole isolated pore cluster (no path to the inlet or
// outlet: its rows sum to zero, the block is singular) gets a coarse
// diagonal that cancels to a rounding residue; 1/residue would blow the
// coarse correction up.  Such a diagonal (below kSingular of its members'
// diagonals in magnitude) gets no coarse correction: inverse diagonal 0.
constexpr float kSingular = 1e-4f;

__global__ void k_mg_galerkin(int npad_f, const int *__restrict__ nbr_f, const float *__restrict__ coef_f,
                              MGLevel C) {
    for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < C.n; I += gridDim.x * blockDim.x) {
        float d = 0.0f, dabs = 0.0f, off[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        for (int q = C.mstart[I]; q < C.mstart[I + 1]; ++q) {
            const int m = C.members[q];
            d += coef_f[m];
            dabs += fabsf(coef_f[m]);
#pragma unroll
            for (int dir = 0; dir < 6; ++dir) {
                const int col = nbr_f[(size_t)dir * npad_f + m];
                if (col < 0) continue;
                const float a = coef_f[(size_t)(dir + 1) * npad_f + m];
                if (C.agg[col] == I) d += a;
                else off[dir] += a;
            }
        }
        C.coef[I] = d;
#pragma unroll
        for (int dir = 0; dir < 6; ++dir) C.coef[(size_t)(dir + 1) * C.npad + I] = off[dir];
        C.invdiag[I] = fabsf(d) > kSingular * dabs ? 1.0f / d : 0.0f;
    }
}

// ---- the FP32 inner iterations as one persistent cooperative kernel ----------
// Same block shape, interleaving, partial regions and grid barrier as the
// FP64 loop kernel (krylov.cu), with FP32 vectors and FP32 sums inside a
// work unit (FP32 pipe), FP64 sums of the unit partials and FP64 scalars.
// FUSED: three phases and grid barriers per iteration instead of five: the
// SpMV phases recompute y = D^-1 p and z = D^-1 s at neighbouring rows from
// r, p, v (cheap in FP32) instead of waiting for a barrier after their owners
// store them; p and v alternate between two buffers so that a phase never
// overwrites what a neighbour still reads.  Otherwise the five phases of the
// FP64 loop.  The FP32
// results follow no fixed-order contract, so the work unit is a quarter
// chunk (MUNIT = 256 rows, MRPL = 2 per lane): a group finishes a unit in one
// round of loads, and a small system spreads over 4x more groups.  Every
// block keeps a copy of the inner state; the kernel ends when every inner
// solve of the round is done or after `max_iters` iterations.

template <bool FUSED, int CAP>
__global__ void __launch_bounds__(LOOP_THREADS, LOOP_MIN_BLOCKS)
    k_m32_loop(const __grid_constant__ MSetArgT<CAP> A, GridBar *bar, int max_iters) {
    static_assert(CAP <= LOOP_THREADS, "one thread copies each system's state");
    __shared__ KState sst[CAP];
    __shared__ int sdc[CAP];
    __shared__ double sm[LOOP_GROUPS][LANES];
    __shared__ int s_ok;
    const int gi = threadIdx.x / LANES, lane = threadIdx.x % LANES;
    const GroupSync gsync{gi + 1};
    const int gstride = gridDim.x * LOOP_GROUPS;
    const int cbegin = blockIdx.x + gridDim.x * gi;
    const int total_units = A.total_chunks * MSUB;
    if (threadIdx.x < A.nsys) {
        sst[threadIdx.x] = *A.sys[threadIdx.x].st;
        sdc[threadIdx.x] = A.sys[threadIdx.x].dc->done;
    }
    unsigned int target = grid_sync_start(bar);
    __syncthreads();
    int it = 0;
    for (; it < max_iters; ++it) {
        if constexpr (FUSED) {
            const bool odd = (it & 1) != 0;
            // A: p' = r + beta (p - w v), y = D^-1 p' (stored for the own rows,
            //    recomputed for neighbours); v' = A y, <r0, v'>.  p and v are read
            //    from one buffer and written to the other.
            for (int u = cbegin; u < total_units; u += gstride) {
                const int si = msys_of_chunk(A, u / MSUB);
                if (!inner_active(sst[si], sdc[si])) continue;
                const MSys &S = A.sys[si];
                const int lc = u - S.chunk_begin * MSUB;
                const int r0 = lc * MUNIT + lane;
                const float beta = (float)sst[si].beta, w = (float)sst[si].w;
                const float *pc = odd ? S.p2 : S.p, *vc = odd ? S.v2 : S.v;
                float *pn = odd ? S.p : S.p2, *vn = odd ? S.v : S.v2;
                auto yf = [&](int k) { return S.invdiag32[k] * __fmaf_rn(beta, __fmaf_rn(-w, vc[k], pc[k]), S.r[k]); };
                float a = 0.0f;
    #pragma unroll
                for (int m = 0; m < MRPL; ++m) {
                    const int row = r0 + m * LANES;
                    const float p = __fmaf_rn(beta, __fmaf_rn(-w, vc[row], pc[row]), S.r[row]);
                    pn[row] = p;
                    S.y[row] = S.invdiag32[row] * p;
                    const float v = spmv_f32_fn(S, row, yf);
                    vn[row] = v;
                    if (row < S.n) a = __fmaf_rn(S.r0[row], v, a);
                }
                const float t = lanes_tree_sum<float>(a, lane, reinterpret_cast<float *>(sm[gi]), gsync);
                if (lane == 0) S.part[4 * (size_t)S.nchunks * MSUB + lc] = (double)t;
            }
            if (!grid_sync(bar, target, &s_ok)) break;
            for (int q = gi; q < A.nsys; q += LOOP_GROUPS) {
                if (!inner_active(sst[q], sdc[q])) continue;
                const MSys &S = A.sys[q];
                const double d = lanes_final_sum(S.part + 4 * (size_t)S.nchunks * MSUB, S.nchunks * MSUB, 1, lane, sm[gi], gsync);
                if (lane == 0) sst[q].alpha = sst[q].rho / d;
            }
            __syncthreads();
            // B: s = r - alpha v', z = D^-1 s (stored for the own rows, recomputed
            //    for neighbours); t = A z, <t, t>, <t, s>
            for (int u = cbegin; u < total_units; u += gstride) {
                const int si = msys_of_chunk(A, u / MSUB);
                if (!inner_active(sst[si], sdc[si])) continue;
                const MSys &S = A.sys[si];
                const int lc = u - S.chunk_begin * MSUB;
                const int r0 = lc * MUNIT + lane;
                const float alpha = (float)sst[si].alpha;
                const float *vn = odd ? S.v : S.v2;
                auto zf = [&](int k) { return S.invdiag32[k] * __fmaf_rn(-alpha, vn[k], S.r[k]); };
                float att = 0.0f, ats = 0.0f;
    #pragma unroll
                for (int m = 0; m < MRPL; ++m) {
                    const int row = r0 + m * LANES;
                    const float sv = __fmaf_rn(-alpha, vn[row], S.r[row]);
                    S.s[row] = sv;
                    S.z[row] = S.invdiag32[row] * sv;
                    const float t = spmv_f32_fn(S, row, zf);
                    S.t[row] = t;
                    if (row < S.n) {
                        att = __fmaf_rn(t, t, att);
                        ats = __fmaf_rn(t, sv, ats);
                    }
                }
                float tt, ts;
                lanes_tree_sum2<float>(att, ats, lane, reinterpret_cast<float *>(sm[gi]), tt, ts, gsync);
                if (lane == 0) reinterpret_cast<double2 *>(S.part)[lc] = make_double2(tt, ts);
            }
            if (!grid_sync(bar, target, &s_ok)) break;
            for (int q = gi; q < A.nsys; q += LOOP_GROUPS) {
                if (!inner_active(sst[q], sdc[q])) continue;
                const MSys &S = A.sys[q];
                double ftt, fts;
                lanes_final_sum2(S.part, S.nchunks * MSUB, lane, sm[gi], ftt, fts, gsync);
                if (lane == 0) sst[q].w = (ftt > 0.0) ? fts / ftt : 0.0;
            }
            __syncthreads();
            // C: x += alpha y + w z; r = s - w t; <r0, r>, <r, r>
            for (int u = cbegin; u < total_units; u += gstride) {
                const int si = msys_of_chunk(A, u / MSUB);
                if (!inner_active(sst[si], sdc[si])) continue;
                const MSys &S = A.sys[si];
                const int lc = u - S.chunk_begin * MSUB;
                const int r0 = lc * MUNIT + lane;
                const float alpha = (float)sst[si].alpha, w = (float)sst[si].w;
                float a0r = 0.0f, arr = 0.0f;
    #pragma unroll
                for (int m = 0; m < MRPL; ++m) {
                    const int row = r0 + m * LANES;
                    S.x[row] = __fmaf_rn(w, S.z[row], __fmaf_rn(alpha, S.y[row], S.x[row]));
                    const float r = __fmaf_rn(-w, S.t[row], S.s[row]);
                    S.r[row] = r;
                    if (row < S.n) {
                        a0r = __fmaf_rn(S.r0[row], r, a0r);
                        arr = __fmaf_rn(r, r, arr);
                    }
                }
                float t0r, trr;
                lanes_tree_sum2<float>(a0r, arr, lane, reinterpret_cast<float *>(sm[gi]), t0r, trr, gsync);
                if (lane == 0)
                    reinterpret_cast<double2 *>(S.part + 2 * (size_t)S.nchunks * MSUB)[lc] = make_double2(t0r, trr);
            }
            if (!grid_sync(bar, target, &s_ok)) break;
            for (int q = gi; q < A.nsys; q += LOOP_GROUPS) {
                if (!inner_active(sst[q], sdc[q])) continue;
                const MSys &S = A.sys[q];
                double f0r, frr;
                lanes_final_sum2(S.part + 2 * (size_t)S.nchunks * MSUB, S.nchunks * MSUB, lane, sm[gi], f0r, frr, gsync);
                if (lane == 0) {
                    KState *st = &sst[q];
                    st->rr = frr;
                    st->iter += 1;
                    st->work += 1;
                    const double eps2 = (double)FLT_EPSILON * FLT_EPSILON;
                    if (!finite(frr) || !finite(st->alpha) || !finite(st->w)) {
                        st->done = 1;
                        st->info = 1;  // breakdown: the outer round discards this correction
                    } else if (!(frr > st->tol2 && st->iter < st->maxit)) {
                        st->done = 1;
                    } else if (fabs(f0r) < eps2 * st->r0_sqnorm || st->w == 0.0) {
                        st->done = 1;  // restart needed: end the round, the next one starts afresh
                    } else {
                        st->beta = (f0r / st->rho) * (st->alpha / st->w);
                        st->rho = f0r;
                    }
                }
            }
            __syncthreads();
        } else {
            // the preconditioner is multilevel for a single-system set with a
            // hierarchy (uniform across the grid: the scalars are per-block copies)
            bool mg_on = false;
            if constexpr (CAP <= KMAX) {
                mg_on = A.nsys == 1 && A.sys[0].mg.nlev > 0 && inner_active(sst[0], sdc[0]);
            } else {
                for (int q = 0; q < A.nsys; ++q)
                    mg_on = mg_on || (A.sys[q].mg.nlev > 0 && inner_active(sst[q], sdc[q]));
            }
            // p = r + beta (p - w v); y = D^-1 p
            for (int u = cbegin; u < total_units; u += gstride) {
                const int si = msys_of_chunk(A, u / MSUB);
                if (!inner_active(sst[si], sdc[si])) continue;
                const MSys &S = A.sys[si];
                const int r0 = (u - S.chunk_begin * MSUB) * MUNIT + lane;
                const float beta = (float)sst[si].beta, w = (float)sst[si].w;
    #pragma unroll
                for (int m = 0; m < MRPL; ++m) {
                    const int row = r0 + m * LANES;
                    const float p = __fmaf_rn(beta, __fmaf_rn(-w, S.v[row], S.p[row]), S.r[row]);
                    S.p[row] = p;
                    // a system with a hierarchy: the V-cycle's start w D^-1 p
                    S.y[row] = S.mg.nlev > 0 ? S.mg.omega * S.invdiag32[row] * p : S.invdiag32[row] * p;
                }
            }
            if (!grid_sync(bar, target, &s_ok)) break;
            // multilevel preconditioning: y = M^-1 p (replaces the Jacobi y)
            if (mg_on && !mg_precondition(A, sst, sdc, 0, bar, target, &s_ok)) break;
            // v = A y, <r0, v>
            for (int u = cbegin; u < total_units; u += gstride) {
                const int si = msys_of_chunk(A, u / MSUB);
                if (!inner_active(sst[si], sdc[si])) continue;
                const MSys &S = A.sys[si];
                const int lc = u - S.chunk_begin * MSUB;
                const int r0 = lc * MUNIT + lane;
                float a = 0.0f;
    #pragma unroll
                for (int m = 0; m < MRPL; ++m) {
                    const int row = r0 + m * LANES;
                    const float v = spmv_f32_row(S, row, S.y);
                    S.v[row] = v;
                    if (row < S.n) a = __fmaf_rn(S.r0[row], v, a);
                }
                const float t = lanes_tree_sum<float>(a, lane, reinterpret_cast<float *>(sm[gi]), gsync);
                if (lane == 0) S.part[4 * (size_t)S.nchunks * MSUB + lc] = (double)t;
            }
            if (!grid_sync(bar, target, &s_ok)) break;
            for (int q = gi; q < A.nsys; q += LOOP_GROUPS) {
                if (!inner_active(sst[q], sdc[q])) continue;
                const MSys &S = A.sys[q];
                const double d = lanes_final_sum(S.part + 4 * (size_t)S.nchunks * MSUB, S.nchunks * MSUB, 1, lane, sm[gi], gsync);
                if (lane == 0) sst[q].alpha = sst[q].rho / d;
            }
            __syncthreads();
            // s = r - alpha v; z = D^-1 s
            for (int u = cbegin; u < total_units; u += gstride) {
                const int si = msys_of_chunk(A, u / MSUB);
                if (!inner_active(sst[si], sdc[si])) continue;
                const MSys &S = A.sys[si];
                const int r0 = (u - S.chunk_begin * MSUB) * MUNIT + lane;
                const float alpha = (float)sst[si].alpha;
    #pragma unroll
                for (int m = 0; m < MRPL; ++m) {
                    const int row = r0 + m * LANES;
                    const float sv = __fmaf_rn(-alpha, S.v[row], S.r[row]);
                    S.s[row] = sv;
                    S.z[row] = S.mg.nlev > 0 ? S.mg.omega * S.invdiag32[row] * sv : S.invdiag32[row] * sv;
                }
            }
            if (!grid_sync(bar, target, &s_ok)) break;
            if (mg_on && !mg_precondition(A, sst, sdc, 1, bar, target, &s_ok)) break;
            // t = A z, <t, t>, <t, s>
            for (int u = cbegin; u < total_units; u += gstride) {
                const int si = msys_of_chunk(A, u / MSUB);
                if (!inner_active(sst[si], sdc[si])) continue;
                const MSys &S = A.sys[si];
                const int lc = u - S.chunk_begin * MSUB;
                const int r0 = lc * MUNIT + lane;
                float att = 0.0f, ats = 0.0f;
    #pragma unroll
                for (int m = 0; m < MRPL; ++m) {
                    const int row = r0 + m * LANES;
                    const float t = spmv_f32_row(S, row, S.z);
                    S.t[row] = t;
                    if (row < S.n) {
                        att = __fmaf_rn(t, t, att);
                        ats = __fmaf_rn(t, S.s[row], ats);
                    }
                }
                float tt, ts;
                lanes_tree_sum2<float>(att, ats, lane, reinterpret_cast<float *>(sm[gi]), tt, ts, gsync);
                if (lane == 0) reinterpret_cast<double2 *>(S.part)[lc] = make_double2(tt, ts);
            }
            if (!grid_sync(bar, target, &s_ok)) break;
            for (int q = gi; q < A.nsys; q += LOOP_GROUPS) {
                if (!inner_active(sst[q], sdc[q])) continue;
                const MSys &S = A.sys[q];
                double ftt, fts;
                lanes_final_sum2(S.part, S.nchunks * MSUB, lane, sm[gi], ftt, fts, gsync);
                if (lane == 0) sst[q].w = (ftt > 0.0) ? fts / ftt : 0.0;
            }
            __syncthreads();
            // x += alpha y + w z; r = s - w t; <r0, r>, <r, r>
            for (int u = cbegin; u < total_units; u += gstride) {
                const int si = msys_of_chunk(A, u / MSUB);
                if (!inner_active(sst[si], sdc[si])) continue;
                const MSys &S = A.sys[si];
                const int lc = u - S.chunk_begin * MSUB;
                const int r0 = lc * MUNIT + lane;
                const float alpha = (float)sst[si].alpha, w = (float)sst[si].w;
                float a0r = 0.0f, arr = 0.0f;
    #pragma unroll
                for (int m = 0; m < MRPL; ++m) {
                    const int row = r0 + m * LANES;
                    S.x[row] = __fmaf_rn(w, S.z[row], __fmaf_rn(alpha, S.y[row], S.x[row]));
                    const float r = __fmaf_rn(-w, S.t[row], S.s[row]);
                    S.r[row] = r;
                    if (row < S.n) {
                        a0r = __fmaf_rn(S.r0[row], r, a0r);
                        arr = __fmaf_rn(r, r, arr);
                    }
                }
                float t0r, trr;
                lanes_tree_sum2<float>(a0r, arr, lane, reinterpret_cast<float *>(sm[gi]), t0r, trr, gsync);
                if (lane == 0)
                    reinterpret_cast<double2 *>(S.part + 2 * (size_t)S.nchunks * MSUB)[lc] = make_double2(t0r, trr);
            }
            if (!grid_sync(bar, target, &s_ok)) break;
            for (int q = gi; q < A.nsys; q += LOOP_GROUPS) {
                if (!inner_active(sst[q], sdc[q])) continue;
                const MSys &S = A.sys[q];
                double f0r, frr;
                lanes_final_sum2(S.part + 2 * (size_t)S.nchunks * MSUB, S.nchunks * MSUB, lane, sm[gi], f0r, frr, gsync);
                if (lane == 0) {
                    KState *st = &sst[q];
                    st->rr = frr;
                    st->iter += 1;
                    st->work += 1;
                    const double eps2 = (double)FLT_EPSILON * FLT_EPSILON;
                    if (!finite(frr) || !finite(st->alpha) || !finite(st->w)) {
                        st->done = 1;
                        st->info = 1;  // breakdown: the outer round discards this correction
                    } else if (!(frr > st->tol2 && st->iter < st->maxit)) {
                        st->done = 1;
                    } else if (fabs(f0r) < eps2 * st->r0_sqnorm || st->w == 0.0) {
                        st->done = 1;  // restart needed: end the round, the next one starts afresh
                    } else {
                        st->beta = (f0r / st->rho) * (st->alpha / st->w);
                        st->rho = f0r;
                    }
                }
            }
            __syncthreads();
        }
        bool any = false;
        if constexpr (CAP <= KMAX) {
            for (int q = 0; q < A.nsys; ++q) any = any || inner_active(sst[q], sdc[q]);
        } else {  // the lanes of each warp split the systems
            for (int q = threadIdx.x & 31; q < A.nsys; q += 32) any = any || inner_active(sst[q], sdc[q]);
            any = __any_sync(0xffffffffu, any);
        }
        if (!any) {
            ++it;
            break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < A.nsys) {
        KState k = sst[threadIdx.x];
        k.counter = 0;
        *A.sys[threadIdx.x].st = k;
    }
}

// Step length of the round's correction delta = double(d) / scale:
// theta = <r64, A64 delta> / <A64 delta, A64 delta> minimizes the FP64
// residual along delta, so a correction from an inaccurate FP32 solve can
// shrink the residual less but never grow it.  The last block to finish
// sets dc->theta.
template <int CAP>
__global__ void __launch_bounds__(LANES) k_dc_step(const __grid_constant__ MSetArgT<CAP> A) {
    __shared__ double sm[LANES];
    __shared__ int sh[4];
    for (int c = blockIdx.x; c < A.total_chunks; c += gridDim.x) {
        const MSys &S = A.sys[msys_of_chunk(A, c)];
        if (!(__ldcg(&S.dc->done) == 0 && __ldcg(&S.st->info) == 0)) continue;
        const double inv = 1.0 / __ldcg(&S.dc->scale);
        const int lc = c - S.chunk_begin;
        const int r0 = lc * CH + threadIdx.x;
        const size_t np = (size_t)S.npad;
        double arq = 0.0, aqq = 0.0;
        for (int m = 0; m < RPL; ++m) {
            const int row = r0 + m * LANES;
            const int *nb = S.nbr + row;
            const double *cf = S.coef64 + row;
            const double q = row_ordered(row, nb[0 * np], nb[1 * np], nb[2 * np], nb[3 * np], nb[4 * np], nb[5 * np],
                                         [&](double acc, int sl, int col) {
                                             return __fma_rn(cf[(size_t)sl * np], (double)S.x[col] * inv, acc);
                                         });
            if (row < S.n) {
                arq = __fma_rn(S.r64[row], q, arq);
                aqq = __fma_rn(q, q, aqq);
            }
        }
        double trq, tqq;
        block_tree_sum2(arq, aqq, sm, trq, tqq);
        if (threadIdx.x == 0) reinterpret_cast<double2 *>(S.part)[lc] = make_double2(trq, tqq);
        if (m_arrive_last(&S.dc->counter, (unsigned)S.nchunks, sh)) {
            double frq, fqq;
            final_partials_sum2(S.part, S.nchunks, sm, frq, fqq);
            if (threadIdx.x == 0) {
                S.dc->counter = 0;
                const double th = (fqq > 0.0) ? frq / fqq : 0.0;
                S.dc->theta = finite(th) ? th : 0.0;
            }
        }
    }
}

template <int CAP>
__global__ void k_dc_update(const __grid_constant__ MSetArgT<CAP> A) {
    for (int c = blockIdx.x; c < A.total_chunks; c += gridDim.x) {
        const MSys &S = A.sys[msys_of_chunk(A, c)];
        if (!(__ldcg(&S.dc->done) == 0 && __ldcg(&S.st->info) == 0)) continue;
        const double inv = 1.0 / __ldcg(&S.dc->scale);
        const double theta = __ldcg(&S.dc->theta);
        const int r0 = (c - S.chunk_begin) * CH + threadIdx.x;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            const int row = r0 + m * LANES;
            S.x64[row] = __fma_rn(theta, (double)S.x[row] * inv, S.x64[row]);
        }
    }
}

#undef NS3D_MCHUNK_LOOP

void launch_mg_galerkin(const MSys &S, cudaStream_t st) {
    for (int k = 1; k <= S.mg.nlev; ++k) {
        const MGLevel &C = S.mg.lev[k];
        const int npad_f = k == 1 ? S.npad : S.mg.lev[k - 1].npad;
        const int *nbr_f = k == 1 ? S.nbr : S.mg.lev[k - 1].nbr;
        const float *coef_f = k == 1 ? S.coef32 : S.mg.lev[k - 1].coef;
        count_launches(1);
        k_mg_galerkin<<<std::max(1, std::min((C.n + 255) / 256, 152 * 8)), 256, 0, st>>>(npad_f, nbr_f, coef_f, C);
    }
}

// FP32 copy of a system's coefficients and inverse diagonal
__global__ void k_to_f32(const double *__restrict__ coef, const double *__restrict__ invdiag, int npad,
                         float *__restrict__ coef32, float *__restrict__ invdiag32) {
    const long total = 8L * npad;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        if (i < 7L * npad) coef32[i] = (float)coef[i];
        else invdiag32[i - 7L * npad] = (float)invdiag[i - 7L * npad];
    }
}

// ---- launchers ------------------------------------------------------------------
static inline int m_grid(int total_chunks) { return std::max(1, std::min(total_chunks, device_sm_count() * 32)); }

void launch_to_f32(const double *coef, const double *invdiag, int npad, float *coef32, float *invdiag32,
                   cudaStream_t st) {
    const long total = 8L * npad;
    count_launches(1);
    k_to_f32<<<(int)std::min<long>((total + 255) / 256, 152L * 32), 256, 0, st>>>(coef, invdiag, npad, coef32,
                                                                                invdiag32);
}

template <int CAP>
void launch_dc_resid(const MSetArgT<CAP> &A, int first, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    count_launches(1);
    k_dc_resid<CAP><<<m_grid(A.total_chunks), LANES, 0, st>>>(A, first);
    if (first) {
        count_launches(1);
        k_dc_zero<CAP><<<m_grid(A.total_chunks), LANES, 0, st>>>(A);
    }
}

template <int CAP>
void launch_m32_init(const MSetArgT<CAP> &A, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    count_launches(1);
    k_m32_init<CAP><<<m_grid(A.total_chunks), LANES, 0, st>>>(A);
}


// Sets up to kFusedRows rows run the three-phase loop (fewer barriers; the
// recomputed neighbour operands are cache hits); larger sets run the
// five-phase loop, whose smaller working set stays in the L2 (measured: a
// 42 K-row solve 9% faster fused, a 1 M-row solve 16% slower).
constexpr long kFusedRows = 1L << 19;

// (the V-cycle runs in the five-phase loop)
bool m32_fused(long rows, bool mg) { return rows <= kFusedRows && !mg; }

template <int CAP>
cudaError_t launch_m32_loop(const MSetArgT<CAP> &A, GridBar *bar, int max_iters, cudaStream_t st, int variant,
                            int share) {
    if (A.total_chunks <= 0 || max_iters <= 0) return cudaSuccess;
    long rows = 0;
    bool mg = false;
    for (int i = 0; i < A.nsys; ++i) {
        rows += A.sys[i].n;
        mg = mg || A.sys[i].mg.nlev > 0;
    }
    const bool fused = variant < 0 ? m32_fused(rows, mg) : (variant == 1 && !mg);
    const void *fn = fused ? (const void *)k_m32_loop<true, CAP> : (const void *)k_m32_loop<false, CAP>;
    static std::atomic<int> occ_cache[2];
    int occ = occ_cache[fused].load();
    if (occ == 0) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, LOOP_THREADS, 0);
        if (e != cudaSuccess) return e;
        if (occ <= 0) return cudaErrorLaunchOutOfResources;
        occ_cache[fused] = occ;
    }
    // a merged set (many solves' systems) spreads over its share of the SMs
    const int grid = CAP > KMAX
                         ? std::max(1, std::min(A.total_chunks * MSUB, device_sm_count() * occ / std::max(share, 1)))
                         : loop_grid(A.total_chunks * MSUB, MSUB, occ);
    cudaError_t e = reset_grid_bar(bar, st);
    if (e != cudaSuccess) return e;
    MSetArgT<CAP> a = A;
    void *args[] = {&a, &bar, &max_iters};
    count_launches(1);
    return cudaLaunchCooperativeKernel(fn, grid, LOOP_THREADS, args, 0, st);
}

template <int CAP>
void launch_dc_update(const MSetArgT<CAP> &A, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    count_launches(2);
    k_dc_step<CAP><<<m_grid(A.total_chunks), LANES, 0, st>>>(A);
    k_dc_update<CAP><<<m_grid(A.total_chunks), LANES, 0, st>>>(A);
}

template void launch_dc_resid<KMAX>(const MSetArg &, int, cudaStream_t);
template void launch_dc_resid<KMAX_MERGED_M>(const MSetArgMerged &, int, cudaStream_t);
template void launch_m32_init<KMAX>(const MSetArg &, cudaStream_t);
template void launch_m32_init<KMAX_MERGED_M>(const MSetArgMerged &, cudaStream_t);
template cudaError_t launch_m32_loop<KMAX>(const MSetArg &, GridBar *, int, cudaStream_t, int, int);
template cudaError_t launch_m32_loop<KMAX_MERGED_M>(const MSetArgMerged &, GridBar *, int, cudaStream_t, int, int);
template void launch_dc_update<KMAX>(const MSetArg &, cudaStream_t);
template void launch_dc_update<KMAX_MERGED_M>(const MSetArgMerged &, cudaStream_t);

}  // namespace ns3d
