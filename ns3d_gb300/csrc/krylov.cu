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
// in constant memory and only reads the system's done flag from global
// memory.  Finished systems make their chunks return at once; the block that
// completes the last chunk of a system reduces that system's partials and
// updates its scalars on the device.  One BiCGSTAB iteration is five kernels:
//   K1 p = r + beta (p - w v); y = D^-1 p
//   K2 v = A y, <r0,v>                      -> alpha
//   K3 s = r - alpha v; z = D^-1 s
//   K4 t = A z, <t,t>, <t,s>                -> w
//   K5 x += alpha y + w z; r = s - w t, <r0,r>, <r,r> -> convergence, beta
// No kernel waits on another block: completion is detected with one atomic
// counter per system, so every launch terminates on its own.
#include <atomic>
#include <cfloat>

#include "device.cuh"
#include "kernels.h"

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
__device__ __forceinline__ double spmv_row(const KSys &S, int row, const double *__restrict__ x) {
    const size_t np = (size_t)S.npad;
    const int *nb = S.nbr + row;
    const double *cf = S.coef + row;
    const int nW = nb[0 * np], nE = nb[1 * np], nS = nb[2 * np], nN = nb[3 * np], nB = nb[4 * np],
              nT = nb[5 * np];
    const double xP = x[row];
    const double xW = x[nW >= 0 ? nW : row], xE = x[nE >= 0 ? nE : row], xS = x[nS >= 0 ? nS : row];
    const double xN = x[nN >= 0 ? nN : row], xB = x[nB >= 0 ? nB : row], xT = x[nT >= 0 ? nT : row];
    const double cP = cf[0], cW = cf[1 * np], cE = cf[2 * np], cS = cf[3 * np], cN = cf[4 * np],
                 cB = cf[5 * np], cT = cf[6 * np];
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

// y = A x for the thread's rows (rows >= n give garbage that callers mask)
__device__ __forceinline__ Row4 spmv4(const KSys &S, int r0, const double *__restrict__ x) {
    Row4 out;
#pragma unroll
    for (int m = 0; m < RPL; ++m) out.v[m] = spmv_row(S, r0 + m * LANES, x);
    return out;
}

// system owning global chunk c (chunk_begin ascending, first system begins at 0)
__device__ __forceinline__ int sys_of_chunk(const KSetArg &A, int c) {
    int s = 0;
#pragma unroll
    for (int q = 1; q < KMAX; ++q)
        if (q < A.nsys && c >= A.sys[q].chunk_begin) s = q;
    return s;
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
__global__ void __launch_bounds__(LANES) k_kr_init(const __grid_constant__ KSetArg A) {
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
__global__ void k_kr_init2(const __grid_constant__ KSetArg A) {
    NS3D_CHUNK_LOOP
        Row4 z;
#pragma unroll
        for (int m = 0; m < RPL; ++m) z.v[m] = 0.0;
        st4(S.p + r0, z);
        st4(S.v + r0, z);
        if (__ldcg(&S.st->zero_rhs)) st4(S.x + r0, z);
    }
}

// K1: p = r + beta (p - w v); y = D^-1 p
__global__ void __launch_bounds__(LANES) k_kr_p(const __grid_constant__ KSetArg A) {
    NS3D_CHUNK_LOOP
        if (!sys_active(S)) continue;
        const double beta = __ldcg(&S.st->beta), w = __ldcg(&S.st->w);
        const Row4 r = ld4(S.r + r0), v = ld4(S.v + r0), iv = ld4(S.invdiag + r0);
        Row4 p = ld4(S.p + r0), y;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            p.v[m] = __fma_rn(beta, __fma_rn(-w, v.v[m], p.v[m]), r.v[m]);
            y.v[m] = iv.v[m] * p.v[m];
        }
        st4(S.p + r0, p);
        st4(S.y + r0, y);
    }
}

// K2: v = A y, <r0, v> -> alpha = rho / <r0, v>
__global__ void __launch_bounds__(LANES) k_kr_v(const __grid_constant__ KSetArg A) {
    __shared__ double sm[LANES];
    __shared__ int sh[2];
    NS3D_CHUNK_LOOP
        if (!sys_active(S)) continue;
        const Row4 v = spmv4(S, r0, S.y);
        const Row4 rr0 = ld4(S.r0 + r0);
        double a = 0.0;
#pragma unroll
        for (int m = 0; m < RPL; ++m)
            if (r0 + m * LANES < S.n) a = __fma_rn(rr0.v[m], v.v[m], a);
        st4(S.v + r0, v);
        const double t = block_tree_sum(a, sm);
        if (threadIdx.x == 0) S.part[2 * (size_t)lc] = t;
        if (arrive_last(S.st, (unsigned)S.nchunks, sh)) {
            const double d = final_partials_sum(S.part, S.nchunks, 2, sm);
            if (threadIdx.x == 0) {
                S.st->counter = 0;
                S.st->alpha = S.st->rho / d;
            }
        }
    }
}

// K3: s = r - alpha v; z = D^-1 s
__global__ void __launch_bounds__(LANES) k_kr_s(const __grid_constant__ KSetArg A) {
    NS3D_CHUNK_LOOP
        if (!sys_active(S)) continue;
        const double alpha = __ldcg(&S.st->alpha);
        const Row4 r = ld4(S.r + r0), v = ld4(S.v + r0), iv = ld4(S.invdiag + r0);
        Row4 s, z;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            s.v[m] = __fma_rn(-alpha, v.v[m], r.v[m]);
            z.v[m] = iv.v[m] * s.v[m];
        }
        st4(S.s + r0, s);
        st4(S.z + r0, z);
    }
}

// K4: t = A z, <t, t>, <t, s> -> w
__global__ void __launch_bounds__(LANES) k_kr_t(const __grid_constant__ KSetArg A) {
    __shared__ double sm[LANES];
    __shared__ int sh[2];
    NS3D_CHUNK_LOOP
        if (!sys_active(S)) continue;
        const Row4 t = spmv4(S, r0, S.z);
        const Row4 s = ld4(S.s + r0);
        double att = 0.0, ats = 0.0;
#pragma unroll
        for (int m = 0; m < RPL; ++m)
            if (r0 + m * LANES < S.n) {
                att = __fma_rn(t.v[m], t.v[m], att);
                ats = __fma_rn(t.v[m], s.v[m], ats);
            }
        st4(S.t + r0, t);
        double tt, ts;
        block_tree_sum2(att, ats, sm, tt, ts);
        if (threadIdx.x == 0) {
            S.part[2 * (size_t)lc + 0] = tt;
            S.part[2 * (size_t)lc + 1] = ts;
        }
        if (arrive_last(S.st, (unsigned)S.nchunks, sh)) {
            double ftt, fts;
            final_partials_sum2(S.part, S.nchunks, sm, ftt, fts);
            if (threadIdx.x == 0) {
                S.st->counter = 0;
                S.st->w = (ftt > 0.0) ? fts / ftt : 0.0;
            }
        }
    }
}

// K5: x += alpha y + w z; r = s - w t; <r0, r>, <r, r> -> loop control
__global__ void __launch_bounds__(LANES) k_kr_x(const __grid_constant__ KSetArg A) {
    __shared__ double sm[LANES];
    __shared__ int sh[2];
    NS3D_CHUNK_LOOP
        if (!sys_active(S)) continue;
        const double alpha = __ldcg(&S.st->alpha), w = __ldcg(&S.st->w);
        const Row4 y = ld4(S.y + r0), z = ld4(S.z + r0), t = ld4(S.t + r0), s = ld4(S.s + r0);
        const Row4 rr0 = ld4(S.r0 + r0);
        Row4 x = ld4(S.x + r0), r;
        double a0r = 0.0, arr = 0.0;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            x.v[m] = __fma_rn(w, z.v[m], __fma_rn(alpha, y.v[m], x.v[m]));
            r.v[m] = __fma_rn(-w, t.v[m], s.v[m]);
            if (r0 + m * LANES < S.n) {
                a0r = __fma_rn(rr0.v[m], r.v[m], a0r);
                arr = __fma_rn(r.v[m], r.v[m], arr);
            }
        }
        // rows >= n of x are padding; they receive values computed from zeros
        st4(S.x + r0, x);
        st4(S.r + r0, r);
        double t0r, trr;
        block_tree_sum2(a0r, arr, sm, t0r, trr);
        if (threadIdx.x == 0) {
            S.part[2 * (size_t)lc + 0] = t0r;
            S.part[2 * (size_t)lc + 1] = trr;
        }
        if (arrive_last(S.st, (unsigned)S.nchunks, sh)) {
            double f0r, frr;
            final_partials_sum2(S.part, S.nchunks, sm, f0r, frr);
            if (threadIdx.x == 0) {
                KState *st = S.st;
                st->counter = 0;
                st->rr = frr;
                st->iter += 1;
                st->work += 1;
                if (!(frr > st->tol2 && st->iter < st->maxit)) {
                    finish_loop(st);
                } else {
                    const double eps2 = DBL_EPSILON * DBL_EPSILON;
                    if (fabs(f0r) < eps2 * st->r0_sqnorm) {
                        st->paused = 1;  // host recomputes r = b - A x and r0
                    } else {
                        st->beta = (f0r / st->rho) * (st->alpha / st->w);
                        st->rho = f0r;
                    }
                }
            }
        }
    }
}

// restart of paused systems: r = b - A x, r0 = r, rho = |r0|^2
__global__ void __launch_bounds__(LANES) k_kr_restart(const __grid_constant__ KSetArg A) {
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

void launch_krylov_init(const KSetArg &A, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    count_launches(2);
    k_kr_init<<<kr_grid(A.total_chunks), LANES, 0, st>>>(A);
    k_kr_init2<<<kr_grid(A.total_chunks), LANES, 0, st>>>(A);
}

void launch_krylov_iteration(const KSetArg &A, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    const int g = kr_grid(A.total_chunks);
    count_launches(5);
    k_kr_p<<<g, LANES, 0, st>>>(A);
    k_kr_v<<<g, LANES, 0, st>>>(A);
    k_kr_s<<<g, LANES, 0, st>>>(A);
    k_kr_t<<<g, LANES, 0, st>>>(A);
    k_kr_x<<<g, LANES, 0, st>>>(A);
}

void launch_krylov_kernel(int which, const KSetArg &A, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    const int g = kr_grid(A.total_chunks);
    count_launches(1);
    switch (which) {
        case 0: k_kr_p<<<g, LANES, 0, st>>>(A); break;
        case 1: k_kr_v<<<g, LANES, 0, st>>>(A); break;
        case 2: k_kr_s<<<g, LANES, 0, st>>>(A); break;
        case 3: k_kr_t<<<g, LANES, 0, st>>>(A); break;
        default: k_kr_x<<<g, LANES, 0, st>>>(A); break;
    }
}

void launch_krylov_restart(const KSetArg &A, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    count_launches(1);
    k_kr_restart<<<kr_grid(A.total_chunks), LANES, 0, st>>>(A);
}

void launch_spmv(const SysView &A, const double *x, double *y, cudaStream_t st) {
    if (A.n <= 0) return;
    count_launches(1);
    k_spmv<<<std::max(1, std::min(A.nchunks, device_sm_count() * 6)), LANES, 0, st>>>(A, x, y);
}

}  // namespace ns3d
