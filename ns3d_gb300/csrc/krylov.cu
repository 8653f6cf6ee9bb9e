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
// A solve set holds several independent systems (the three momentum
// components, or the pressure system, or many images).  Their rows are
// processed as one list of 1024-row chunks; every kernel below walks the
// chunks grid-stride, skips systems that have finished, and the block that
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

struct ChunkCtx {
    int sys, lc, r0;  // system, local chunk, first row of this thread
    bool active;
};

__device__ __forceinline__ ChunkCtx chunk_ctx(const KSys *sys, const int *chunk_sys, int c, int *sh) {
    ChunkCtx cx;
    if (threadIdx.x == 0) {
        int s = chunk_sys[c];
        const KState *st = sys[s].st;
        int act = (__ldcg(&st->done) == 0 && __ldcg(&st->paused) == 0) ? 1 : 0;
        sh[0] = s;
        sh[1] = act;
    }
    __syncthreads();
    cx.sys = sh[0];
    cx.active = sh[1] != 0;
    __syncthreads();
    cx.lc = c - sys[cx.sys].chunk_begin;
    cx.r0 = cx.lc * CH + threadIdx.x;
    return cx;
}

__device__ __forceinline__ bool arrive_last(KState *st, unsigned int total, int *sh) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int prev = atomicAdd(&st->counter, 1u);
        sh[2] = (prev == total - 1) ? 1 : 0;
    }
    __syncthreads();
    bool last = sh[2] != 0;
    if (last) __threadfence();
    return last;
}

__device__ __forceinline__ void finish_loop(KState *st) {
    // loop exit: error() and info() as Eigen reports them
    st->done = 1;
    st->error = sqrt(st->rr / st->rhs_sqnorm);
    st->info = (st->error <= st->tol) ? 0 : 2;
}

// ---- init: r = b - A x, r0 = r, |r|^2, |b|^2 ---------------------------------
__global__ void __launch_bounds__(LANES) k_kr_init(const KSys *__restrict__ sys, const int *__restrict__ chunk_sys,
                                                   int total_chunks) {
    __shared__ double sm[LANES];
    __shared__ int sh[4];
    for (int c = blockIdx.x; c < total_chunks; c += gridDim.x) {
        ChunkCtx cx = chunk_ctx(sys, chunk_sys, c, sh);
        const KSys &S = sys[cx.sys];
        double arr = 0.0, abb = 0.0;
        {
            const Row4 ax = spmv4(S, cx.r0, S.x);
            const Row4 b = ld4(S.b + cx.r0);
            Row4 r;
#pragma unroll
            for (int m = 0; m < RPL; ++m) {
                r.v[m] = b.v[m] - ax.v[m];
                if (cx.r0 + m * LANES < S.n) {
                    arr = __fma_rn(r.v[m], r.v[m], arr);
                    abb = __fma_rn(b.v[m], b.v[m], abb);
                }
            }
            st4(S.r + cx.r0, r);
            st4(S.r0 + cx.r0, r);
        }
        double trr = block_tree_sum(arr, sm);
        double tbb = block_tree_sum(abb, sm);
        if (threadIdx.x == 0) {
            S.part[2 * (size_t)cx.lc + 0] = trr;
            S.part[2 * (size_t)cx.lc + 1] = tbb;
        }
        if (arrive_last(S.st, (unsigned)S.nchunks, sh)) {
            double rr = final_partials_sum(S.part + 0, S.nchunks, 2, sm);
            double bb = final_partials_sum(S.part + 1, S.nchunks, 2, sm);
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
__global__ void k_kr_init2(const KSys *__restrict__ sys, const int *__restrict__ chunk_sys, int total_chunks) {
    __shared__ int sh[4];
    for (int c = blockIdx.x; c < total_chunks; c += gridDim.x) {
        if (threadIdx.x == 0) sh[0] = chunk_sys[c];
        __syncthreads();
        const KSys &S = sys[sh[0]];
        __syncthreads();
        const int r0 = (c - S.chunk_begin) * CH + threadIdx.x;
        Row4 z;
#pragma unroll
        for (int m = 0; m < RPL; ++m) z.v[m] = 0.0;
        st4(S.p + r0, z);
        st4(S.v + r0, z);
        if (__ldcg(&S.st->zero_rhs)) st4(S.x + r0, z);
    }
}

// K1: p = r + beta (p - w v); y = D^-1 p
__global__ void __launch_bounds__(LANES) k_kr_p(const KSys *__restrict__ sys, const int *__restrict__ chunk_sys,
                                                int total_chunks) {
    __shared__ int sh[4];
    for (int c = blockIdx.x; c < total_chunks; c += gridDim.x) {
        ChunkCtx cx = chunk_ctx(sys, chunk_sys, c, sh);
        if (!cx.active) continue;
        const KSys &S = sys[cx.sys];
        const double beta = __ldcg(&S.st->beta), w = __ldcg(&S.st->w);
        const Row4 r = ld4(S.r + cx.r0), v = ld4(S.v + cx.r0), iv = ld4(S.invdiag + cx.r0);
        Row4 p = ld4(S.p + cx.r0), y;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            p.v[m] = __fma_rn(beta, __fma_rn(-w, v.v[m], p.v[m]), r.v[m]);
            y.v[m] = iv.v[m] * p.v[m];
        }
        st4(S.p + cx.r0, p);
        st4(S.y + cx.r0, y);
    }
}

// K2: v = A y, <r0, v> -> alpha = rho / <r0, v>
__global__ void __launch_bounds__(LANES) k_kr_v(const KSys *__restrict__ sys, const int *__restrict__ chunk_sys,
                                                int total_chunks) {
    __shared__ double sm[LANES];
    __shared__ int sh[4];
    for (int c = blockIdx.x; c < total_chunks; c += gridDim.x) {
        ChunkCtx cx = chunk_ctx(sys, chunk_sys, c, sh);
        if (!cx.active) continue;
        const KSys &S = sys[cx.sys];
        const Row4 v = spmv4(S, cx.r0, S.y);
        const Row4 r0 = ld4(S.r0 + cx.r0);
        double a = 0.0;
#pragma unroll
        for (int m = 0; m < RPL; ++m)
            if (cx.r0 + m * LANES < S.n) a = __fma_rn(r0.v[m], v.v[m], a);
        st4(S.v + cx.r0, v);
        double t = block_tree_sum(a, sm);
        if (threadIdx.x == 0) S.part[2 * (size_t)cx.lc] = t;
        if (arrive_last(S.st, (unsigned)S.nchunks, sh)) {
            double d = final_partials_sum(S.part, S.nchunks, 2, sm);
            if (threadIdx.x == 0) {
                S.st->counter = 0;
                S.st->alpha = S.st->rho / d;
            }
        }
    }
}

// K3: s = r - alpha v; z = D^-1 s
__global__ void __launch_bounds__(LANES) k_kr_s(const KSys *__restrict__ sys, const int *__restrict__ chunk_sys,
                                                int total_chunks) {
    __shared__ int sh[4];
    for (int c = blockIdx.x; c < total_chunks; c += gridDim.x) {
        ChunkCtx cx = chunk_ctx(sys, chunk_sys, c, sh);
        if (!cx.active) continue;
        const KSys &S = sys[cx.sys];
        const double alpha = __ldcg(&S.st->alpha);
        const Row4 r = ld4(S.r + cx.r0), v = ld4(S.v + cx.r0), iv = ld4(S.invdiag + cx.r0);
        Row4 s, z;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            s.v[m] = __fma_rn(-alpha, v.v[m], r.v[m]);
            z.v[m] = iv.v[m] * s.v[m];
        }
        st4(S.s + cx.r0, s);
        st4(S.z + cx.r0, z);
    }
}

// K4: t = A z, <t, t>, <t, s> -> w
__global__ void __launch_bounds__(LANES) k_kr_t(const KSys *__restrict__ sys, const int *__restrict__ chunk_sys,
                                                int total_chunks) {
    __shared__ double sm[LANES];
    __shared__ int sh[4];
    for (int c = blockIdx.x; c < total_chunks; c += gridDim.x) {
        ChunkCtx cx = chunk_ctx(sys, chunk_sys, c, sh);
        if (!cx.active) continue;
        const KSys &S = sys[cx.sys];
        const Row4 t = spmv4(S, cx.r0, S.z);
        const Row4 s = ld4(S.s + cx.r0);
        double att = 0.0, ats = 0.0;
#pragma unroll
        for (int m = 0; m < RPL; ++m)
            if (cx.r0 + m * LANES < S.n) {
                att = __fma_rn(t.v[m], t.v[m], att);
                ats = __fma_rn(t.v[m], s.v[m], ats);
            }
        st4(S.t + cx.r0, t);
        double tt = block_tree_sum(att, sm);
        double ts = block_tree_sum(ats, sm);
        if (threadIdx.x == 0) {
            S.part[2 * (size_t)cx.lc + 0] = tt;
            S.part[2 * (size_t)cx.lc + 1] = ts;
        }
        if (arrive_last(S.st, (unsigned)S.nchunks, sh)) {
            double ftt = final_partials_sum(S.part + 0, S.nchunks, 2, sm);
            double fts = final_partials_sum(S.part + 1, S.nchunks, 2, sm);
            if (threadIdx.x == 0) {
                S.st->counter = 0;
                S.st->w = (ftt > 0.0) ? fts / ftt : 0.0;
            }
        }
    }
}

// K5: x += alpha y + w z; r = s - w t; <r0, r>, <r, r> -> loop control
__global__ void __launch_bounds__(LANES) k_kr_x(const KSys *__restrict__ sys, const int *__restrict__ chunk_sys,
                                                int total_chunks) {
    __shared__ double sm[LANES];
    __shared__ int sh[4];
    for (int c = blockIdx.x; c < total_chunks; c += gridDim.x) {
        ChunkCtx cx = chunk_ctx(sys, chunk_sys, c, sh);
        if (!cx.active) continue;
        const KSys &S = sys[cx.sys];
        const double alpha = __ldcg(&S.st->alpha), w = __ldcg(&S.st->w);
        const Row4 y = ld4(S.y + cx.r0), z = ld4(S.z + cx.r0), t = ld4(S.t + cx.r0), s = ld4(S.s + cx.r0);
        const Row4 r0 = ld4(S.r0 + cx.r0);
        Row4 x = ld4(S.x + cx.r0), r;
        double a0r = 0.0, arr = 0.0;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            x.v[m] = __fma_rn(w, z.v[m], __fma_rn(alpha, y.v[m], x.v[m]));
            r.v[m] = __fma_rn(-w, t.v[m], s.v[m]);
            if (cx.r0 + m * LANES < S.n) {
                a0r = __fma_rn(r0.v[m], r.v[m], a0r);
                arr = __fma_rn(r.v[m], r.v[m], arr);
            }
        }
        // x may be a field whose padding is shared with nothing: rows >= n
        // are written with the values computed from zero padding
        st4(S.x + cx.r0, x);
        st4(S.r + cx.r0, r);
        double t0r = block_tree_sum(a0r, sm);
        double trr = block_tree_sum(arr, sm);
        if (threadIdx.x == 0) {
            S.part[2 * (size_t)cx.lc + 0] = t0r;
            S.part[2 * (size_t)cx.lc + 1] = trr;
        }
        if (arrive_last(S.st, (unsigned)S.nchunks, sh)) {
            double f0r = final_partials_sum(S.part + 0, S.nchunks, 2, sm);
            double frr = final_partials_sum(S.part + 1, S.nchunks, 2, sm);
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
__global__ void __launch_bounds__(LANES) k_kr_restart(const KSys *__restrict__ sys,
                                                      const int *__restrict__ chunk_sys, int total_chunks) {
    __shared__ double sm[LANES];
    __shared__ int sh[4];
    for (int c = blockIdx.x; c < total_chunks; c += gridDim.x) {
        if (threadIdx.x == 0) {
            int s = chunk_sys[c];
            sh[0] = s;
            sh[1] = (__ldcg(&sys[s].st->paused) != 0 && __ldcg(&sys[s].st->done) == 0) ? 1 : 0;
        }
        __syncthreads();
        const int sidx = sh[0];
        const bool act = sh[1] != 0;
        __syncthreads();
        if (!act) continue;
        const KSys &S = sys[sidx];
        const int lc = c - S.chunk_begin, r0i = lc * CH + threadIdx.x;
        const Row4 ax = spmv4(S, r0i, S.x);
        const Row4 b = ld4(S.b + r0i);
        Row4 r;
        double arr = 0.0;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            r.v[m] = b.v[m] - ax.v[m];
            if (r0i + m * LANES < S.n) arr = __fma_rn(r.v[m], r.v[m], arr);
        }
        st4(S.r + r0i, r);
        st4(S.r0 + r0i, r);
        double trr = block_tree_sum(arr, sm);
        if (threadIdx.x == 0) S.part[2 * (size_t)lc] = trr;
        if (arrive_last(S.st, (unsigned)S.nchunks, sh)) {
            double rr = final_partials_sum(S.part, S.nchunks, 2, sm);
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

// plain y = A x over one system (tests and diagnostics)
__global__ void k_spmv(SysView A, const double *__restrict__ x, double *__restrict__ y) {
    KSys S;
    S.n = A.n; S.npad = A.npad; S.coef = A.coef; S.nbr = A.nbr;
    for (int c = blockIdx.x; c < A.nchunks; c += gridDim.x) {
        const int r0 = c * CH + threadIdx.x;
        const Row4 v = spmv4(S, r0, x);
        st4(y + r0, v);
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

void launch_krylov_init(const KSys *sys, int nsys, const int *chunk_sys, int total_chunks, cudaStream_t st) {
    (void)nsys;
    if (total_chunks <= 0) return;
    count_launches(1); k_kr_init<<<kr_grid(total_chunks), LANES, 0, st>>>(sys, chunk_sys, total_chunks);
    count_launches(1); k_kr_init2<<<kr_grid(total_chunks), LANES, 0, st>>>(sys, chunk_sys, total_chunks);
}

void launch_krylov_iteration(const KSys *sys, int nsys, const int *chunk_sys, int total_chunks, cudaStream_t st) {
    (void)nsys;
    if (total_chunks <= 0) return;
    const int g = kr_grid(total_chunks);
    count_launches(1); k_kr_p<<<g, LANES, 0, st>>>(sys, chunk_sys, total_chunks);
    count_launches(1); k_kr_v<<<g, LANES, 0, st>>>(sys, chunk_sys, total_chunks);
    count_launches(1); k_kr_s<<<g, LANES, 0, st>>>(sys, chunk_sys, total_chunks);
    count_launches(1); k_kr_t<<<g, LANES, 0, st>>>(sys, chunk_sys, total_chunks);
    count_launches(1); k_kr_x<<<g, LANES, 0, st>>>(sys, chunk_sys, total_chunks);
}

void launch_krylov_kernel(int which, const KSys *sys, int nsys, const int *chunk_sys, int total_chunks,
                          cudaStream_t st) {
    (void)nsys;
    if (total_chunks <= 0) return;
    const int g = kr_grid(total_chunks);
    count_launches(1);
    switch (which) {
        case 0: k_kr_p<<<g, LANES, 0, st>>>(sys, chunk_sys, total_chunks); break;
        case 1: k_kr_v<<<g, LANES, 0, st>>>(sys, chunk_sys, total_chunks); break;
        case 2: k_kr_s<<<g, LANES, 0, st>>>(sys, chunk_sys, total_chunks); break;
        case 3: k_kr_t<<<g, LANES, 0, st>>>(sys, chunk_sys, total_chunks); break;
        default: k_kr_x<<<g, LANES, 0, st>>>(sys, chunk_sys, total_chunks); break;
    }
}

void launch_krylov_restart(const KSys *sys, int nsys, const int *chunk_sys, int total_chunks, cudaStream_t st) {
    (void)nsys;
    if (total_chunks <= 0) return;
    count_launches(1); k_kr_restart<<<kr_grid(total_chunks), LANES, 0, st>>>(sys, chunk_sys, total_chunks);
}

void launch_spmv(const SysView &A, const double *x, double *y, cudaStream_t st) {
    if (A.n <= 0) return;
    count_launches(1); k_spmv<<<std::max(1, std::min(A.nchunks, device_sm_count() * 6)), LANES, 0, st>>>(A, x, y);
}

}  // namespace ns3d
