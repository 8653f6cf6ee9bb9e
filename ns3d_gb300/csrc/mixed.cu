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
//   k_m32_p/v/s/t/x   the five BiCGSTAB kernels in FP32 on A32 d = f
//   k_dc_update  x += double(d) / scale
// An inner solve stops at its relative target, at the iteration budget, or
// at a breakdown (|rho| tiny, non-finite scalars); the next round restarts
// from the new FP64 residual.  iterations() reports the inner iterations.
#include <cfloat>

#include "device.cuh"
#include "kernels.h"
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
    const int nW = nb[0 * np], nE = nb[1 * np], nS = nb[2 * np], nN = nb[3 * np], nB = nb[4 * np], nT = nb[5 * np];
    float acc = cf[0] * x[row];
    acc = __fmaf_rn(cf[1 * np], x[nW >= 0 ? nW : row], acc);
    acc = __fmaf_rn(cf[3 * np], x[nS >= 0 ? nS : row], acc);
    acc = __fmaf_rn(cf[5 * np], x[nB >= 0 ? nB : row], acc);
    acc = __fmaf_rn(cf[6 * np], x[nT >= 0 ? nT : row], acc);
    acc = __fmaf_rn(cf[4 * np], x[nN >= 0 ? nN : row], acc);
    acc = __fmaf_rn(cf[2 * np], x[nE >= 0 ? nE : row], acc);
    return acc;
}

__device__ __forceinline__ double spmv_f64_row(const MSys &S, int row, const double *__restrict__ x) {
    const size_t np = (size_t)S.npad;
    const int *nb = S.nbr + row;
    const double *cf = S.coef64 + row;
    return row_ordered(row, nb[0 * np], nb[1 * np], nb[2 * np], nb[3 * np], nb[4 * np], nb[5 * np],
                       [&](double acc, int s, int col) { return __fma_rn(cf[(size_t)s * np], x[col], acc); });
}

// system owning global chunk c (systems in chunk order, first begins at 0)
__device__ __forceinline__ int msys_of_chunk(const MSetArg &A, int c) {
    int s = 0;
#pragma unroll
    for (int q = 1; q < KMAX; ++q)
        if (q < A.nsys && c >= A.sys[q].chunk_begin) s = q;
    return s;
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
__global__ void __launch_bounds__(LANES) k_dc_resid(const __grid_constant__ MSetArg A, int first) {
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
                    st->maxit = dc->maxit - dc->total_iter;
                }
            }
        }
    }
}

// x64 = 0 for systems with a zero right-hand side (first round)
__global__ void k_dc_zero(const __grid_constant__ MSetArg A) {
    for (int c = blockIdx.x; c < A.total_chunks; c += gridDim.x) {
        const MSys &S = A.sys[msys_of_chunk(A, c)];
        if (!__ldcg(&S.dc->zero_rhs)) continue;
        const int r0 = (c - S.chunk_begin) * CH + threadIdx.x;
#pragma unroll
        for (int m = 0; m < RPL; ++m) S.x64[r0 + m * LANES] = 0.0;
    }
}

// ---- FP32 inner solve -------------------------------------------------------
__global__ void __launch_bounds__(LANES) k_m32_init(const __grid_constant__ MSetArg A) {
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

__global__ void __launch_bounds__(LANES) k_m32_p(const __grid_constant__ MSetArg A) {
    __shared__ int sh[4];
    NS3D_MCHUNK_LOOP(true)
        const float beta = (float)__ldcg(&S.st->beta), w = (float)__ldcg(&S.st->w);
        const RowF4 r = ldf4(S.r + r0), v = ldf4(S.v + r0), iv = ldf4(S.invdiag32 + r0);
        RowF4 p = ldf4(S.p + r0), y;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            p.v[m] = __fmaf_rn(beta, __fmaf_rn(-w, v.v[m], p.v[m]), r.v[m]);
            y.v[m] = iv.v[m] * p.v[m];
        }
        stf4(S.p + r0, p);
        stf4(S.y + r0, y);
    }
}

__global__ void __launch_bounds__(LANES) k_m32_v(const __grid_constant__ MSetArg A) {
    __shared__ double sm[LANES];
    __shared__ int sh[4];
    NS3D_MCHUNK_LOOP(true)
        float a = 0.0f;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            const int row = r0 + m * LANES;
            const float v = spmv_f32_row(S, row, S.y);
            S.v[row] = v;
            if (row < S.n) a = __fmaf_rn(S.r0[row], v, a);
        }
        const double t = block_tree_sum((double)a, sm);
        if (threadIdx.x == 0) S.part[2 * (size_t)lc] = t;
        if (m_arrive_last(&S.st->counter, (unsigned)S.nchunks, sh)) {
            const double d = final_partials_sum(S.part, S.nchunks, 2, sm);
            if (threadIdx.x == 0) {
                S.st->counter = 0;
                S.st->alpha = S.st->rho / d;
            }
        }
    }
}

__global__ void __launch_bounds__(LANES) k_m32_s(const __grid_constant__ MSetArg A) {
    __shared__ int sh[4];
    NS3D_MCHUNK_LOOP(true)
        const float alpha = (float)__ldcg(&S.st->alpha);
        const RowF4 r = ldf4(S.r + r0), v = ldf4(S.v + r0), iv = ldf4(S.invdiag32 + r0);
        RowF4 s, z;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            s.v[m] = __fmaf_rn(-alpha, v.v[m], r.v[m]);
            z.v[m] = iv.v[m] * s.v[m];
        }
        stf4(S.s + r0, s);
        stf4(S.z + r0, z);
    }
}

__global__ void __launch_bounds__(LANES) k_m32_t(const __grid_constant__ MSetArg A) {
    __shared__ double sm[LANES];
    __shared__ int sh[4];
    NS3D_MCHUNK_LOOP(true)
        float att = 0.0f, ats = 0.0f;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            const int row = r0 + m * LANES;
            const float t = spmv_f32_row(S, row, S.z);
            S.t[row] = t;
            if (row < S.n) {
                att = __fmaf_rn(t, t, att);
                ats = __fmaf_rn(t, S.s[row], ats);
            }
        }
        double tt, ts;
        block_tree_sum2((double)att, (double)ats, sm, tt, ts);
        if (threadIdx.x == 0) {
            S.part[2 * (size_t)lc + 0] = tt;
            S.part[2 * (size_t)lc + 1] = ts;
        }
        if (m_arrive_last(&S.st->counter, (unsigned)S.nchunks, sh)) {
            double ftt, fts;
            final_partials_sum2(S.part, S.nchunks, sm, ftt, fts);
            if (threadIdx.x == 0) {
                S.st->counter = 0;
                S.st->w = (ftt > 0.0) ? fts / ftt : 0.0;
            }
        }
    }
}

__global__ void __launch_bounds__(LANES) k_m32_x(const __grid_constant__ MSetArg A) {
    __shared__ double sm[LANES];
    __shared__ int sh[4];
    NS3D_MCHUNK_LOOP(true)
        const float alpha = (float)__ldcg(&S.st->alpha), w = (float)__ldcg(&S.st->w);
        const RowF4 y = ldf4(S.y + r0), z = ldf4(S.z + r0), t = ldf4(S.t + r0), s = ldf4(S.s + r0);
        const RowF4 rr0 = ldf4(S.r0 + r0);
        RowF4 x = ldf4(S.x + r0), r;
        float a0r = 0.0f, arr = 0.0f;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            x.v[m] = __fmaf_rn(w, z.v[m], __fmaf_rn(alpha, y.v[m], x.v[m]));
            r.v[m] = __fmaf_rn(-w, t.v[m], s.v[m]);
            if (r0 + m * LANES < S.n) {
                a0r = __fmaf_rn(rr0.v[m], r.v[m], a0r);
                arr = __fmaf_rn(r.v[m], r.v[m], arr);
            }
        }
        stf4(S.x + r0, x);
        stf4(S.r + r0, r);
        double t0r, trr;
        block_tree_sum2((double)a0r, (double)arr, sm, t0r, trr);
        if (threadIdx.x == 0) {
            S.part[2 * (size_t)lc + 0] = t0r;
            S.part[2 * (size_t)lc + 1] = trr;
        }
        if (m_arrive_last(&S.st->counter, (unsigned)S.nchunks, sh)) {
            double f0r, frr;
            final_partials_sum2(S.part, S.nchunks, sm, f0r, frr);
            if (threadIdx.x == 0) {
                KState *st = S.st;
                st->counter = 0;
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
    }
}

__global__ void k_dc_update(const __grid_constant__ MSetArg A) {
    for (int c = blockIdx.x; c < A.total_chunks; c += gridDim.x) {
        const MSys &S = A.sys[msys_of_chunk(A, c)];
        if (!(__ldcg(&S.dc->done) == 0 && __ldcg(&S.st->info) == 0)) continue;
        const double inv = 1.0 / __ldcg(&S.dc->scale);
        const int r0 = (c - S.chunk_begin) * CH + threadIdx.x;
#pragma unroll
        for (int m = 0; m < RPL; ++m) {
            const int row = r0 + m * LANES;
            S.x64[row] = __fma_rn((double)S.x[row], inv, S.x64[row]);
        }
    }
}

#undef NS3D_MCHUNK_LOOP

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

void launch_dc_resid(const MSetArg &A, int first, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    count_launches(1);
    k_dc_resid<<<m_grid(A.total_chunks), LANES, 0, st>>>(A, first);
    if (first) {
        count_launches(1);
        k_dc_zero<<<m_grid(A.total_chunks), LANES, 0, st>>>(A);
    }
}

void launch_m32_init(const MSetArg &A, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    count_launches(1);
    k_m32_init<<<m_grid(A.total_chunks), LANES, 0, st>>>(A);
}

void launch_m32_iteration(const MSetArg &A, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    const int g = m_grid(A.total_chunks);
    count_launches(5);
    k_m32_p<<<g, LANES, 0, st>>>(A);
    k_m32_v<<<g, LANES, 0, st>>>(A);
    k_m32_s<<<g, LANES, 0, st>>>(A);
    k_m32_t<<<g, LANES, 0, st>>>(A);
    k_m32_x<<<g, LANES, 0, st>>>(A);
}

void launch_dc_update(const MSetArg &A, cudaStream_t st) {
    if (A.total_chunks <= 0) return;
    count_launches(1);
    k_dc_update<<<m_grid(A.total_chunks), LANES, 0, st>>>(A);
}

}  // namespace ns3d
