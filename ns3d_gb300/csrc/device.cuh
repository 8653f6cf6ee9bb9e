// device.cuh -- device-side data layout of the NS3D GB300 solver.
//
// HBM layout (all int32 / FP64, one allocation family per solver instance):
//   image      uint8  nx*ny*nz        binarized, rotated, padded (0 = fluid)
//   pmap, vmap, wmap  int32 nx*ny*nz  index maps (-1 = no node), C order
//   umap       int32 (nx+1)*ny*nz
//   per system (u, v, w on faces; p on cells), rows padded to a multiple of
//   the 1024-row reduction chunk:
//     cell     int32 [npad]     row -> linear position in its map
//     coef     f64   [7][npad]  slots P,W,E,S,N,B,T (structure of arrays)
//     nbr      int32 [6][npad]  columns of W,E,S,N,B,T (-1 = no entry)
//     rhs, rowsum, invdiag  f64 [npad]
//   Krylov workspace per system: r, r0, p, v, y, s, z, t  f64 [npad]
#pragma once

#include "common.cuh"

namespace ns3d {

enum Slot { SP = 0, SW = 1, SE = 2, SS = 3, SN = 4, SB = 5, ST = 6 };

struct Grid {
    int nx, ny, nz;
    const int *pmap, *umap, *vmap, *wmap;
    __host__ __device__ __forceinline__ long lin(int i, int j, int k) const { return ((long)i * ny + j) * nz + k; }
    __device__ __forceinline__ int P(int i, int j, int k) const { return pmap[lin(i, j, k)]; }
    __device__ __forceinline__ int U(int i, int j, int k) const { return umap[lin(i, j, k)]; }
    __device__ __forceinline__ int V(int i, int j, int k) const { return vmap[lin(i, j, k)]; }
    __device__ __forceinline__ int W(int i, int j, int k) const { return wmap[lin(i, j, k)]; }
    __device__ __forceinline__ void ijk(long c, int &i, int &j, int &k) const {
        k = (int)(c % nz);
        long t = c / nz;
        j = (int)(t % ny);
        i = (int)(t / ny);
    }
    // SafeVectorValue (src/NSBase.cxx:1757-1771): the node value or 0
    __device__ __forceinline__ double su(const double *f, int i, int j, int k) const {
        if (i >= nx + 1 || i < 0 || j >= ny || j < 0 || k >= nz || k < 0) return 0;
        int r = U(i, j, k);
        return r > -1 ? f[r] : 0;
    }
    __device__ __forceinline__ double sv(const double *f, int i, int j, int k) const {
        if (i >= nx || i < 0 || j >= ny || j < 0 || k >= nz || k < 0) return 0;
        int r = V(i, j, k);
        return r > -1 ? f[r] : 0;
    }
    __device__ __forceinline__ double sw(const double *f, int i, int j, int k) const {
        if (i >= nx || i < 0 || j >= ny || j < 0 || k >= nz || k < 0) return 0;
        int r = W(i, j, k);
        return r > -1 ? f[r] : 0;
    }
};

struct SysView {
    int n, npad, nchunks;
    const int *cell;
    double *coef;  // [7][npad]
    int *nbr;      // [6][npad]
    double *rhs, *rowsum, *invdiag;
    __device__ __forceinline__ double &c(int s, int r) const { return coef[(size_t)s * npad + r]; }
    __device__ __forceinline__ int nb(int s, int r) const { return nbr[(size_t)s * npad + r]; }
};

// Row sum / product in ascending column order.  For every system of this
// solver the ascending order of a row's columns is W,S,B,P,T,N,E except that
// W comes after S and B when W is the previous row, and E comes before T and
// N when E is the next row (the u outlet faces are numbered right after the
// last cell's west face).
template <class Op>
__device__ __forceinline__ double row_ordered(int row, int nW, int nE, int nS, int nN, int nB, int nT, Op op) {
    double acc = 0.0;
    // nW >= 0 matters for row 0: a missing W (-1) must not read as "row - 1"
    if (nW >= 0 && nW == row - 1) {
        if (nS >= 0) acc = op(acc, SS, nS);
        if (nB >= 0) acc = op(acc, SB, nB);
        acc = op(acc, SW, nW);
    } else {
        if (nW >= 0) acc = op(acc, SW, nW);
        if (nS >= 0) acc = op(acc, SS, nS);
        if (nB >= 0) acc = op(acc, SB, nB);
    }
    acc = op(acc, SP, row);
    if (nE >= 0 && nE == row + 1) {
        acc = op(acc, SE, nE);
        if (nT >= 0) acc = op(acc, ST, nT);
        if (nN >= 0) acc = op(acc, SN, nN);
    } else {
        if (nT >= 0) acc = op(acc, ST, nT);
        if (nN >= 0) acc = op(acc, SN, nN);
        if (nE >= 0) acc = op(acc, SE, nE);
    }
    return acc;
}

// ---- BiCGSTAB state of one system ---------------------------------------
struct KState {
    double rho, alpha, w, beta;   // Krylov scalars (beta = next step's beta)
    double r0_sqnorm, rhs_sqnorm, tol, tol2, rr, error;
    int iter, maxit, restarts;
    int done;      // loop finished
    int paused;    // restart requested: host recomputes the residual
    int info;      // Eigen ComputationInfo
    int zero_rhs;  // rhs == 0: x = 0, iterations() = maxit
    int work;      // iterations executed, restarts included (work accounting)
    unsigned int counter;  // arrivals of chunks in the current kernel
    unsigned int pad2_;
};

struct KSys {  // one system of a solve set (device array)
    int n, npad, nchunks, chunk_begin;
    const double *coef;
    const int *nbr;
    const double *invdiag;
    const double *b;
    double *x, *r, *r0, *p, *v, *y, *s, *z, *t;
    double *part;  // [PART_PER_CHUNK * nchunks]: reduction partials (layout in krylov.cu)
    KState *st;
};

// chunk partials held per system (the FP64 loop uses 5 per chunk, the FP32
// loop 5 per quarter chunk)
constexpr int PART_PER_CHUNK = 20;

// A solve set as a kernel argument (passed by value, read from constant
// memory): the systems in chunk order, sys[0].chunk_begin == 0.  A solver
// instance's own sets hold up to KMAX systems (its three momentum
// components, or its pressure system); a merged set holds the systems of
// many concurrent solves (up to KMAX_MERGED, 8.7 KB of kernel parameters).
constexpr int KMAX = 4;
constexpr int KMAX_MERGED = 64;
template <int CAP>
struct KSetArgT {
    int nsys, total_chunks;
    KSys sys[CAP];
};
using KSetArg = KSetArgT<KMAX>;
using KSetArgMerged = KSetArgT<KMAX_MERGED>;
static_assert(sizeof(KSetArgMerged) <= 32000, "kernel parameter space");

// The persistent BiCGSTAB loop kernel: block shape and its grid barrier.
// Loads of global data that no thread writes during the kernel (matrix
// coefficients, neighbour tables, the multilevel hierarchy) go through the
// read-only data path (measured 0.6% faster in the FP64 loop, 1.3% in the
// FP32 multilevel loop); never for shared memory or for vectors the kernel
// itself updates.
template <class T>
__device__ __forceinline__ T ro(const T *p) { return __ldg(p); }

#ifndef NS3D_LOOP_THREADS
#define NS3D_LOOP_THREADS 1024
#endif
constexpr int LOOP_THREADS = NS3D_LOOP_THREADS;
constexpr int LOOP_GROUPS = LOOP_THREADS / LANES;
// blocks per SM the loop kernels are compiled for (64 registers a thread)
constexpr int LOOP_MIN_BLOCKS = LOOP_THREADS >= 1024 ? 1 : 1024 / LOOP_THREADS;
static_assert(LOOP_GROUPS >= KMAX, "the FP32 loop kernel: group s combines the partials of system s");
struct GridBar {  // arrival counter and error flag on separate 128-byte lines
    unsigned int count;
    // Zero in normal launches.  A test (ns3d_debug_barrier_timeout) sets
    // `bias`, arrivals every barrier waits for beyond the grid's own, which
    // never come, and `limit_ns`, a short wait limit (0 = kBarrierLimitNs).
    unsigned int bias;
    unsigned long long limit_ns;
    unsigned int pad0_[28];
    int err, pad1_[31];
};
static_assert(sizeof(GridBar) == 256, "GridBar: two 128-byte lines");
// per-phase time of the loop kernel (block 0, ns of the global timer)
struct LoopProf {
    unsigned long long ns[5];
    long long iters;
    int ok, pad_;
};

}  // namespace ns3d
