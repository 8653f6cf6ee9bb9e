// common.cuh -- shared definitions of the NS3D GB300 kernels.
//
// Floating-point contract (every FP64 translation unit is compiled with
// --fmad=false): expressions round exactly as written, and fused
// multiply-adds appear only where __fma_rn is called.  Together with the
// fixed reduction order below this makes the device results reproducible
// run to run and identical to the CPU restatement used by the tests.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ns3d {

// ---- fixed-order reductions ---------------------------------------------
// Rows are cut into chunks of CH = 1024.  A chunk is processed by one block
// of LANES = 256 threads; thread (lane) l owns rows 4l..4l+3 of the chunk and
// accumulates them in order.  The 256 lane values are combined by a halving
// tree (offsets 128, 64, ..., 1).  Chunk partials of one system are combined
// the same way by the last block to finish: lane l sums partials l, l+256, ...
// in order, then the tree.
constexpr int CH = 1024;
constexpr int LANES = 256;
constexpr int RPL = 4;

__device__ __forceinline__ double warp_tree_sum(double v) {
    // offsets 16..1 of the halving tree inside one warp; lane 0 ends with the
    // value the tree assigns to position 0 of this warp's 32-lane group
    v = v + __shfl_down_sync(0xffffffffu, v, 16);
    v = v + __shfl_down_sync(0xffffffffu, v, 8);
    v = v + __shfl_down_sync(0xffffffffu, v, 4);
    v = v + __shfl_down_sync(0xffffffffu, v, 2);
    v = v + __shfl_down_sync(0xffffffffu, v, 1);
    return v;
}

// Block of exactly LANES threads; returns the tree sum in thread 0 (other
// threads get an unspecified value).  `sm` needs LANES doubles.
__device__ __forceinline__ double block_tree_sum(double v, double *sm) {
    const int t = threadIdx.x;
    sm[t] = v;
    __syncthreads();
    if (t < 128) sm[t] = sm[t] + sm[t + 128];
    __syncthreads();
    if (t < 64) sm[t] = sm[t] + sm[t + 64];
    __syncthreads();
    double r = 0.0;
    if (t < 32) {
        r = sm[t] + sm[t + 32];
        r = warp_tree_sum(r);
    }
    __syncthreads();
    return r;
}

__device__ __forceinline__ double dmaxv(double a, double b) { return (b > a) ? b : a; }
__device__ __forceinline__ double dminv(double a, double b) { return (b < a) ? b : a; }

// tree of maxima (order is irrelevant for max, kept identical for clarity)
__device__ __forceinline__ double block_tree_max(double v, double *sm) {
    const int t = threadIdx.x;
    sm[t] = v;
    __syncthreads();
    for (int off = 128; off >= 1; off >>= 1) {
        if (t < off) sm[t] = dmaxv(sm[t], sm[t + off]);
        __syncthreads();
    }
    double r = sm[0];
    __syncthreads();
    return r;
}
__device__ __forceinline__ double block_tree_min(double v, double *sm) {
    const int t = threadIdx.x;
    sm[t] = v;
    __syncthreads();
    for (int off = 128; off >= 1; off >>= 1) {
        if (t < off) sm[t] = dminv(sm[t], sm[t + off]);
        __syncthreads();
    }
    double r = sm[0];
    __syncthreads();
    return r;
}

// Final combination of `n` chunk partials (strided by `stride` doubles):
// lane l sums partials l, l+256, ... in order, then the halving tree.
// Result valid in thread 0.
__device__ __forceinline__ double final_partials_sum(const double *part, int n, int stride, double *sm) {
    double a = 0.0;
    for (int i = threadIdx.x; i < n; i += LANES) a = a + __ldcg(part + (size_t)i * stride);
    return block_tree_sum(a, sm);
}

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace ns3d

#define NS3D_CUDA_CHECK(expr)                                                          \
    do {                                                                               \
        cudaError_t _e = (expr);                                                       \
        if (_e != cudaSuccess) throw ns3d::CudaError(_e, #expr, __FILE__, __LINE__);   \
    } while (0)
