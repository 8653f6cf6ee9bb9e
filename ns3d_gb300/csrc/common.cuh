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
// of LANES = 128 threads; thread (lane) l owns rows l, l+128, ..., l+896 of
// the chunk (coalesced) and accumulates them in that order.  Each warp's 32
// lane values are combined by a halving tree (offsets 16, 8, 4, 2, 1), then
// the 4 warp sums by a halving tree (offsets 2, 1).  Chunk partials of one
// system are combined the same way by the last block to finish: lane l sums
// partials l, l+128, ... in order, then the trees.
constexpr int LANES = 128;
constexpr int RPL = 8;
constexpr int CH = LANES * RPL;

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

// Tree sum over LANES threads (lane = this thread's index among them) that
// synchronize with `sync`: the block's __syncthreads when a block has exactly
// LANES threads, a named barrier when a larger block holds several groups of
// LANES threads.  Returns the tree sum in lane 0 (other lanes get an
// unspecified value).  `sm` needs LANES doubles.
template <class T, class Sync>
__device__ __forceinline__ T lanes_tree_sum(T v, int lane, T *sm, Sync sync) {
    v = v + __shfl_down_sync(0xffffffffu, v, 16);
    v = v + __shfl_down_sync(0xffffffffu, v, 8);
    v = v + __shfl_down_sync(0xffffffffu, v, 4);
    v = v + __shfl_down_sync(0xffffffffu, v, 2);
    v = v + __shfl_down_sync(0xffffffffu, v, 1);
    if ((lane & 31) == 0) sm[lane >> 5] = v;
    sync();
    T r = T(0);
    if (lane < 32) {
        r = (lane < LANES / 32) ? sm[lane] : T(0);
        for (int off = LANES / 64; off >= 1; off >>= 1) r = r + __shfl_down_sync(0xffffffffu, r, off);
    }
    sync();
    return r;
}

// Two tree sums at once, each with exactly the pairings of lanes_tree_sum.
// After the first level of a warp, lanes 0-15 carry the first sum and lanes
// 16-31 the second, so every later level is one shuffle and one add for
// both (FP64 issue is scarce on this GPU).  Results valid in lane 0.
template <class T, class Sync>
__device__ __forceinline__ void lanes_tree_sum2(T a, T b, int lane, T *sm, T &ra, T &rb, Sync sync) {
    static_assert(2 * (LANES / 32) <= 32, "warp sums of both trees fit one warp");
    ra = T(0);
    rb = T(0);
    const bool lo = (lane & 16) == 0;
    // offset 16: lane l < 16 forms a_l + a_(l+16), lane l >= 16 forms b_(l-16) + b_l
    T v = (lo ? a : b) + __shfl_xor_sync(0xffffffffu, lo ? b : a, 16);
    v = v + __shfl_down_sync(0xffffffffu, v, 8);
    v = v + __shfl_down_sync(0xffffffffu, v, 4);
    v = v + __shfl_down_sync(0xffffffffu, v, 2);
    v = v + __shfl_down_sync(0xffffffffu, v, 1);
    constexpr int NW = LANES / 32;
    if ((lane & 31) == 0) sm[lane >> 5] = v;
    if ((lane & 31) == 16) sm[NW + (lane >> 5)] = v;
    sync();
    if (lane < 32) {
        T r = (lane < 2 * NW) ? sm[lane] : T(0);
        for (int off = NW / 2; off >= 1; off >>= 1) r = r + __shfl_down_sync(0xffffffffu, r, off);
        const T r2 = __shfl_sync(0xffffffffu, r, NW);
        ra = r;
        rb = r2;
    }
    sync();
}

struct BlockSync {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
// named barrier `id` (1..15) over the LANES threads of one group
struct GroupSync {
    int id;
    __device__ __forceinline__ void operator()() const {
        asm volatile("bar.sync %0, %1;" ::"r"(id), "n"(LANES) : "memory");
    }
};

// Block of exactly LANES threads; the tree sum in thread 0.
__device__ __forceinline__ double block_tree_sum(double v, double *sm) {
    return lanes_tree_sum<double>(v, threadIdx.x, sm, BlockSync());
}
__device__ __forceinline__ void block_tree_sum2(double a, double b, double *sm, double &ra, double &rb) {
    lanes_tree_sum2<double>(a, b, threadIdx.x, sm, ra, rb, BlockSync());
}

__device__ __forceinline__ double dmaxv(double a, double b) { return (b > a) ? b : a; }
__device__ __forceinline__ double dminv(double a, double b) { return (b < a) ? b : a; }

// maxima / minima over the block (exact in any order); result in every thread
template <bool MAX>
__device__ __forceinline__ double block_extreme(double v, double *sm) {
    const int t = threadIdx.x;
    for (int off = 16; off >= 1; off >>= 1) {
        double o = __shfl_down_sync(0xffffffffu, v, off);
        v = MAX ? dmaxv(v, o) : dminv(v, o);
    }
    if ((t & 31) == 0) sm[t >> 5] = v;
    __syncthreads();
    double r = sm[0];
    for (int w = 1; w < LANES / 32; ++w) r = MAX ? dmaxv(r, sm[w]) : dminv(r, sm[w]);
    __syncthreads();
    return r;
}
__device__ __forceinline__ double block_tree_max(double v, double *sm) { return block_extreme<true>(v, sm); }
__device__ __forceinline__ double block_tree_min(double v, double *sm) { return block_extreme<false>(v, sm); }

// Final combination of `n` chunk partials (strided by `stride` doubles):
// lane l sums partials l, l+LANES, ... in order, then the halving tree.
// Result valid in lane 0.
// The partials a lane adds are loaded 8 at a time before they are added (in
// the same order), so the sum waits for one L2 round trip per 8 partials
// instead of one per partial.
constexpr int FINAL_BATCH = 8;

template <class Sync>
__device__ __forceinline__ double lanes_final_sum(const double *part, int n, int stride, int lane, double *sm,
                                                  Sync sync) {
    double a = 0.0;
    for (int base = lane; base < n; base += FINAL_BATCH * LANES) {
        double v[FINAL_BATCH];
#pragma unroll
        for (int k = 0; k < FINAL_BATCH; ++k) {
            const int i = base + k * LANES;
            v[k] = (i < n) ? __ldcg(part + (size_t)i * stride) : 0.0;
        }
#pragma unroll
        for (int k = 0; k < FINAL_BATCH; ++k)
            if (base + k * LANES < n) a = a + v[k];
    }
    return lanes_tree_sum<double>(a, lane, sm, sync);
}
// the same for the interleaved pairs part[2i] and part[2i+1] (16-byte aligned)
template <class Sync>
__device__ __forceinline__ void lanes_final_sum2(const double *part, int n, int lane, double *sm, double &ra,
                                                 double &rb, Sync sync) {
    double a = 0.0, b = 0.0;
    for (int base = lane; base < n; base += FINAL_BATCH * LANES) {
        double2 v[FINAL_BATCH];
#pragma unroll
        for (int k = 0; k < FINAL_BATCH; ++k) {
            const int i = base + k * LANES;
            v[k] = (i < n) ? __ldcg(reinterpret_cast<const double2 *>(part) + i) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int k = 0; k < FINAL_BATCH; ++k)
            if (base + k * LANES < n) {
                a = a + v[k].x;
                b = b + v[k].y;
            }
    }
    lanes_tree_sum2<double>(a, b, lane, sm, ra, rb, sync);
}

__device__ __forceinline__ double final_partials_sum(const double *part, int n, int stride, double *sm) {
    return lanes_final_sum(part, n, stride, threadIdx.x, sm, BlockSync());
}
__device__ __forceinline__ void final_partials_sum2(const double *part, int n, double *sm, double &ra, double &rb) {
    lanes_final_sum2(part, n, threadIdx.x, sm, ra, rb, BlockSync());
}

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace ns3d

#define NS3D_CUDA_CHECK(expr)                                                          \
    do {                                                                               \
        cudaError_t _e = (expr);                                                       \
        if (_e != cudaSuccess) throw ns3d::CudaError(_e, #expr, __FILE__, __LINE__);   \
    } while (0)
