// loop.cuh -- grid-wide synchronisation of the persistent (cooperative)
// solver kernels.
#pragma once

#include "device.cuh"

namespace ns3d {

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier of a cooperative launch.  The arrival counter only
// grows: barrier k of a launch ends when it reaches k * gridDim.x, so a
// waiting block sees the end as soon as the last arrival lands (no reset, no
// second flag).  The wait gives up after kBarrierLimitNs (or 2^31 polls):
// the block records the failure in bar->err and returns false, and the
// kernel stops at once -- so a launch always terminates, and the host
// reports the error.
constexpr unsigned long long kBarrierLimitNs = 4000000000ull;

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void red_release_add(unsigned int *p, unsigned int v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// The block barrier orders every thread's writes before thread 0's release
// arrival; thread 0's acquire poll plus the closing block barrier order the
// block's later reads after every other block's arrival.
__device__ __forceinline__ bool grid_sync(GridBar *bar, unsigned int &target, int *s_ok) {
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        target += gridDim.x;
        red_release_add(&bar->count, 1u);
        if ((int)(ld_acquire(&bar->count) - target) < 0) {
            const unsigned long long t0 = global_ns();
            const unsigned long long lim = bar->limit_ns ? bar->limit_ns : kBarrierLimitNs;
            unsigned int polls = 0;
            while ((int)(ld_acquire(&bar->count) - target) < 0) {
                if ((++polls & 255u) == 0 && (global_ns() - t0 > lim || polls > 0x7fffffffu)) {
                    atomicExch(&bar->err, 1);
                    ok = 0;
                    break;
                }
            }
        }
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

// The arrival target a launch starts from (thread 0 keeps it): 0, or the
// test bias of GridBar.
__device__ __forceinline__ unsigned int grid_sync_start(const GridBar *bar) {
    return threadIdx.x == 0 ? bar->bias : 0u;
}

}  // namespace ns3d
