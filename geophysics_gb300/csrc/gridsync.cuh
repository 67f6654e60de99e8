// Grid-wide barrier of a cooperative launch, shared by the persistent
// whole-shot kernels.
#pragma once

#include "tc_util.cuh"

namespace geo {

// Arrival counter read with acquire semantics at GPU scope.
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// One arrival per block on a counter that only grows (barrier k completes at
// k*gridDim.x arrivals).  The fence before the arrival publishes the block's
// writes; the wait is bounded (2 s) and a timeout sets the error word and
// ends the block, after which every other block's next wait times out too.
// Values other blocks wrote before the barrier are read through L2
// (__ldcg): L1 is not coherent with them.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned target, int *err) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        int ok = 1;
        __threadfence();
        atomicAdd(bar, 1u);
        if (ld_acquire_u32(bar) < target) {
            const uint64_t t0 = tc::gtimer();
            while (ld_acquire_u32(bar) < target)
                if (tc::gtimer() - t0 > 2000000000ull) {
                    atomicExch(err, 1);
                    ok = 0;
                    break;
                }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

}  // namespace geo
