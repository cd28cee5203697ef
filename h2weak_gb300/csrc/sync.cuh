// Device-side synchronisation shared by the persistent matvec kernels.
#pragma once
#include <cstdint>

namespace h2w {

// Grid-wide barrier for cooperative launches (all CTAs are co-resident by
// construction of the launch). bar[0] counts arrivals, bar[1] is the
// generation. The spin is bounded by `limit` polls: a barrier that does not
// complete in time sets *err and lets the CTA continue, so the kernel always
// ends (with wrong results, which the error word reports).
constexpr long long GRID_SPIN_LIMIT = 1LL << 26;
static __device__ __forceinline__ void grid_barrier(unsigned *bar, unsigned nblocks, int32_t *err,
                                                    long long limit = GRID_SPIN_LIMIT) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == nblocks - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long it = 0;
            while (*vgen == gen) {
                if (++it > limit) {
                    atomicExch(err, 1);
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

}  // namespace h2w
