// Bounded grid barrier of the persistent cooperative kernels (band LDL^T
// factors and solves).
#pragma once

#include <cuda_runtime.h>

#include "internal.hpp"

namespace cb {

// Grid barrier for a cooperative launch. bar->count is zeroed before the
// launch and only grows: the k-th barrier of a kernel (epoch, counted by
// every thread) is passed once count reaches k * nblocks, so a CTA arrives
// with one atomic and nothing is reset on the critical path. The leader
// thread arrives for its CTA after a CTA barrier, with an acq_rel atomic at
// gpu scope (releasing the CTA's writes) and polls with acquire loads (so
// the CTA reads the others' writes after the closing CTA barrier). The wait
// is bounded: after max_polls polls (the default 2^24 is well over a
// second) the CTA records a timeout in bar->err; with max_polls < 0 a CTA
// that is not the last to arrive records it at once, without polling. Once
// the flag is set no CTA waits any more. Returns false when the flag is set,
// and the caller then leaves the kernel, so a fault cannot hang the GPU; the
// host turns the flag into CB_ERR_TIMEOUT.
__device__ __forceinline__ unsigned barrier_arrive(unsigned *count)
{
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;\n" : "=r"(old) : "l"(count) : "memory");
    return old + 1u;
}

__device__ __forceinline__ unsigned barrier_count(const unsigned *count)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(count) : "memory");
    return v;
}

__device__ __forceinline__ bool grid_barrier(GridBarrier *bar, unsigned nblocks, unsigned &epoch,
                                             long long max_polls, unsigned leader = 0)
{
    __shared__ int failed;
    __syncthreads();
    ++epoch;
    if (threadIdx.x == leader) {
        volatile int *verr = &bar->err;
        failed = *verr;
        if (!failed) {
            const unsigned target = epoch * nblocks;
            if (barrier_arrive(&bar->count) < target) {
                long long polls = 0;
                while (max_polls < 0 || barrier_count(&bar->count) < target) {
                    if (*verr) {
                        failed = 1;
                        break;
                    }
                    if (++polls > max_polls) {
                        atomicExch(&bar->err, 1);
                        failed = 1;
                        break;
                    }
                }
            }
        }
    }
    __syncthreads();
    return !failed;
}

}  // namespace cb
