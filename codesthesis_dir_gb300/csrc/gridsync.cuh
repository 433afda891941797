// Bounded grid-wide barrier for persistent cooperative kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>

// Grid-wide barrier of a persistent (cooperatively launched) kernel.  Every wait is bounded: a
// block that waits longer than `limit` polls sets the error flag and every
// block leaves the kernel at its next barrier, so a lost block cannot hang
// the GPU.
struct GridSync {
    unsigned *count;
    unsigned *gen;
    int *err;
    long long limit;
};

__device__ __forceinline__ bool grid_sync(const GridSync &gs)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = gs.gen;
        const unsigned g = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(gs.count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(gs.count, 0u);
            __threadfence();
            atomicAdd(gs.gen, 1u);
        } else {
            long long it = 0;
            while (*vgen == g) {
                if (++it > gs.limit || *(volatile int *)gs.err) {
                    atomicExch(gs.err, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int *)gs.err == 0;
}

