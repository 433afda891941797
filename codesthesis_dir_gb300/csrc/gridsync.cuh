// Bounded grid-wide barrier for persistent cooperative kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>

// Grid-wide barrier of a persistent (cooperatively launched) kernel.  Every wait is bounded: a
// block that waits longer than `limit` polls sets the error flag and every
// block leaves the kernel at its next barrier, so a lost block cannot hang
// the GPU.  The outcome is read once per block (by the thread that waited)
// and handed to the whole block through shared memory, so all threads of a
// block leave together even when another block raises the flag meanwhile.
struct GridSync {
    unsigned *count;
    unsigned *gen;
    int *err;
    long long limit;
    unsigned long long *tally;   // optional (may be null): barriers passed, counted once per barrier by block 0
};

// Default wait limit: about 1-2 s of polling at 64 ns per poll.
#define GB_GRID_WAIT_LIMIT_DEFAULT (1LL << 24)

__device__ __forceinline__ bool grid_sync(const GridSync &gs)
{
    __shared__ int s_grid_ok;
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
        s_grid_ok = *(volatile int *)gs.err == 0;
        if (gs.tally && blockIdx.x == 0) atomicAdd(gs.tally, 1ull);
    }
    __syncthreads();
    return s_grid_ok != 0;
}

