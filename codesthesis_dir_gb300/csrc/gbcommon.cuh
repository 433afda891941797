// Shared definitions of the GB300 convection library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/gb300_convection.h"

#define GB_CUDA_TRY(expr)                                                        \
    do {                                                                         \
        cudaError_t _e = (expr);                                                 \
        if (_e != cudaSuccess) {                                                 \
            gb_set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr,              \
                         cudaGetErrorString(_e));                                \
            return GB_ERR_CUDA;                                                  \
        }                                                                        \
    } while (0)

// Value of an instance's abort flag once a gang run has taken all of its
// steps (gb_prb_gang_*, gb_axi_gang_*): the instance's kernels skip their
// work from then on, and its run_end reports success.
#define GB_RUN_DONE 4

// Records the last error message (thread-local) returned by gb_last_error().
void gb_set_error(const char *fmt, ...);

// Column-major (i fastest) addressing of a (0:ld-1, 0:np) field.
#define GIX(i, k, ld) ((size_t)(i) + (size_t)(ld) * (size_t)(k))

static inline unsigned gb_ceil_div(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }
