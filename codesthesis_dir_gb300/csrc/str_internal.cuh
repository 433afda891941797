// Internal interface between the stretched-grid multigrid (str.cu) and the
// axisymmetric annulus on a stretched grid (axi.cu).
#pragma once

#include "gbcommon.cuh"

// Queues the stretched multigrid solve of h on device arrays psi, rhs
// ((0:n1, 0:n2), leading dimension n1 + 1) on stream s; see str.cu.
cudaError_t gb_str_launch_device(const gb_str *h, double *psi, const double *rhs, int *status, int *abort, int mixed,
                                 double tolcon, int maxsweeps, int nrel, int mode, cudaStream_t s);
