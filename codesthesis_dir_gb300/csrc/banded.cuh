// Banded line solvers on the device.
//
// The reference solves every line of a sweep with the same matrix
// (tdma/ptdma/pdma of velvor2dperiodicrbconv.f:3046-3164), redoing the
// elimination of the matrix for each line.  Here the matrix part of each
// elimination is done once (factor_* below, one thread, same operations in
// the same order) and every line then applies only the right-hand-side part.
// Both parts round exactly as the reference's interleaved loop does, so a
// line solved here is bit-identical to the reference algorithm on the same
// right-hand side (this file must be compiled with -fmad=false).  The
// factors also hold the reciprocals of the pivots (IEEE divisions done once),
// and every division of a line's elimination is the correctly rounded
// quotient formed from them (divrn.cuh), the same bits as the division.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "divrn.cuh"

// Doubles of each factor layout.
__host__ __device__ inline size_t tdma_fac_len(int n) { return 4 * (size_t)n; }
__host__ __device__ inline size_t ptdma_fac_len(int n) { return 6 * (size_t)n + 3; }
__host__ __device__ inline size_t pdma_fac_len(int n) { return 6 * (size_t)n + 2; }

// ---------------------------------------------------------------------------
// Tridiagonal (tdma, velvor2dperiodicrbconv.f:3046-3064), n unknowns.
// Factor layout (4n doubles): fact[0..n), bp[0..n), c[0..n), 1/bp[0..n).
// ---------------------------------------------------------------------------
__device__ inline void factor_tdma(const double *a, const double *b, const double *c, int n,
                                   double *fac)
{
    double *fact = fac, *bp = fac + n, *cc = fac + 2 * n, *ibp = fac + 3 * n;
    bp[0] = b[0];
    fact[0] = 0.0;
    for (int j = 0; j < n; ++j) cc[j] = c[j];
    for (int j = 1; j < n; ++j) {
        fact[j] = a[j] / bp[j - 1];
        bp[j] = b[j] - fact[j] * c[j - 1];
    }
    for (int j = 0; j < n; ++j) ibp[j] = 1.0 / bp[j];
}

// Solve in place: x[j*stride] holds r on entry, the solution on exit.
// rhs(j) supplies r lazily when x == nullptr-like use is not wanted; the
// generic form below reads r from x.
__device__ inline void apply_tdma(const double *fac, int n, double *x, int stride)
{
    const double *fact = fac, *bp = fac + n, *c = fac + 2 * n, *ibp = fac + 3 * n;
    double prev = x[0];
    for (int j = 1; j < n; ++j) {
        double rj = x[(size_t)j * stride] - fact[j] * prev;
        x[(size_t)j * stride] = rj;
        prev = rj;
    }
    double y = div_by_rcp(x[(size_t)(n - 1) * stride], bp[n - 1], ibp[n - 1]);
    x[(size_t)(n - 1) * stride] = y;
    for (int j = n - 2; j >= 0; --j) {
        y = div_by_rcp(x[(size_t)j * stride] - c[j] * y, bp[j], ibp[j]);
        x[(size_t)j * stride] = y;
    }
}

// ---------------------------------------------------------------------------
// Periodic tridiagonal (ptdma, velvor2dperiodicrbconv.f:3066-3116), n >= 4.
// Factor layout (6n + 3 doubles): f1[n), f2[n), a'[n), b'[n), c'[n), 1/b'[n),
// then fA, fB, fC.
// ---------------------------------------------------------------------------
__device__ inline void factor_ptdma(const double *a0, const double *b0, const double *c0, int n,
                                    double *fac)
{
    double *f1 = fac, *f2 = fac + n, *a = fac + 2 * n, *b = fac + 3 * n, *c = fac + 4 * n;
    const int N = n - 1;
    for (int j = 0; j < n; ++j) {
        a[j] = a0[j];
        b[j] = b0[j];
        c[j] = c0[j];
        f1[j] = 0.0;
        f2[j] = 0.0;
    }
    for (int j = 1; j <= n - 3; ++j) {
        double fact = a[j] / b[j - 1];
        f1[j] = fact;
        b[j] = b[j] - fact * c[j - 1];
        a[j] = -fact * a[j - 1];
        fact = c[N] / b[j - 1];
        f2[j] = fact;
        c[N] = -fact * c[j - 1];
        b[N] = b[N] - fact * a[j - 1];
    }
    double fA = a[n - 2] / b[n - 3];
    b[n - 2] = b[n - 2] - fA * c[n - 3];
    c[n - 2] = c[n - 2] - fA * a[n - 3];
    double fB = c[N] / b[n - 3];
    a[N] = a[N] - fB * c[n - 3];
    b[N] = b[N] - fB * a[n - 3];
    double fC = a[N] / b[n - 2];
    b[N] = b[N] - fC * c[n - 2];
    for (int j = 0; j < n; ++j) fac[5 * n + j] = 1.0 / b[j];
    fac[6 * n + 0] = fA;
    fac[6 * n + 1] = fB;
    fac[6 * n + 2] = fC;
}

__device__ inline void apply_ptdma(const double *fac, int n, double *x, int stride)
{
    const double *f1 = fac, *f2 = fac + n, *a = fac + 2 * n, *b = fac + 3 * n, *c = fac + 4 * n;
    const double *ib = fac + 5 * n;
    const double fA = fac[6 * n], fB = fac[6 * n + 1], fC = fac[6 * n + 2];
    const int N = n - 1;
    double rN = x[(size_t)N * stride];
    double prev = x[0];
    for (int j = 1; j <= n - 3; ++j) {
        double rj = x[(size_t)j * stride] - f1[j] * prev;
        rN = rN - f2[j] * prev;
        x[(size_t)j * stride] = rj;
        prev = rj;
    }
    // prev = r(n-3) final
    double rn2 = x[(size_t)(n - 2) * stride] - fA * prev;
    rN = rN - fB * prev;
    rN = rN - fC * rn2;
    double yN = div_by_rcp(rN, b[N], ib[N]);
    double y = div_by_rcp(rn2 - c[n - 2] * yN, b[n - 2], ib[n - 2]);
    x[(size_t)N * stride] = yN;
    x[(size_t)(n - 2) * stride] = y;
    for (int j = n - 3; j >= 0; --j) {
        y = div_by_rcp(x[(size_t)j * stride] - c[j] * y - a[j] * yN, b[j], ib[j]);
        x[(size_t)j * stride] = y;
    }
}

// ---------------------------------------------------------------------------
// Pentadiagonal (pdma, velvor2dperiodicrbconv.f:3118-3164), n >= 3.
// a: 2nd sub, b: sub, c: diag, d: super, e: 2nd super.
// Factor layout (6n + 2 doubles): cdiv[n), bk1[n), a[n), dn[n), en[n), cN,
// 1/cdiv[n), 1/cN.
// ---------------------------------------------------------------------------
__device__ inline void factor_pdma(const double *a0, const double *b0, const double *c0,
                                   const double *d0, const double *e0, int n, double *fac,
                                   double *work /* 2n doubles */)
{
    double *cdiv = fac, *bk1 = fac + n, *aa = fac + 2 * n, *d = fac + 3 * n, *e = fac + 4 * n;
    double *b = work, *c = work + n;
    for (int j = 0; j < n; ++j) {
        aa[j] = a0[j];
        b[j] = b0[j];
        c[j] = c0[j];
        d[j] = d0[j];
        e[j] = e0[j];
        cdiv[j] = 0.0;
        bk1[j] = 0.0;
    }
    for (int k = 0; k <= n - 2; ++k) {
        cdiv[k] = c[k];
        d[k] = d[k] / c[k];
        e[k] = e[k] / c[k];
        c[k] = 1.0;
        bk1[k] = b[k + 1];
        c[k + 1] = c[k + 1] - b[k + 1] * d[k];
        if (k != n - 2) d[k + 1] = d[k + 1] - b[k + 1] * e[k];
        b[k + 1] = 0.0;
        if (k != n - 2) {
            b[k + 2] = b[k + 2] - aa[k + 2] * d[k];
            c[k + 2] = c[k + 2] - aa[k + 2] * e[k];
        }
    }
    fac[5 * n] = c[n - 1];
    for (int k = 0; k <= n - 2; ++k) fac[5 * n + 1 + k] = 1.0 / cdiv[k];
    fac[6 * n + 1] = 1.0 / c[n - 1];
}

// Solve with the right-hand side produced by rhs(j) (0-based row j), writing
// the normalised eliminated rows and then the solution to x[j*stride].
template <class Rhs>
__device__ inline void apply_pdma_rhs(const double *fac, int n, double *x, int stride, Rhs rhs)
{
    const double *cdiv = fac, *bk1 = fac + n, *aa = fac + 2 * n, *dn = fac + 3 * n, *en = fac + 4 * n;
    const double *icdiv = fac + 5 * n + 1;
    const double cN = fac[5 * n], icN = fac[6 * n + 1];
    double rk = rhs(0);
    double rk1 = rhs(1);
#pragma unroll 4
    for (int k = 0; k <= n - 2; ++k) {
        rk = div_by_rcp(rk, cdiv[k], icdiv[k]);
        x[(size_t)k * stride] = rk;
        rk1 = rk1 - bk1[k] * rk;
        double rk2 = 0.0;
        if (k != n - 2) rk2 = rhs(k + 2) - aa[k + 2] * rk;
        rk = rk1;
        rk1 = rk2;
    }
    double x1 = div_by_rcp(rk, cN, icN);
    x[(size_t)(n - 1) * stride] = x1;
    double x0 = x[(size_t)(n - 2) * stride] - dn[n - 2] * x1;
    x[(size_t)(n - 2) * stride] = x0;
#pragma unroll 4
    for (int j = n - 3; j >= 0; --j) {
        double xj = x[(size_t)j * stride] - dn[j] * x0 - en[j] * x1;
        x[(size_t)j * stride] = xj;
        x1 = x0;
        x0 = xj;
    }
}

// Tridiagonal solve with a lazily produced right-hand side.
template <class Rhs>
__device__ inline void apply_tdma_rhs(const double *fac, int n, double *x, int stride, Rhs rhs)
{
    const double *fact = fac, *bp = fac + n, *c = fac + 2 * n, *ibp = fac + 3 * n;
    double prev = rhs(0);
    x[0] = prev;
#pragma unroll 4
    for (int j = 1; j < n; ++j) {
        double rj = rhs(j) - fact[j] * prev;
        x[(size_t)j * stride] = rj;
        prev = rj;
    }
    double y = div_by_rcp(prev, bp[n - 1], ibp[n - 1]);
    x[(size_t)(n - 1) * stride] = y;
#pragma unroll 4
    for (int j = n - 2; j >= 0; --j) {
        y = div_by_rcp(x[(size_t)j * stride] - c[j] * y, bp[j], ibp[j]);
        x[(size_t)j * stride] = y;
    }
}

template <class Rhs>
__device__ inline void apply_ptdma_rhs(const double *fac, int n, double *x, int stride, Rhs rhs)
{
    for (int j = 0; j < n; ++j) x[(size_t)j * stride] = rhs(j);
    apply_ptdma(fac, n, x, stride);
}

// ---------------------------------------------------------------------------
// FP32 eliminations in place on a line held in shared memory at x[k * pitch]
// (the mixed-precision correction cycles).  Factor layouts: pentadiagonal
// 1/cdiv[n), bk1[n), a[n), dn[n), en[n), 1/cN; tridiagonal fact[n), 1/bp[n),
// c[n).  Pivots are multiplied by their stored reciprocals.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pdma32_smem(const float *fac, int n, float *x, int pitch)
{
    const float *icdiv = fac, *bk1 = fac + n, *aa = fac + 2 * n, *dn = fac + 3 * n, *en = fac + 4 * n;
    float rk = x[0], rk1 = x[pitch];
#pragma unroll 4
    for (int k = 0; k <= n - 2; ++k) {
        const float xr = (k + 2 < n) ? x[(k + 2) * pitch] : 0.f;
        rk = rk * icdiv[k];
        x[k * pitch] = rk;
        rk1 = rk1 - bk1[k] * rk;
        const float rk2 = (k != n - 2) ? xr - aa[k + 2] * rk : 0.f;
        rk = rk1;
        rk1 = rk2;
    }
    float x1 = rk * fac[5 * n];
    x[(n - 1) * pitch] = x1;
    float x0 = x[(n - 2) * pitch] - dn[n - 2] * x1;
    x[(n - 2) * pitch] = x0;
#pragma unroll 4
    for (int j = n - 3; j >= 0; --j) {
        const float xj = x[j * pitch] - dn[j] * x0 - en[j] * x1;
        x[j * pitch] = xj;
        x1 = x0;
        x0 = xj;
    }
}

__device__ __forceinline__ void tdma32_smem(const float *fac, int n, float *x, int pitch)
{
    const float *fact = fac, *ibp = fac + n, *c = fac + 2 * n;
    float prev = x[0];
#pragma unroll 4
    for (int j = 1; j < n; ++j) {
        prev = x[j * pitch] - fact[j] * prev;
        x[j * pitch] = prev;
    }
    float y = prev * ibp[n - 1];
    x[(n - 1) * pitch] = y;
#pragma unroll 4
    for (int j = n - 2; j >= 0; --j) {
        y = (x[j * pitch] - c[j] * y) * ibp[j];
        x[j * pitch] = y;
    }
}
