// Banded line solvers on the device.
//
// The reference solves every line of a sweep with the same matrix
// (tdma/ptdma/pdma of velvor2dperiodicrbconv.f:3046-3164), redoing the
// elimination of the matrix for each line.  Here the matrix part of each
// elimination is done once (factor_* below, one thread, same operations in
// the same order) and every line then applies only the right-hand-side part.
// Both parts round exactly as the reference's interleaved loop does, so a
// line solved here is bit-identical to the reference algorithm on the same
// right-hand side (this file must be compiled with -fmad=false).
#pragma once

#include <cuda_runtime.h>

// ---------------------------------------------------------------------------
// Tridiagonal (tdma, velvor2dperiodicrbconv.f:3046-3064), n unknowns.
// Factor layout (3n doubles): fact[0..n), bp[0..n), c[0..n).
// ---------------------------------------------------------------------------
__device__ inline void factor_tdma(const double *a, const double *b, const double *c, int n,
                                   double *fac)
{
    double *fact = fac, *bp = fac + n, *cc = fac + 2 * n;
    bp[0] = b[0];
    fact[0] = 0.0;
    for (int j = 0; j < n; ++j) cc[j] = c[j];
    for (int j = 1; j < n; ++j) {
        fact[j] = a[j] / bp[j - 1];
        bp[j] = b[j] - fact[j] * c[j - 1];
    }
}

// Solve in place: x[j*stride] holds r on entry, the solution on exit.
// rhs(j) supplies r lazily when x == nullptr-like use is not wanted; the
// generic form below reads r from x.
__device__ inline void apply_tdma(const double *fac, int n, double *x, int stride)
{
    const double *fact = fac, *bp = fac + n, *c = fac + 2 * n;
    double prev = x[0];
    for (int j = 1; j < n; ++j) {
        double rj = x[(size_t)j * stride] - fact[j] * prev;
        x[(size_t)j * stride] = rj;
        prev = rj;
    }
    double y = x[(size_t)(n - 1) * stride] / bp[n - 1];
    x[(size_t)(n - 1) * stride] = y;
    for (int j = n - 2; j >= 0; --j) {
        y = (x[(size_t)j * stride] - c[j] * y) / bp[j];
        x[(size_t)j * stride] = y;
    }
}

// ---------------------------------------------------------------------------
// Periodic tridiagonal (ptdma, velvor2dperiodicrbconv.f:3066-3116), n >= 4.
// Factor layout (6n + 3 doubles): f1[n), f2[n), a'[n), b'[n), c'[n), spare[n),
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
    fac[6 * n + 0] = fA;
    fac[6 * n + 1] = fB;
    fac[6 * n + 2] = fC;
}

__device__ inline void apply_ptdma(const double *fac, int n, double *x, int stride)
{
    const double *f1 = fac, *f2 = fac + n, *a = fac + 2 * n, *b = fac + 3 * n, *c = fac + 4 * n;
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
    double yN = rN / b[N];
    double y = (rn2 - c[n - 2] * yN) / b[n - 2];
    x[(size_t)N * stride] = yN;
    x[(size_t)(n - 2) * stride] = y;
    for (int j = n - 3; j >= 0; --j) {
        y = (x[(size_t)j * stride] - c[j] * y - a[j] * yN) / b[j];
        x[(size_t)j * stride] = y;
    }
}

// ---------------------------------------------------------------------------
// Pentadiagonal (pdma, velvor2dperiodicrbconv.f:3118-3164), n >= 3.
// a: 2nd sub, b: sub, c: diag, d: super, e: 2nd super.
// Factor layout (5n + 1 doubles): cdiv[n), bk1[n), a[n), dn[n), en[n), cN.
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
}

// Solve with the right-hand side produced by rhs(j) (0-based row j), writing
// the normalised eliminated rows and then the solution to x[j*stride].
template <class Rhs>
__device__ inline void apply_pdma_rhs(const double *fac, int n, double *x, int stride, Rhs rhs)
{
    const double *cdiv = fac, *bk1 = fac + n, *aa = fac + 2 * n, *dn = fac + 3 * n, *en = fac + 4 * n;
    const double cN = fac[5 * n];
    double rk = rhs(0);
    double rk1 = rhs(1);
    for (int k = 0; k <= n - 2; ++k) {
        rk = rk / cdiv[k];
        x[(size_t)k * stride] = rk;
        rk1 = rk1 - bk1[k] * rk;
        double rk2 = 0.0;
        if (k != n - 2) rk2 = rhs(k + 2) - aa[k + 2] * rk;
        rk = rk1;
        rk1 = rk2;
    }
    double x1 = rk / cN;
    x[(size_t)(n - 1) * stride] = x1;
    double x0 = x[(size_t)(n - 2) * stride] - dn[n - 2] * x1;
    x[(size_t)(n - 2) * stride] = x0;
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
    const double *fact = fac, *bp = fac + n, *c = fac + 2 * n;
    double prev = rhs(0);
    x[0] = prev;
    for (int j = 1; j < n; ++j) {
        double rj = rhs(j) - fact[j] * prev;
        x[(size_t)j * stride] = rj;
        prev = rj;
    }
    double y = prev / bp[n - 1];
    x[(size_t)(n - 1) * stride] = y;
    for (int j = n - 2; j >= 0; --j) {
        y = (x[(size_t)j * stride] - c[j] * y) / bp[j];
        x[(size_t)j * stride] = y;
    }
}

template <class Rhs>
__device__ inline void apply_ptdma_rhs(const double *fac, int n, double *x, int stride, Rhs rhs)
{
    for (int j = 0; j < n; ++j) x[(size_t)j * stride] = rhs(j);
    apply_ptdma(fac, n, x, stride);
}
