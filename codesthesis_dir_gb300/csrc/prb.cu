// 2D periodic Rayleigh-Benard hot path on the device: compact-scheme
// Dufort-Frankel transport of vorticity and temperature, wall boundary
// conditions, Poisson right-hand sides, Nusselt integrals and the
// velocity-component multigrid solves of
// monashubuntudir_velvor2dperiodicrbconvdir/velvor2dperiodicrbconv.f (PRB).
//
// Numerics: every expression keeps the reference's operation order and this
// translation unit is compiled with -fmad=false, so results are bit-identical
// to the reference algorithm (and to the C oracle) for the same inputs.
//
// Layout: each field is a column-major (0:ld-1, 0:np) array, ld = nr+2, all
// twenty fields of one instance in one allocation.  For the grids these
// drivers use (nr <= 512, np <= 2048) an instance is at most ~170 MB and the
// working set of a step stays in the 126 MB L2 for nr*np up to ~1.5e6.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "banded.cuh"
#include "gbcommon.cuh"
#include "prb_internal.cuh"

// ---------------------------------------------------------------------------
// Matrix factors of the compact-derivative line solves (one thread).
// ---------------------------------------------------------------------------
__global__ void k_transport_factors(int nr, int np, double *fac_r1, double *fac_x,
                                    double *fac_rT, double *work, double *fac_xw1, double *fac_xw2)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int nmax = (nr > np ? nr : np) + 2;
    double *a = work, *b = work + nmax, *c = work + 2 * nmax;
    // (1,4,1) on nr-1 rows: Cr and thr of Cvorticity (PRB:812-829, 855-879)
    for (int j = 0; j < nr - 1; ++j) { a[j] = 1.0; b[j] = 4.0; c[j] = 1.0; }
    factor_tdma(a, b, c, nr - 1, fac_r1);
    // periodic (1,4,1) on np+1 rows: Ch, thh (PRB:834-850, 884-896, 1271-1289)
    for (int j = 0; j < np + 1; ++j) { a[j] = 1.0; b[j] = 4.0; c[j] = 1.0; }
    factor_ptdma(a, b, c, np + 1, fac_x);
    // thr of temperature on nr rows with the wall rows of PRB:1249-1258
    for (int j = 0; j < nr; ++j) { a[j] = 1.0; b[j] = 4.0; c[j] = 1.0; }
    b[0] = 1.0; c[0] = 2.0;
    a[nr - 1] = 2.0; b[nr - 1] = 1.0;
    factor_tdma(a, b, c, nr, fac_rT);
    if (fac_xw1) {
        // the tank's x-lines: (1,4,1) over k = 1..np-1 (C points) and over the
        // cells k = 1..np (T), velvor2dhorconvtank.f:355-369, :616-624
        for (int j = 0; j < np; ++j) { a[j] = 1.0; b[j] = 4.0; c[j] = 1.0; }
        factor_tdma(a, b, c, np - 1, fac_xw1);
        factor_tdma(a, b, c, np, fac_xw2);
    }
}

// REAL*4 literals 2./3. and 1./6. of PRB:865-872, as the doubles they widen to.
#define F23 ((double)(2.0f / 3.0f))
#define F16 ((double)(1.0f / 6.0f))

// Cr (tdma along r) -> A and thr at C points (tdma along r) -> An, one thread
// per column k.  PRB:810-830 and PRB:854-880.
__device__ __forceinline__ void k_cvort_deriv_r_body(const PrbDev &d, int bidx)
{
    const int k = bidx * blockDim.x + threadIdx.x;
    if (k > d.np || *d.abort) return;
    const int ld = d.ld, nr = d.nr, np = d.np;
    const double dri = d.dri;
    const double *C = d.f[GB_F_C], *th = d.f[GB_F_th];
    auto rhsC = [&](int j) -> double {
        const int i = j + 1;
        if (i == 1)
            return 3.0 * (C[GIX(2, k, ld)] - C[GIX(0, k, ld)]) * dri -
                   (-1.5 * C[GIX(0, k, ld)] + 2.0 * C[GIX(1, k, ld)] - 0.5 * C[GIX(2, k, ld)]) * dri;
        if (i == nr - 1)
            return 3.0 * (C[GIX(nr, k, ld)] - C[GIX(nr - 2, k, ld)]) * dri -
                   (0.5 * C[GIX(nr - 2, k, ld)] - 2.0 * C[GIX(nr - 1, k, ld)] + 1.5 * C[GIX(nr, k, ld)]) * dri;
        return 3.0 * (C[GIX(i + 1, k, ld)] - C[GIX(i - 1, k, ld)]) * dri;
    };
    apply_tdma_rhs(d.fac_r1, nr - 1, d.f[GB_F_A] + GIX(1, k, ld), 1, rhsC);
    const int ka = (k == np) ? 1 : k + 1;
    auto rhsT = [&](int j) -> double {
        const int i = j + 1;
        if (i == 1)
            return 1.5 * (th[GIX(2, k, ld)] + th[GIX(2, ka, ld)] - th[GIX(1, k, ld)] - th[GIX(1, ka, ld)]) * dri -
                   (-F23 * (th[GIX(0, k, ld)] + th[GIX(0, ka, ld)]) + 0.5 * (th[GIX(1, k, ld)] + th[GIX(1, ka, ld)]) +
                    F16 * (th[GIX(2, k, ld)] + th[GIX(2, ka, ld)])) * dri;
        if (i == nr - 1)
            return 1.5 * (th[GIX(nr, k, ld)] + th[GIX(nr, ka, ld)] - th[GIX(nr - 1, k, ld)] - th[GIX(nr - 1, ka, ld)]) * dri -
                   (-F16 * (th[GIX(nr - 1, k, ld)] + th[GIX(nr - 1, ka, ld)]) - 0.5 * (th[GIX(nr, k, ld)] + th[GIX(nr, ka, ld)]) +
                    F23 * (th[GIX(nr + 1, k, ld)] + th[GIX(nr + 1, ka, ld)])) * dri;
        return 1.5 * (th[GIX(i + 1, k, ld)] + th[GIX(i + 1, ka, ld)] - th[GIX(i, k, ld)] - th[GIX(i, ka, ld)]) * dri;
    };
    apply_tdma_rhs(d.fac_r1, nr - 1, d.f[GB_F_An] + GIX(1, k, ld), 1, rhsT);
}

__global__ void k_cvort_deriv_r(PrbDev d) { k_cvort_deriv_r_body(d, blockIdx.x); }

// Ch (periodic tdma along x) -> B and thh at C points -> Bn, one thread per
// row i = 1..nr-1.  PRB:833-851 and PRB:882-897.
__device__ __forceinline__ void k_cvort_deriv_x_body(const PrbDev &d, int bidx)
{
    const int i = bidx * blockDim.x + threadIdx.x + 1;
    if (i > d.nr - 1 || *d.abort) return;
    const int ld = d.ld, np = d.np;
    const double dpi = d.dpi;
    const double *C = d.f[GB_F_C], *th = d.f[GB_F_th];
    auto rhsC = [&](int k) -> double {
        if (k == np || k == 0) return 3.0 * (C[GIX(i, 1, ld)] - C[GIX(i, np - 1, ld)]) * dpi;
        return 3.0 * (C[GIX(i, k + 1, ld)] - C[GIX(i, k - 1, ld)]) * dpi;
    };
    apply_ptdma_rhs(d.fac_x, np + 1, d.f[GB_F_B] + GIX(i, 0, ld), ld, rhsC);
    auto rhsT = [&](int k) -> double {
        const int ka = (k == np) ? 1 : k + 1;
        return 1.5 * (th[GIX(i + 1, ka, ld)] + th[GIX(i, ka, ld)] - th[GIX(i + 1, k, ld)] - th[GIX(i, k, ld)]) * dpi;
    };
    apply_ptdma_rhs(d.fac_x, np + 1, d.f[GB_F_Bn] + GIX(i, 0, ld), ld, rhsT);
}

__global__ void k_cvort_deriv_x(PrbDev d) { k_cvort_deriv_x_body(d, blockIdx.x); }

// Vorticity update, PRB:706-776 (first) / PRB:900-982 (leapfrog).  Annulus
// (velvor2dnewsch3.4.f:710-786 / :911-993): radius r = r0 + i dr, the Cra/r
// term, 0.5*Cp in the leapfrog RHS1 and the rotational buoyancy in RHS2.
// Oblique gravity (mpkoks.f): RHS2 = -Ra thr 0.707106781 with thr = An.
__device__ __forceinline__ void k_cvort_update_body(const PrbDev &d, int first, int bidx)
{
    const int t = bidx * blockDim.x + threadIdx.x;
    const int nrow = d.nr - 1;
    if (t >= nrow * (d.np + 1) || *d.abort) return;
    const int i = t % nrow + 1, k = t / nrow;
    const int ld = d.ld, np = d.np;
    const double dri = d.dri, dpi = d.dpi, Ptl = d.Pr, dt = d.dt, Ra = d.Ra;
    const double *C = d.f[GB_F_C], *Cp = d.f[GB_F_Cp];
    const double *uel = d.f[GB_F_uel], *vel = d.f[GB_F_vel];
    const int ip = i + 1;
    int km = k - 1, ka = k + 1;
    if (k == 0) km = np - 1;
    if (k == np) ka = 1;
    const double ri = d.polar ? 1.0 / (d.r0 + (double)i * d.dr) : 1.0;
    const double u = (uel[GIX(i, ka, ld)] + uel[GIX(i, k, ld)]) * 0.5;
    const double v = (vel[GIX(i, k, ld)] + vel[GIX(ip, k, ld)]) * 0.5;
    const double Chha = (C[GIX(i, ka, ld)] + C[GIX(i, km, ld)]) * (dpi * dpi);
    const double Ch = d.f[GB_F_B][GIX(i, k, ld)];
    const double Crra = (C[GIX(i - 1, k, ld)] + C[GIX(i + 1, k, ld)]) * (dri * dri);
    const double cnr = -1.0 * (dri * dri);
    const double Cr = d.f[GB_F_A][GIX(i, k, ld)];
    const double thh = d.f[GB_F_Bn][GIX(i, k, ld)];
    const double cnh = (-1.0 * (dpi * dpi)) * (ri * ri);
    double RHS1, RHS2, cf1;
    if (d.polar) {
        const double Cra = (C[GIX(i + 1, k, ld)] - C[GIX(i - 1, k, ld)]) * 0.5 * dri;
        const double thr = d.f[GB_F_An][GIX(i, k, ld)];
        if (first) {
            RHS1 = Crra + Cra * ri + Chha * (ri * ri) + C[GIX(i, k, ld)] / (Ptl * dt);
            cf1 = 1.0 / (Ptl * dt) - cnr - cnh;
        } else {
            RHS1 = Crra + Cra * ri + Chha * (ri * ri) + 0.5 * Cp[GIX(i, k, ld)] / (Ptl * dt);
            cf1 = 0.5 / (Ptl * dt) - cnr - cnh;
        }
        RHS2 = -Ra * thh + 2.0 * Ra * (-thr * u - thh * v * ri) / d.Re / Ptl;
    } else {
        if (first) {
            RHS1 = Crra + Chha * (ri * ri) + C[GIX(i, k, ld)] / (Ptl * dt);
            cf1 = 1.0 / (Ptl * dt) - cnr - cnh;
        } else {
            RHS1 = Crra + Chha * (ri * ri) + 0.5 * C[GIX(i, k, ld)] / (Ptl * dt);
            cf1 = 0.5 / (Ptl * dt) - cnr - cnh;
        }
        // mpkoks.f:769-770, :974-975: gravity along the diagonal, REAL*4 0.707106781
        RHS2 = d.oblique ? -Ra * d.f[GB_F_An][GIX(i, k, ld)] * (double)0.707106781f : -Ra * thh;
    }
    const double ULT = (u * Cr + v * Ch * ri) / Ptl;
    const double cf2 = cnr + cnh;
    const double cn = (cf2 * Cp[GIX(i, k, ld)] - ULT - RHS2 + RHS1) / cf1;
    d.f[GB_F_Cn][GIX(i, k, ld)] = cn;
    if (!first) d.f[GB_F_Ap][GIX(i, k, ld)] = cn;
}

__global__ void k_cvort_update(PrbDev d, int first) { k_cvort_update_body(d, first, blockIdx.x); }

// Robert filter X += gamma (Xn - 2X + Xp) on rows 1..imax, gamma = 0.02
// (PRB:1041-1045, PRB:1435-1440) or 0.05 in the annulus
// (velvor2dnewsch3.4.f:1055, :1454).
__device__ __forceinline__ void k_robert_body(const PrbDev &d, int fx, int fxn, int fxp, int imax, int bidx)
{
    const int t = bidx * blockDim.x + threadIdx.x;
    if (t >= imax * (d.np + 1) || *d.abort) return;
    const int i = t % imax + 1, k = t / imax;
    const size_t c = GIX(i, k, d.ld);
    const double gamma = d.robert;
    double *X = d.f[fx];
    X[c] = X[c] + gamma * (d.f[fxn][c] - 2.0 * X[c] + d.f[fxp][c]);
}

__global__ void k_robert(PrbDev d, int fx, int fxn, int fxp, int imax) { k_robert_body(d, fx, fxn, fxp, imax, blockIdx.x); }

// thr (tdma along r, third-order wall rows) -> A, one thread per column k
// (PRB:1244-1268).
__device__ __forceinline__ void k_temp_deriv_r_body(const PrbDev &d, int bidx)
{
    const int k = bidx * blockDim.x + threadIdx.x;
    if (k > d.np || *d.abort) return;
    const int ld = d.ld, nr = d.nr;
    const double dri = d.dri;
    const double *th = d.f[GB_F_th];
    auto rhs = [&](int j) -> double {
        const int i = j + 1;
        if (i == 1)
            return dri * (0.533333333 * th[GIX(0, k, ld)] - 3.6 * th[GIX(1, k, ld)] +
                          2.966666667 * th[GIX(2, k, ld)] + 0.1 * th[GIX(4, k, ld)]);
        if (i == nr)
            return dri * (-0.1 * th[GIX(nr - 3, k, ld)] - 2.966666667 * th[GIX(nr - 1, k, ld)] +
                          3.6 * th[GIX(nr, k, ld)] - 0.533333333 * th[GIX(nr + 1, k, ld)]);
        return 3.0 * (th[GIX(i + 1, k, ld)] - th[GIX(i - 1, k, ld)]) * dri;
    };
    apply_tdma_rhs(d.fac_rT, nr, d.f[GB_F_A] + GIX(1, k, ld), 1, rhs);
}

__global__ void k_temp_deriv_r(PrbDev d) { k_temp_deriv_r_body(d, blockIdx.x); }

// thh (periodic tdma along x) -> B, one thread per row i = 1..nr (PRB:1271-1289).
__device__ __forceinline__ void k_temp_deriv_x_body(const PrbDev &d, int bidx)
{
    const int i = bidx * blockDim.x + threadIdx.x + 1;
    if (i > d.nr || *d.abort) return;
    const int ld = d.ld, np = d.np;
    const double dpi = d.dpi;
    const double *th = d.f[GB_F_th];
    auto rhs = [&](int k) -> double {
        if (k == np || k == 0) return 3.0 * (th[GIX(i, 1, ld)] - th[GIX(i, np - 1, ld)]) * dpi;
        return 3.0 * (th[GIX(i, k + 1, ld)] - th[GIX(i, k - 1, ld)]) * dpi;
    };
    apply_ptdma_rhs(d.fac_x, np + 1, d.f[GB_F_B] + GIX(i, 0, ld), ld, rhs);
}

__global__ void k_temp_deriv_x(PrbDev d) { k_temp_deriv_x_body(d, blockIdx.x); }

// Temperature update, PRB:1142-1207 (first) / PRB:1292-1377 (Dufort-Frankel).
// Annulus (velvor2dnewsch3.4.f:1140-1223 / :1308-1393): cell-centre radius
// r = r0 + (i-1/2) dr and the thra/r term.
__device__ __forceinline__ void k_temp_update_body(const PrbDev &d, int first, int bidx)
{
    const int t = bidx * blockDim.x + threadIdx.x;
    const int nr = d.nr;
    if (t >= nr * (d.np + 1) || *d.abort) return;
    const int i = t % nr + 1, k = t / nr;
    const int ld = d.ld, np = d.np;
    const double dri = d.dri, dpi = d.dpi, dt = d.dt;
    const double *th = d.f[GB_F_th], *thp = d.f[GB_F_thp];
    const double *uel = d.f[GB_F_uel], *vel = d.f[GB_F_vel];
    const int im = i - 1;
    int km = k - 1, ka = k + 1;
    if (k == 0) km = np - 1;
    if (k == np) ka = 1;
    const double ri = d.polar ? 1.0 / (d.r0 + ((double)i - 0.5) * d.dr) : 1.0;
    const double u = (uel[GIX(i, k, ld)] + uel[GIX(im, k, ld)]) * 0.5;
    const double v = (vel[GIX(i, k, ld)] + vel[GIX(i, km, ld)]) * 0.5;
    double thrra, thra, cnr;
    const double thr = d.f[GB_F_A][GIX(i, k, ld)];
    if (i == 1) {
        thrra = (3.2 * th[GIX(i - 1, k, ld)] + 2.0 * th[GIX(i + 1, k, ld)] - 0.2 * th[GIX(i + 2, k, ld)]) * (dri * dri);
        thra = (-4.0 * th[GIX(i - 1, k, ld)] / 3.0 + th[GIX(i + 1, k, ld)] / 3.0) * dri;
        cnr = -2.5 * (dri * dri) + 0.5 * dri * ri;
    } else if (i == nr) {
        thrra = (3.2 * th[GIX(i + 1, k, ld)] + 2.0 * th[GIX(i - 1, k, ld)] - 0.2 * th[GIX(i - 2, k, ld)]) * (dri * dri);
        thra = (-th[GIX(i - 1, k, ld)] / 3.0 + 4.0 * th[GIX(i + 1, k, ld)] / 3.0) * dri;
        cnr = -2.5 * (dri * dri) - 0.5 * dri * ri;
    } else {
        thrra = (th[GIX(i - 1, k, ld)] + th[GIX(i + 1, k, ld)]) * (dri * dri);
        thra = (th[GIX(i + 1, k, ld)] - th[GIX(i - 1, k, ld)]) * 0.5 * dri;
        cnr = -1.0 * (dri * dri);
    }
    const double thhha = (th[GIX(i, ka, ld)] + th[GIX(i, km, ld)]) * (dpi * dpi);
    const double thh = d.f[GB_F_B][GIX(i, k, ld)];
    const double cnp = -(1.0 * (dpi * dpi)) * (ri * ri);
    double RHS1, cf1;
    if (d.polar) {
        if (first) {
            RHS1 = thrra + thra * ri + thhha * (ri * ri) + th[GIX(i, k, ld)] / dt;
            cf1 = 1.0 / dt - cnr - cnp;
        } else {
            RHS1 = thrra + thra * ri + thhha * (ri * ri) + 0.5 * thp[GIX(i, k, ld)] / dt;
            cf1 = 0.5 / dt - cnr - cnp;
        }
    } else if (first) {
        RHS1 = thrra + thhha * (ri * ri) + th[GIX(i, k, ld)] / dt;
        cf1 = 1.0 / dt - cnr - cnp;
    } else {
        RHS1 = thrra + thhha * (ri * ri) + 0.5 * thp[GIX(i, k, ld)] / dt;
        cf1 = 0.5 / dt - cnr - cnp;
    }
    const double ULT = u * thr + v * thh * ri;
    const double cf2 = cnr + cnp;
    const double tn = (cf2 * thp[GIX(i, k, ld)] - ULT + RHS1) / cf1;
    d.f[GB_F_thn][GIX(i, k, ld)] = tn;
    if (!first) d.f[GB_F_Ap][GIX(i, k, ld)] = tn;
}

__global__ void k_temp_update(PrbDev d, int first) { k_temp_update_body(d, first, blockIdx.x); }

// Wall heat fluxes, PRB:1452-1500.  The per-column five-point derivatives are
// formed in parallel; one thread then sums them in the reference's order.
__device__ __forceinline__ void k_heat_body(const PrbDev &d, int k0, int k1, int bidx)
{
    extern __shared__ double sh[];
    if (*d.abort) return;
    const int ld = d.ld, nr = d.nr, np = d.np;
    const double dri = d.dri, dp = d.dp;
    const double *th = d.f[GB_F_th];
    double *P0 = sh, *P1 = sh + (np + 1);
    for (int k = threadIdx.x; k <= np; k += blockDim.x) {
        P0[k] = 0.5 * dp * (-3.35238095 * th[GIX(0, k, ld)] + 4.375 * th[GIX(1, k, ld)] -
                            1.45833333 * th[GIX(2, k, ld)] + 0.525 * th[GIX(3, k, ld)] -
                            0.08928571 * th[GIX(4, k, ld)]) * dri;
        P1[k] = 0.5 * dp * (-3.35238095 * th[GIX(nr + 1, k, ld)] + 4.375 * th[GIX(nr, k, ld)] -
                            1.45833333 * th[GIX(nr - 1, k, ld)] + 0.525 * th[GIX(nr - 2, k, ld)] -
                            0.08928571 * th[GIX(nr - 3, k, ld)]) * dri;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t1 = 0.0, t2 = 0.0;
        for (int k = k0; k <= k1; ++k) {
            const int ka = (k == np) ? 1 : k + 1;
            t1 = t1 + P0[k] + P0[ka];
            t2 = t2 + P1[k] + P1[ka];
        }
        d.heat[0] = t1;
        d.heat[1] = t2;
    }
}

__global__ void k_heat(PrbDev d, int k0, int k1) { k_heat_body(d, k0, k1, blockIdx.x); }

// rhsv (PRB:1629-1676) and rhsu (PRB:1679-1721) in one pass; the annulus
// adds the Cn/r terms of velvor2dnewsch3.4.f:1666-1686 and divides the u
// source by the face radius (:1714-1730).
__device__ __forceinline__ void k_rhs_body(const PrbDev &d, int do_v, int do_u, int bidx)
{
    const int t = bidx * blockDim.x + threadIdx.x;
    const int nr = d.nr, np = d.np, ld = d.ld;
    if (t >= nr * (np + 1) || *d.abort) return;
    const int i = t % nr + 1, k = t / nr;
    const double *Cn = d.f[GB_F_Cn];
    if (do_v) {
        const double Cr = (Cn[GIX(i, k, ld)] - Cn[GIX(i - 1, k, ld)]) / d.dr;
        double v;
        if (d.polar) {
            const double r = d.r0 + ((double)i - 0.5) * d.dr;
            if (i == 1) v = Cn[GIX(1, k, ld)] / d.dr + Cn[GIX(1, k, ld)] / r;
            else if (i == nr) {
                v = -Cn[GIX(nr - 1, k, ld)] / d.dr + Cn[GIX(nr - 1, k, ld)] / r;
                if (d.taycou) {
                    // the moving wall's term, velvor2dtaycouheat.f:1668-1670
                    const double velo = d.velo, rvali = 1.0 / d.rmax, hri = 1.0 / d.dr;
                    const double hhri = hri * hri;
                    v = v - 8.0 / 15.0 * velo * hhri + rvali * hri * velo - 4.0 / 3.0 * velo * hri * rvali +
                        velo * (rvali * rvali);
                }
            }
            else v = Cr + (Cn[GIX(i, k, ld)] + Cn[GIX(i - 1, k, ld)]) / r;
        } else if (i == 1) v = Cn[GIX(1, k, ld)] / d.dr;
        else if (i == nr) v = -Cn[GIX(nr - 1, k, ld)] / d.dr;
        else v = Cr;
        d.f[GB_F_vrh][GIX(i, k, ld)] = v;
    }
    if (do_u && i <= nr - 1) {
        const int km = (k == 0) ? np - 1 : k - 1;
        const double r = d.polar ? d.r0 + (double)i * d.dr : 1.0;
        const double Ch = (Cn[GIX(i, k, ld)] - Cn[GIX(i, km, ld)]) / d.dp;
        d.f[GB_F_urh][GIX(i, k, ld)] = -Ch / r;
    }
}

__global__ void k_rhs(PrbDev d, int do_v, int do_u) { k_rhs_body(d, do_v, do_u, blockIdx.x); }

// update, PRB:1557-1626.  Each thread owns one (i,k) of rows 0..nr+1; the
// wall values it writes are only read back by the same thread.
// Warp maximum of the CFL candidates (non-negative, never NaN), one atomic
// per warp into the step's history slot (zeroed when the run began).
__device__ __forceinline__ void prb_cfl_reduce(const PrbDev &d, double cu, double cv)
{
    for (int o = 16; o > 0; o >>= 1) {
        cu = fmax(cu, __shfl_xor_sync(0xffffffffu, cu, o));
        cv = fmax(cv, __shfl_xor_sync(0xffffffffu, cv, o));
    }
    const int s = *d.step_index;
    if ((threadIdx.x & 31) == 0 && s < d.hist_cap) {
        if (cu > 0.0) atomicMax(&d.cfl_hist[2 * s + 0], (unsigned long long)__double_as_longlong(cu));
        if (cv > 0.0) atomicMax(&d.cfl_hist[2 * s + 1], (unsigned long long)__double_as_longlong(cv));
    }
}

// The diagnostics of point (i, k) = c after the step's update: at kt >= 2
// the running means m = (1/(kt-1)) m (kt-2) + (1/(kt-1)) x of T^2, T, u^2,
// v^2, and the point's candidates for the CFL maxima (PRB:404-459).
__device__ __forceinline__ void prb_diag_point(const PrbDev &d, int i, size_t c, double tn, double u, double v,
                                               double &cu, double &cv)
{
    const int kt = *d.diag_kt;
    if (kt < 2) return;
    const size_t n = d.diag_stride;
    double *mT2 = d.diag, *mT = d.diag + n, *mU2 = d.diag + 2 * n, *mV2 = d.diag + 3 * n;
    const double tkti = 1.0 / (double)(kt - 1), w = (double)(kt - 2);
    mT2[c] = tkti * mT2[c] * w + tkti * (tn * tn);
    mT[c] = tkti * mT[c] * w + tkti * tn;
    mU2[c] = tkti * mU2[c] * w + tkti * (u * u);
    mV2[c] = tkti * mV2[c] * w + tkti * (v * v);
    if (i >= 1 && i <= d.nr) {
        const double x = fabs(u * d.dt / d.dr);
        if (x > cu) cu = x;
    }
    if (i >= 1 && i <= d.nr - 1) {
        const double r = d.polar ? d.r0 + ((double)i - 0.5) * d.dr : 1.0;
        const double x = fabs(v * d.dt / (r * d.dp));
        if (x > cv) cv = x;
    }
}

//
// DIAG: the time loop's diagnostics of the step, fused (PRB:404-459,
// velvor2dnewsch3.4.f:404-459): at kt >= 2 the running means
// m = (1/(kt-1)) m (kt-2) + (1/(kt-1)) x of T^2, T, u^2, v^2 at every point,
// and the step's CFL maxima max |u dt/dr| (rows 1..nr) and max |v dt/(r dp)|
// (rows 1..nr-1; r = 1 in the layer, r0 + (i - 1/2) dr in the annulus) into
// the step's history slot.  A NaN never wins the reference's comparison.
template <bool DIAG>
__device__ __forceinline__ void k_update_body(const PrbDev &d, int bidx)
{
    const int t = bidx * blockDim.x + threadIdx.x;
    const int nr = d.nr, np = d.np, ld = d.ld;
    if (*d.abort) return;   // uniform across the grid
    double cu = 0.0, cv = 0.0;
    if (t < (nr + 2) * (np + 1)) {
        const int i = t % (nr + 2), k = t / (nr + 2);
        double *const *f = d.f;
        const double dr = d.dr;
        const size_t c = GIX(i, k, ld);
        if (i == 0) {
            f[GB_F_Bn][c] = -(3.0 * f[GB_F_wel][GIX(1, k, ld)] - f[GB_F_wel][GIX(2, k, ld)] / 3.0) / dr;
            f[GB_F_Cn][c] = (3.0 * f[GB_F_vel][GIX(1, k, ld)] - f[GB_F_vel][GIX(2, k, ld)] / 3.0) / dr;
            f[GB_F_thn][c] = 0.0;
        } else if (i == nr) {
            f[GB_F_Bn][c] = -(f[GB_F_wel][GIX(nr - 1, k, ld)] / 3.0 - 3.0 * f[GB_F_wel][GIX(nr, k, ld)]) / dr;
            if (d.taycou)
                // velvor2dtaycouheat.f:1587-1590; v(nr+1) is the wall speed the
                // i = nr+1 thread stores
                f[GB_F_Cn][c] = (8.0 / 3.0 * d.velo + f[GB_F_vel][GIX(nr - 1, k, ld)] / 3.0 -
                                 3.0 * f[GB_F_vel][GIX(nr, k, ld)]) / dr + d.velo / d.rmax;
            else
                f[GB_F_Cn][c] = (f[GB_F_vel][GIX(nr - 1, k, ld)] / 3.0 - 3.0 * f[GB_F_vel][GIX(nr, k, ld)]) / dr;
        } else if (i == nr + 1) {
            f[GB_F_thn][c] = 1.0;
            if (d.taycou) f[GB_F_vel][c] = d.velo;
        }
        f[GB_F_Cp][c] = f[GB_F_C][c];
        f[GB_F_C][c] = f[GB_F_Cn][c];
        f[GB_F_thp][c] = f[GB_F_th][c];
        double tn = f[GB_F_thn][c];
        unsigned long long clamped = 0;
        if (tn > 1.0) { tn = 0.99; clamped++; }
        if (tn < 0.0) { tn = 0.01; clamped++; }
        f[GB_F_thn][c] = tn;
        f[GB_F_th][c] = tn;
        if (clamped) atomicAdd(d.clamps, clamped);
        if (DIAG) prb_diag_point(d, i, c, tn, f[GB_F_uel][c], f[GB_F_vel][c], cu, cv);
    }
    if (DIAG) prb_cfl_reduce(d, cu, cv);   // every lane of every warp
}

template <bool DIAG>
__global__ void k_update(PrbDev d) { k_update_body<DIAG>(d, blockIdx.x); }

// The diagnostics alone, after the tank's and the cavity's update: the same
// running means and CFL scans over the same rows and columns k = 0..np
// (velvor2dhorconvtank.f:424-479, velvor2ddvdbenchmark.f:434-486).
__global__ void k_prb_diag(PrbDev d)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (*d.abort) return;   // uniform across the grid
    double cu = 0.0, cv = 0.0;
    if (t < (d.nr + 2) * (d.np + 1)) {
        const int i = t % (d.nr + 2), k = t / (d.nr + 2);
        const size_t c = GIX(i, k, d.ld);
        prb_diag_point(d, i, c, d.f[GB_F_th][c], d.f[GB_F_uel][c], d.f[GB_F_vel][c], cu, cv);
    }
    prb_cfl_reduce(d, cu, cv);
}

// Per-step bookkeeping for graph-replayed steps: copies the step's Nusselt
// numbers and sweep counts into the history slot given by *d.step_index.
// Nu = heat * c / div: c = rmax - r0, div = xx in PRB (PRB:386-388);
// c = -r0 ln(r0/rmax) (inner) and -rmax ln(r0/rmax) (outer), div = 2 pi in
// the annulus (velvor2dnewsch3.4.f:386-387).
// swap: the tank's first step stores 2 trans2 in httrans and leaves httrans2
// at zero (velvor2dhorconvtank.f:197-198).
__device__ __forceinline__ void k_record_body(const PrbDev &d, double c1, double c2, double div, int swap, int bidx)
{
    if (threadIdx.x != 0 || bidx != 0) return;
    const int s = *d.step_index;
    if (s < d.hist_cap) {
        d.nu_hist[2 * s + 0] = swap ? d.heat[1] * c2 / div : d.heat[0] * c1 / div;
        d.nu_hist[2 * s + 1] = swap ? 0.0 : d.heat[1] * c2 / div;
        d.sweep_hist[2 * s + 0] = d.mg_status[1];
        d.sweep_hist[2 * s + 1] = d.mg_status[3];
    }
    if (!*d.abort) {
        *d.step_index = s + 1;
        if (d.diag_kt) *d.diag_kt += 1;
    }
}

__global__ void k_record(PrbDev d, double c1, double c2, double div, int swap) { k_record_body(d, c1, c2, div, swap, blockIdx.x); }

__global__ void k_prb_set_kt(int *kt, int value) { *kt = value; }

// Zonal means of the running means, one thread per row i = 0..nr+1, summed
// over k = 0..np in order (PRB:474-493): out[3 i + 0] the zonal-mean time
// variance of T, out[3 i + 1..2] the zonal rms of u and v.  The reference
// evaluates **0.5d0 through libm's pow; sqrt here (correctly rounded; the two
// agree to an ulp).
__global__ void k_prb_zonal(PrbDev d, double *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > d.nr + 1) return;
    const int ld = d.ld, np = d.np;
    const size_t n = d.diag_stride;
    const double *mT2 = d.diag, *mT = d.diag + n, *mU2 = d.diag + 2 * n, *mV2 = d.diag + 3 * n;
    double a = 0.0, b = 0.0, cu = 0.0, cv = 0.0;
    for (int k = 0; k <= np; ++k) {
        const size_t c = GIX(i, k, ld);
        a = a + mT2[c];
        b = b + mT[c] * mT[c];
        cu = cu + mU2[c];
        cv = cv + mV2[c];
    }
    const double m = (double)(np + 1);
    out[3 * i + 0] = (a - b) / m;
    out[3 * i + 1] = sqrt(cu / m);
    out[3 * i + 2] = sqrt(cv / m);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static const int TPB = 256;

int prb_launch_cvorticity(gb_prb *h, int first, cudaStream_t s)
{
    if (h->dev.tank) return tank_launch_cvorticity(h, first, s);
    PrbDev &d = h->dev;
    k_cvort_deriv_r<<<gb_ceil_div(d.np + 1, 64), 64, 0, s>>>(d);
    k_cvort_deriv_x<<<gb_ceil_div(d.nr - 1, 64), 64, 0, s>>>(d);
    k_cvort_update<<<gb_ceil_div((size_t)(d.nr - 1) * (d.np + 1), TPB), TPB, 0, s>>>(d, first);
    if (!first)
        k_robert<<<gb_ceil_div((size_t)(d.nr - 1) * (d.np + 1), TPB), TPB, 0, s>>>(d, GB_F_C, GB_F_Cn, GB_F_Cp, d.nr - 1);
    h->launches += first ? 3 : 4;
    return GB_OK;
}

int prb_launch_temperature(gb_prb *h, int first, cudaStream_t s)
{
    if (h->dev.tank) return tank_launch_temperature(h, first, s);
    PrbDev &d = h->dev;
    k_temp_deriv_r<<<gb_ceil_div(d.np + 1, 64), 64, 0, s>>>(d);
    k_temp_deriv_x<<<gb_ceil_div(d.nr, 64), 64, 0, s>>>(d);
    k_temp_update<<<gb_ceil_div((size_t)d.nr * (d.np + 1), TPB), TPB, 0, s>>>(d, first);
    if (!first)
        k_robert<<<gb_ceil_div((size_t)d.nr * (d.np + 1), TPB), TPB, 0, s>>>(d, GB_F_th, GB_F_thn, GB_F_thp, d.nr);
    h->launches += first ? 3 : 4;
    return GB_OK;
}

int prb_launch_heat(gb_prb *h, cudaStream_t s)
{
    PrbDev &d = h->dev;
    // the tank integrates over k = np/2..np-1 (velvor2dhorconvtank.f:778)
    if (d.tank) k_heat<<<1, 256, 2 * (d.np + 1) * sizeof(double), s>>>(d, d.dvd ? 2 : d.np / 2, d.np - 1);
    else k_heat<<<1, 256, 2 * (d.np + 1) * sizeof(double), s>>>(d, 1, d.np);
    h->launches += 1;
    return GB_OK;
}

int prb_launch_rhs(gb_prb *h, int do_v, int do_u, cudaStream_t s)
{
    if (h->dev.tank) return tank_launch_rhs(h, do_v, do_u, s);
    PrbDev &d = h->dev;
    k_rhs<<<gb_ceil_div((size_t)d.nr * (d.np + 1), TPB), TPB, 0, s>>>(d, do_v, do_u);
    h->launches += 1;
    return GB_OK;
}

int prb_launch_update(gb_prb *h, cudaStream_t s, bool diag)
{
    PrbDev &d = h->dev;
    if (d.tank) {
        const int st = tank_launch_update(h, s);
        if (st != GB_OK || !(diag && d.diag)) return st;
        k_prb_diag<<<gb_ceil_div((size_t)(d.nr + 2) * (d.np + 1), TPB), TPB, 0, s>>>(d);
        h->launches += 1;
        return GB_OK;
    }
    if (diag && d.diag)
        k_update<true><<<gb_ceil_div((size_t)(d.nr + 2) * (d.np + 1), TPB), TPB, 0, s>>>(d);
    else
        k_update<false><<<gb_ceil_div((size_t)(d.nr + 2) * (d.np + 1), TPB), TPB, 0, s>>>(d);
    h->launches += 1;
    return GB_OK;
}

int prb_launch_record(gb_prb *h, cudaStream_t s, int first)
{
    double c1 = h->p.rmax - h->p.r0, c2 = c1, div = h->p.xx;
    if (h->p.variant == GB_PRB_TANK || h->p.variant == GB_PRB_DVD) {
        // httrans = 2 trans (velvor2dhorconvtank.f:209-210), trans in the cavity
        c1 = c2 = h->p.variant == GB_PRB_DVD ? 1.0 : 2.0;
        div = 1.0;
    }
    if (h->p.variant == GB_PRB_ANNULUS || h->p.variant == GB_PRB_TAYCOU) {
        const double L = log(h->p.r0 / h->p.rmax);
        c1 = -h->p.r0 * L;
        c2 = -h->p.rmax * L;
        div = 2.0 * acos(-1.0);
    }
    k_record<<<1, 32, 0, s>>>(h->dev, c1, c2, div, (h->dev.tank && first) ? 1 : 0);
    h->launches += 1;
    return GB_OK;
}

extern "C" void gb_prb_default_params(gb_prb_params *p, int nr, int np)
{
    memset(p, 0, sizeof(*p));
    p->nr = nr;
    p->np = np;
    p->dt = 1e-7;
    p->r0 = 0.5;
    p->rmax = 1.0;
    p->xx = 3.0;
    p->Ra = 1e7;
    p->Pr = 0.71;
    p->tolcon = 2e-6;
    p->sor = 1.2;
    p->maxsweeps = 500;
    p->smoother = GB_SMOOTHER_LEX;
    p->variant = GB_PRB_LAYER;
    p->Re = 0.0;
}

extern "C" void gb_prb_default_params_annulus(gb_prb_params *p, int nr, int np)
{
    gb_prb_default_params(p, nr, np);
    p->variant = GB_PRB_ANNULUS;
    p->dt = 2e-8;
    p->r0 = 0.5;
    p->rmax = 1.0;
    p->xx = 2.0 * acos(-1.0);
    p->Ra = 8e8;
    p->Re = 1.06148e5;
    p->Pr = 0.71;
    p->tolcon = 10e-6;
    p->maxsweeps = 10000;
}

extern "C" void gb_prb_default_params_tank(gb_prb_params *p, int nr, int np)
{
    gb_prb_default_params(p, nr, np);
    p->variant = GB_PRB_TANK;
    p->dt = 5e-8;
    p->r0 = 0.5;
    p->rmax = 1.5;
    p->xx = 3.1;
    p->Ra = 8.63e7;
    p->Pr = 10.0;
    p->tolcon = 5e-6;
    p->maxsweeps = 500;
}

extern "C" void gb_prb_default_params_dvd(gb_prb_params *p, int nr, int np)
{
    gb_prb_default_params_tank(p, nr, np);
    p->variant = GB_PRB_DVD;
    p->dt = 2e-6;
    p->r0 = 0.0;
    p->rmax = 1.0;
    p->xx = 1.0;
    p->Ra = 1e6;
    p->Pr = 0.71;
}

extern "C" void gb_prb_default_params_taycou(gb_prb_params *p, int nr, int np)
{
    gb_prb_default_params_annulus(p, nr, np);
    p->variant = GB_PRB_TAYCOU;
    p->Ra = 6e8;
    p->Re = 91927.0;
    p->Ta = 0.0;
    p->tolcon = 1e-5;
    p->maxsweeps = 500;
}

// Level count of poissoninit (PRB:1744-1767; the annulus caps at 5,
// velvor2dnewsch3.4.f:1778).
int prb_mg_levels(int nr, int variant)
{
    int nlev = 0, itest = nr, itest2 = nr;
    for (int i = 2; i <= 8; ++i) {
        itest = itest / 2;
        if (itest * 2 - itest2 == 0) {
            if (itest2 >= 4) nlev = nlev + 1;
            itest2 = itest;
        } else {
            break;
        }
    }
    if (variant == GB_PRB_ANNULUS) {
        if (nlev > 5) nlev = 5;
    } else if (nlev >= 5) {
        nlev = 4;
    }
    return nlev;
}

int prb_refresh_scalars(gb_prb *h)
{
    PrbDev &d = h->dev;
    d.dt = h->p.dt;
    d.Ra = h->p.Ra;
    d.Pr = h->p.Pr;
    d.polar = h->p.variant == GB_PRB_ANNULUS || h->p.variant == GB_PRB_TAYCOU;
    d.oblique = h->p.variant == GB_PRB_OBLIQUE;
    d.taycou = h->p.variant == GB_PRB_TAYCOU;
    d.tank = h->p.variant == GB_PRB_TANK || h->p.variant == GB_PRB_DVD;
    d.dvd = h->p.variant == GB_PRB_DVD;
    d.rmax = h->p.rmax;
    d.velo = d.taycou ? -(pow(h->p.Ta, 0.5) * h->p.Pr * 0.5 * h->p.rmax) : 0.0;
    d.robert = h->p.variant == GB_PRB_ANNULUS ? 0.05 : d.taycou ? 0.01 : 0.02;
    d.r0 = h->p.r0;
    d.Re = h->p.Re;
    d.dr = h->dr_set != 0.0 ? h->dr_set : (h->p.rmax - h->p.r0) / (double)h->p.nr;
    if (h->dp_set != 0.0) d.dp = h->dp_set;
    else if (d.polar) d.dp = 2.0 * acos(-1.0) / (double)h->p.np;   // velvor2dnewsch3.4.f:124
    else d.dp = h->p.xx / (double)h->p.np;
    d.dri = 1.0 / d.dr;
    d.dpi = 1.0 / d.dp;
    return GB_OK;
}

// dr, dp: grid spacings to use verbatim (the Fortran caller's /num/ values),
// or 0 to derive them as the reference main program does (PRB:127-133).
int gb_prb_create_ex(const gb_prb_params *p, double dr, double dp, gb_prb **out, int *nlev_out)
{
    if (!p || !out) { gb_set_error("gb_prb_create: null argument"); return GB_ERR_INVALID; }
    *out = nullptr;
    const int nr = p->nr, np = p->np;
    const int nlev = prb_mg_levels(nr, p->variant);
    if (nlev_out) *nlev_out = nlev;
    if (p->variant != GB_PRB_LAYER && p->variant != GB_PRB_ANNULUS && p->variant != GB_PRB_OBLIQUE &&
        p->variant != GB_PRB_TAYCOU && p->variant != GB_PRB_TANK && p->variant != GB_PRB_DVD) {
        gb_set_error("gb_prb_create: unknown variant %d", p->variant);
        return GB_ERR_INVALID;
    }
    if ((p->variant == GB_PRB_ANNULUS || p->variant == GB_PRB_TAYCOU) &&
        !(p->r0 > 0.0 && p->rmax > p->r0 && p->Re != 0.0 && p->Ta >= 0.0)) {
        gb_set_error("gb_prb_create: the annulus needs 0 < r0 < rmax and Re != 0 (r0=%g rmax=%g Re=%g)", p->r0, p->rmax, p->Re);
        return GB_ERR_INVALID;
    }
    if ((p->variant == GB_PRB_TANK || p->variant == GB_PRB_DVD) && p->precision != GB_PRB_FP64) {
        gb_set_error("gb_prb_create: the tank and the cavity run in FP64 only");
        return GB_ERR_INVALID;
    }
    if (nr < 4 || np < 4 || (np & 1) || nlev < 1 || nr > 8192 || np > 65536) {
        gb_set_error("gb_prb_create: unsupported grid nr=%d np=%d (need even nr >= 4 with >= 1 multigrid level, even np >= 4)", nr, np);
        return GB_ERR_INVALID;
    }
    gb_prb *h = new gb_prb();
    h->p = *p;
    h->nlev = nlev;
    PrbDev &d = h->dev;
    d.nr = nr;
    d.np = np;
    d.ld = nr + 2;
    // the tank's and the cavity's T and u ghost column np+1
    h->ncol = (p->variant == GB_PRB_TANK || p->variant == GB_PRB_DVD) ? np + 2 : np + 1;
    h->fsz = (size_t)d.ld * (size_t)h->ncol;
    h->dr_set = dr;
    h->dp_set = dp;
    prb_refresh_scalars(h);
    cudaError_t e = cudaMalloc(&h->fields, sizeof(double) * h->fsz * GB_F_COUNT);
    if (e != cudaSuccess) { gb_set_error("gb_prb_create: %s", cudaGetErrorString(e)); delete h; return GB_ERR_ALLOC; }
    cudaMemset(h->fields, 0, sizeof(double) * h->fsz * GB_F_COUNT);
    for (int f = 0; f < GB_F_COUNT; ++f) d.f[f] = h->fields + (size_t)f * h->fsz;
    // factors + small device state
    const size_t nwork = 3 * ((size_t)(nr > np ? nr : np) + 2);
    const size_t nfac = tdma_fac_len(nr) + ptdma_fac_len(np + 1) + tdma_fac_len(nr) + nwork + 2 * tdma_fac_len(np + 1);
    e = cudaMalloc(&h->factors, sizeof(double) * nfac);
    if (e != cudaSuccess) { gb_prb_destroy(h); gb_set_error("gb_prb_create: factor alloc"); return GB_ERR_ALLOC; }
    double *fr1 = h->factors;
    double *fx = fr1 + tdma_fac_len(nr);
    double *frT = fx + ptdma_fac_len(np + 1);
    double *work = frT + tdma_fac_len(nr);
    double *fxw1 = work + nwork;
    double *fxw2 = fxw1 + tdma_fac_len(np + 1);
    d.fac_r1 = fr1;
    d.fac_x = fx;
    d.fac_rT = frT;
    d.fac_xw1 = fxw1;
    d.fac_xw2 = fxw2;
    k_transport_factors<<<1, 1>>>(nr, np, fr1, fx, frT, work, d.tank ? fxw1 : nullptr, fxw2);
    e = cudaMalloc(&h->small, 4096);
    if (e != cudaSuccess) { gb_prb_destroy(h); gb_set_error("gb_prb_create: small alloc"); return GB_ERR_ALLOC; }
    cudaMemset(h->small, 0, 4096);
    char *sm = (char *)h->small;
    d.heat = (double *)(sm + 0);
    d.clamps = (unsigned long long *)(sm + 64);
    d.abort = (int *)(sm + 128);
    d.step_index = (int *)(sm + 192);
    d.mg_status = (int *)(sm + 256);  // [status_v, sweeps_v, status_u, sweeps_u]
    d.mg_resmax = (double *)(sm + 320);
    d.nu_hist = nullptr;
    d.sweep_hist = nullptr;
    d.hist_cap = 0;
    int st = prb_mg_create(h);
    if (st != GB_OK) { gb_prb_destroy(h); return st; }
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { gb_prb_destroy(h); gb_set_error("gb_prb_create: stream"); return GB_ERR_CUDA; }
    e = cudaStreamSynchronize(0);   // the creation's kernels and copies, not other instances' streams
    if (e != cudaSuccess) { gb_set_error("gb_prb_create: %s", cudaGetErrorString(e)); gb_prb_destroy(h); return GB_ERR_CUDA; }
    *out = h;
    return GB_OK;
}

extern "C" int gb_prb_create(const gb_prb_params *p, gb_prb **out, int *nlev_out)
{
    return gb_prb_create_ex(p, 0.0, 0.0, out, nlev_out);
}

extern "C" int gb_prb_destroy(gb_prb *h)
{
    if (!h) return GB_OK;
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->graph_exec1) cudaGraphExecDestroy(h->graph_exec1);
    prb_mg_destroy(h);
    cudaFree(h->fields);
    cudaFree(h->factors);
    cudaFree(h->small);
    cudaFree(h->hist);
    cudaFree(h->diag_buf);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return GB_OK;
}

extern "C" int gb_prb_set_field(gb_prb *h, int field, const double *host, int ld)
{
    if (!h || !host || field < 0 || field >= GB_F_COUNT || ld < h->dev.nr + 2) {
        gb_set_error("gb_prb_set_field: invalid argument");
        return GB_ERR_INVALID;
    }
    GB_CUDA_TRY(cudaMemcpy2DAsync(h->dev.f[field], sizeof(double) * h->dev.ld, host, sizeof(double) * (size_t)ld,
                                  sizeof(double) * (h->dev.nr + 2), h->ncol, cudaMemcpyHostToDevice, h->stream));
    GB_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return GB_OK;
}

extern "C" int gb_prb_get_field(gb_prb *h, int field, double *host, int ld)
{
    if (!h || !host || field < 0 || field >= GB_F_COUNT || ld < h->dev.nr + 2) {
        gb_set_error("gb_prb_get_field: invalid argument");
        return GB_ERR_INVALID;
    }
    GB_CUDA_TRY(cudaMemcpy2DAsync(host, sizeof(double) * (size_t)ld, h->dev.f[field], sizeof(double) * h->dev.ld,
                                  sizeof(double) * (h->dev.nr + 2), h->ncol, cudaMemcpyDeviceToHost, h->stream));
    GB_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return GB_OK;
}

extern "C" int gb_prb_field_device_ptr(gb_prb *h, int field, double **dev, int *ld)
{
    if (!h || field < 0 || field >= GB_F_COUNT) { gb_set_error("gb_prb_field_device_ptr: invalid argument"); return GB_ERR_INVALID; }
    if (dev) *dev = h->dev.f[field];
    if (ld) *ld = h->dev.ld;
    return GB_OK;
}

// Clears the step-abort flag so that an earlier failed solve does not make
// the kernels of an individual routine call skip their work.
static void prb_begin(gb_prb *h)
{
    prb_refresh_scalars(h);
    cudaMemsetAsync(h->dev.abort, 0, sizeof(int), h->stream);
}

static int prb_sync(gb_prb *h, const char *what)
{
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) { gb_set_error("%s: %s", what, cudaGetErrorString(e)); return GB_ERR_CUDA; }
    e = cudaGetLastError();
    if (e != cudaSuccess) { gb_set_error("%s: %s", what, cudaGetErrorString(e)); return GB_ERR_CUDA; }
    return GB_OK;
}

extern "C" int gb_prb_cvorticity(gb_prb *h, int first)
{
    if (!h) return GB_ERR_INVALID;
    prb_begin(h);
    prb_launch_cvorticity(h, first, h->stream);
    return prb_sync(h, "gb_prb_cvorticity");
}

extern "C" int gb_prb_temperature(gb_prb *h, int first)
{
    if (!h) return GB_ERR_INVALID;
    prb_begin(h);
    prb_launch_temperature(h, first, h->stream);
    return prb_sync(h, "gb_prb_temperature");
}

extern "C" int gb_prb_heat(gb_prb *h, double *trans1, double *trans2)
{
    if (!h) return GB_ERR_INVALID;
    prb_begin(h);
    prb_launch_heat(h, h->stream);
    double t[2];
    GB_CUDA_TRY(cudaMemcpyAsync(t, h->dev.heat, sizeof(t), cudaMemcpyDeviceToHost, h->stream));
    int st = prb_sync(h, "gb_prb_heat");
    if (st != GB_OK) return st;
    if (trans1) *trans1 = t[0];
    if (trans2) *trans2 = t[1];
    return GB_OK;
}

extern "C" int gb_prb_rhsv(gb_prb *h)
{
    if (!h) return GB_ERR_INVALID;
    prb_begin(h);
    prb_launch_rhs(h, 1, 0, h->stream);
    return prb_sync(h, "gb_prb_rhsv");
}

extern "C" int gb_prb_rhsu(gb_prb *h)
{
    if (!h) return GB_ERR_INVALID;
    prb_begin(h);
    prb_launch_rhs(h, 0, 1, h->stream);
    return prb_sync(h, "gb_prb_rhsu");
}

extern "C" int gb_prb_update(gb_prb *h, long long *clamps)
{
    if (!h) return GB_ERR_INVALID;
    prb_begin(h);
    GB_CUDA_TRY(cudaMemsetAsync(h->dev.clamps, 0, sizeof(unsigned long long), h->stream));
    prb_launch_update(h, h->stream, false);
    unsigned long long c = 0;
    GB_CUDA_TRY(cudaMemcpyAsync(&c, h->dev.clamps, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    int st = prb_sync(h, "gb_prb_update");
    if (clamps) *clamps = (long long)c;
    return st;
}

extern "C" int gb_prb_poisson(gb_prb *h, int which, int *sweeps)
{
    if (!h || (which != 2 && which != 3)) { gb_set_error("gb_prb_poisson: which must be 2 or 3"); return GB_ERR_INVALID; }
    prb_begin(h);
    prb_launch_mg(h, which == 2 ? 1 : 0, which == 3 ? 1 : 0, h->stream);
    int stat[4];
    GB_CUDA_TRY(cudaMemcpyAsync(stat, h->dev.mg_status, sizeof(stat), cudaMemcpyDeviceToHost, h->stream));
    int st = prb_sync(h, "gb_prb_poisson");
    if (st != GB_OK) return st;
    const int o = (which == 2) ? 0 : 2;
    if (sweeps) *sweeps = stat[o + 1];
    return stat[o];
}

// One step's launches on stream s (v and u solves in one multigrid launch).
static void prb_enqueue_step(gb_prb *h, int first, cudaStream_t s)
{
    prb_launch_cvorticity(h, first, s);
    prb_launch_temperature(h, first, s);
    prb_launch_heat(h, s);
    prb_launch_rhs(h, 1, 1, s);
    prb_launch_mg(h, 1, 1, s);
    prb_launch_update(h, s, true);
    prb_launch_record(h, s, first);
}

static int prb_build_graph(gb_prb *h, int first, cudaGraphExec_t *exec)
{
    cudaGraph_t g;
    GB_CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const long long l0 = h->launches;
    prb_enqueue_step(h, first, h->stream);
    h->launches_per_step = h->launches - l0;
    h->launches = l0;
    GB_CUDA_TRY(cudaStreamEndCapture(h->stream, &g));
    GB_CUDA_TRY(cudaGraphInstantiate(exec, g, 0));
    cudaGraphDestroy(g);
    return GB_OK;
}

static int prb_diag_alloc(gb_prb *h, int cap);

// Asynchronous stepping: run_begin sizes the history and resets the step
// counters, run_enqueue queues graph launches on the instance's stream
// without waiting, run_query polls it, run_end waits and collects.
extern "C" int gb_prb_run_begin(gb_prb *h, int nsteps_total)
{
    if (!h || nsteps_total < 0) { gb_set_error("gb_prb_run_begin: invalid argument"); return GB_ERR_INVALID; }
    prb_refresh_scalars(h);
    PrbDev &d = h->dev;
    const int cap = nsteps_total > 0 ? nsteps_total : 1;
    if (h->hist_cap < cap) {
        cudaFree(h->hist);
        h->hist = nullptr;
        GB_CUDA_TRY(cudaMalloc(&h->hist, (sizeof(double) * 2 + sizeof(int) * 2) * (size_t)cap));
        h->hist_cap = cap;
        if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; }
        if (h->graph_exec1) { cudaGraphExecDestroy(h->graph_exec1); h->graph_exec1 = nullptr; }
    }
    d.nu_hist = (double *)h->hist;
    d.sweep_hist = (int *)((double *)h->hist + 2 * (size_t)h->hist_cap);
    d.hist_cap = h->hist_cap;
    if (h->diag_buf) {
        if (h->diag_cap < h->hist_cap) {
            int st = prb_diag_alloc(h, h->hist_cap);
            if (st != GB_OK) return st;
        }
        GB_CUDA_TRY(cudaMemsetAsync(d.cfl_hist, 0, sizeof(unsigned long long) * 2 * (size_t)h->hist_cap, h->stream));
    }
    // scalars are baked into the graphs: rebuild when they change
    if (memcmp(&h->graph_scalars, &h->p, sizeof(gb_prb_params)) != 0) {
        if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; }
        if (h->graph_exec1) { cudaGraphExecDestroy(h->graph_exec1); h->graph_exec1 = nullptr; }
        h->graph_scalars = h->p;
    }
    GB_CUDA_TRY(cudaMemsetAsync(d.abort, 0, sizeof(int), h->stream));
    GB_CUDA_TRY(cudaMemsetAsync(d.step_index, 0, sizeof(int), h->stream));
    GB_CUDA_TRY(cudaMemsetAsync(d.clamps, 0, sizeof(unsigned long long), h->stream));
    return GB_OK;
}

extern "C" int gb_prb_run_enqueue(gb_prb *h, int kt0, int nsteps)
{
    if (!h || nsteps < 0 || kt0 < 1) { gb_set_error("gb_prb_run_enqueue: invalid argument"); return GB_ERR_INVALID; }
    int st;
    if (h->dev.diag && nsteps > 0) {
        k_prb_set_kt<<<1, 1, 0, h->stream>>>(h->dev.diag_kt, kt0);
        h->launches += 1;
    }
    for (int s = 0; s < nsteps; ++s) {
        const int first = (kt0 + s == 1);
        cudaGraphExec_t *ex = first ? &h->graph_exec1 : &h->graph_exec;
        if (!*ex && (st = prb_build_graph(h, first, ex)) != GB_OK) return st;
        GB_CUDA_TRY(cudaGraphLaunch(*ex, h->stream));
        h->launches += h->launches_per_step;
    }
    return GB_OK;
}

extern "C" int gb_prb_run_query(gb_prb *h)
{
    if (!h) return -GB_ERR_INVALID;
    const cudaError_t e = cudaStreamQuery(h->stream);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) { cudaGetLastError(); return 0; }
    gb_set_error("gb_prb_run_query: %s", cudaGetErrorString(e));
    return -GB_ERR_CUDA;
}

extern "C" int gb_prb_run_end(gb_prb *h, int nsteps, double *nu, int *sweeps, int *steps_done)
{
    if (!h || nsteps < 0 || nsteps > h->hist_cap) { gb_set_error("gb_prb_run_end: invalid argument"); return GB_ERR_INVALID; }
    PrbDev &d = h->dev;
    int info[2] = {0, 0}, stat[4] = {0, 0, 0, 0};
    GB_CUDA_TRY(cudaMemcpyAsync(info, d.step_index, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    GB_CUDA_TRY(cudaMemcpyAsync(info + 1, d.abort, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    GB_CUDA_TRY(cudaMemcpyAsync(stat, d.mg_status, sizeof(stat), cudaMemcpyDeviceToHost, h->stream));
    std::vector<double> nuh(2 * (size_t)nsteps + 1);
    std::vector<int> swh(2 * (size_t)nsteps + 1);
    if (nsteps > 0) {
        GB_CUDA_TRY(cudaMemcpyAsync(nuh.data(), d.nu_hist, sizeof(double) * 2 * nsteps, cudaMemcpyDeviceToHost, h->stream));
        GB_CUDA_TRY(cudaMemcpyAsync(swh.data(), d.sweep_hist, sizeof(int) * 2 * nsteps, cudaMemcpyDeviceToHost, h->stream));
    }
    int st = prb_sync(h, "gb_prb_run_end");
    if (st != GB_OK) return st;
    if (nu) memcpy(nu, nuh.data(), sizeof(double) * 2 * nsteps);
    if (sweeps) memcpy(sweeps, swh.data(), sizeof(int) * 2 * nsteps);
    h->steps_done = info[0];
    if (steps_done) *steps_done = info[0];
    if (info[1] && info[1] != GB_RUN_DONE) {
        gb_set_error("gb_prb_step: multigrid failed at step %d (status v=%d u=%d)", info[0] + 1, stat[0], stat[2]);
        return stat[0] != GB_OK ? stat[0] : stat[2];
    }
    return GB_OK;
}

extern "C" int gb_prb_step(gb_prb *h, int kt0, int nsteps, double *nu, int *sweeps)
{
    if (!h || nsteps < 0 || kt0 < 1) { gb_set_error("gb_prb_step: invalid argument"); return GB_ERR_INVALID; }
    if (nsteps == 0) return GB_OK;
    int st = gb_prb_run_begin(h, nsteps);
    if (st == GB_OK) st = gb_prb_run_enqueue(h, kt0, nsteps);
    if (st != GB_OK) return st;
    return gb_prb_run_end(h, nsteps, nu, sweeps, nullptr);
}

extern "C" void *gb_prb_stream(gb_prb *h) { return h ? (void *)h->stream : nullptr; }

// ---------------------------------------------------------------------------
// Time-loop diagnostics (PRB:404-493)
// ---------------------------------------------------------------------------
static void prb_drop_graphs(gb_prb *h)
{
    if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; }
    if (h->graph_exec1) { cudaGraphExecDestroy(h->graph_exec1); h->graph_exec1 = nullptr; }
}

// (Re)allocates the diagnostics buffer for `cap` history slots; the running
// means start at zero (as weln, welp and vrms do; Bp's initial value is
// multiplied by zero at the block's first step).
static int prb_diag_alloc(gb_prb *h, int cap)
{
    PrbDev &d = h->dev;
    const size_t n = h->fsz;
    const size_t bytes = sizeof(double) * 4 * n + 64 + sizeof(unsigned long long) * 2 * (size_t)cap;
    double *buf = nullptr;
    cudaError_t e = cudaMalloc(&buf, bytes);
    if (e != cudaSuccess) { gb_set_error("gb_prb_diag_enable: %s", cudaGetErrorString(e)); return GB_ERR_ALLOC; }
    cudaMemsetAsync(buf, 0, bytes, h->stream);
    if (h->diag_buf) {
        // keep the running means across a history resize
        cudaMemcpyAsync(buf, h->diag_buf, sizeof(double) * 4 * n + 64, cudaMemcpyDeviceToDevice, h->stream);
        cudaStreamSynchronize(h->stream);
        cudaFree(h->diag_buf);
    }
    h->diag_buf = buf;
    h->diag_cap = cap;
    d.diag = buf;
    d.diag_stride = n;
    d.diag_kt = (int *)(buf + 4 * n);
    d.cfl_hist = (unsigned long long *)(buf + 4 * n + 8);
    prb_drop_graphs(h);
    return GB_OK;
}

extern "C" int gb_prb_diag_enable(gb_prb *h, int on)
{
    if (!h) { gb_set_error("gb_prb_diag_enable: null handle"); return GB_ERR_INVALID; }
    PrbDev &d = h->dev;
    if (!on) {
        if (h->diag_buf) {
            GB_CUDA_TRY(cudaStreamSynchronize(h->stream));
            cudaFree(h->diag_buf);
        }
        h->diag_buf = nullptr;
        h->diag_cap = 0;
        d.diag = nullptr;
        d.diag_kt = nullptr;
        d.cfl_hist = nullptr;
        prb_drop_graphs(h);
        return GB_OK;
    }
    if (h->diag_buf) {
        // a fresh start: clear the running means
        GB_CUDA_TRY(cudaMemsetAsync(h->diag_buf, 0, sizeof(double) * 4 * h->fsz, h->stream));
        return prb_sync(h, "gb_prb_diag_enable");
    }
    int st = prb_diag_alloc(h, h->hist_cap > 0 ? h->hist_cap : 1);
    if (st != GB_OK) return st;
    return prb_sync(h, "gb_prb_diag_enable");
}

extern "C" int gb_prb_diag_zonal(gb_prb *h, double *out)
{
    if (!h || !out || !h->dev.diag) { gb_set_error("gb_prb_diag_zonal: diagnostics not enabled"); return GB_ERR_INVALID; }
    const int rows = h->dev.nr + 2;
    double *dout = nullptr;
    GB_CUDA_TRY(cudaMallocAsync(&dout, sizeof(double) * 3 * (size_t)rows, h->stream));
    k_prb_zonal<<<gb_ceil_div(rows, 64), 64, 0, h->stream>>>(h->dev, dout);
    GB_CUDA_TRY(cudaMemcpyAsync(out, dout, sizeof(double) * 3 * (size_t)rows, cudaMemcpyDeviceToHost, h->stream));
    GB_CUDA_TRY(cudaFreeAsync(dout, h->stream));
    return prb_sync(h, "gb_prb_diag_zonal");
}

extern "C" int gb_prb_diag_mean(gb_prb *h, int q, double *host, int ld)
{
    if (!h || !host || q < 0 || q > 3 || !h->dev.diag || ld < h->dev.ld) {
        gb_set_error("gb_prb_diag_mean: invalid argument or diagnostics not enabled");
        return GB_ERR_INVALID;
    }
    const PrbDev &d = h->dev;
    GB_CUDA_TRY(cudaMemcpy2DAsync(host, sizeof(double) * (size_t)ld, d.diag + (size_t)q * h->fsz,
                                  sizeof(double) * (size_t)d.ld, sizeof(double) * (size_t)d.ld, (size_t)d.np + 1,
                                  cudaMemcpyDeviceToHost, h->stream));
    return prb_sync(h, "gb_prb_diag_mean");
}

extern "C" int gb_prb_diag_cfl(gb_prb *h, int nsteps, double *cfl)
{
    if (!h || nsteps < 0 || !h->dev.diag || nsteps > h->hist_cap) {
        gb_set_error("gb_prb_diag_cfl: invalid argument or diagnostics not enabled");
        return GB_ERR_INVALID;
    }
    if (nsteps == 0) return GB_OK;
    GB_CUDA_TRY(cudaMemcpyAsync(cfl, h->dev.cfl_hist, sizeof(double) * 2 * (size_t)nsteps, cudaMemcpyDeviceToHost,
                                h->stream));
    return prb_sync(h, "gb_prb_diag_cfl");
}

// ---------------------------------------------------------------------------
// Gangs: many device-resident instances of different grid sizes stepped
// together.  Every phase of a step is one launch over the blocks of all
// members (a block finds its member in the phase's block-offset table and
// runs that member's kernel body with its local block index), and the two
// velocity solves of every member are the blocks of one multigrid launch.
// Each member runs exactly the kernel bodies of its own step, so its fields,
// Nusselt numbers and sweep counts are bit-identical to stepping it alone.
// A member whose step index reaches its step count sets its abort flag to
// GB_RUN_DONE and takes no further part.
// ---------------------------------------------------------------------------
enum GangPhase { GP_CDR, GP_CDX, GP_CUPD, GP_CROB, GP_TDR, GP_TDX, GP_TUPD, GP_TROB, GP_HEAT, GP_RHS, GP_UPD, GP_REC,
                 GP_COUNT };

struct GangRec {
    double c1, c2, div;   // Nusselt scalings of k_record
};

struct GangTab {
    const PrbDev *dev;    // [n]
    const int *off;       // [GP_COUNT][n + 1]: first block of each member in each phase's launch
    const GangRec *rec;   // [n]
    const int *limit;     // [n]: the member's total step count of the run
    int n;
};

__device__ __forceinline__ int gang_member(const int *off, int n, int b)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int PH>
__global__ void k_prb_gang(GangTab g)
{
    const int *off = g.off + (size_t)PH * (g.n + 1);
    const int m = gang_member(off, g.n, blockIdx.x);
    const PrbDev &d = g.dev[m];
    const int b = blockIdx.x - off[m];
    switch (PH) {
    case GP_CDR: k_cvort_deriv_r_body(d, b); break;
    case GP_CDX: k_cvort_deriv_x_body(d, b); break;
    case GP_CUPD: k_cvort_update_body(d, 0, b); break;
    case GP_CROB: k_robert_body(d, GB_F_C, GB_F_Cn, GB_F_Cp, d.nr - 1, b); break;
    case GP_TDR: k_temp_deriv_r_body(d, b); break;
    case GP_TDX: k_temp_deriv_x_body(d, b); break;
    case GP_TUPD: k_temp_update_body(d, 0, b); break;
    case GP_TROB: k_robert_body(d, GB_F_th, GB_F_thn, GB_F_thp, d.nr, b); break;
    case GP_HEAT: k_heat_body(d, 1, d.np, b); break;
    case GP_RHS: k_rhs_body(d, 1, 1, b); break;
    case GP_UPD: k_update_body<false>(d, b); break;
    case GP_REC: {
        const GangRec r = g.rec[m];
        k_record_body(d, r.c1, r.c2, r.div, 0, b);
        if (threadIdx.x == 0 && b == 0 && *d.abort == 0 && *d.step_index >= g.limit[m]) *d.abort = GB_RUN_DONE;
        break;
    }
    default: break;
    }
}

struct gb_prb_gang {
    int n = 0, mixed = 0;
    int spread = 1;                // CTAs per equation of the batched multigrid (1 or a cluster)
    size_t mg_smem = 0;            // shared memory of the mixed solves: the largest member's
    PrbDev *d_dev = nullptr;
    int *d_off = nullptr, *d_limit = nullptr;
    GangRec *d_rec = nullptr;
    MgEq *d_eqs = nullptr;
    std::vector<int> blocks;       // [GP_COUNT] total blocks of each phase
    int threads[GP_COUNT];
    size_t heat_smem = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    long long launches_per_step = 0;
};

extern "C" int gb_prb_gang_destroy(gb_prb_gang *g)
{
    if (!g) return GB_OK;
    if (g->graph) cudaGraphExecDestroy(g->graph);
    cudaFree(g->d_dev);
    cudaFree(g->d_off);
    cudaFree(g->d_limit);
    cudaFree(g->d_rec);
    cudaFree(g->d_eqs);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
    return GB_OK;
}

extern "C" int gb_prb_gang_create(gb_prb *const *members, const int *nsteps_total, int n, gb_prb_gang **out)
{
    if (!members || !nsteps_total || n < 1 || !out) {
        gb_set_error("gb_prb_gang_create: invalid argument");
        return GB_ERR_INVALID;
    }
    *out = nullptr;
    const int mixed = members[0]->p.precision == GB_PRB_MIXED;
    for (int q = 0; q < n; ++q) {
        const gb_prb *h = members[q];
        if (!h || h->dev.tank || h->dev.diag || (h->p.precision == GB_PRB_MIXED) != (mixed != 0) ||
            nsteps_total[q] < 0 || nsteps_total[q] > h->hist_cap) {
            gb_set_error("gb_prb_gang_create: member %d must be a layer or annulus instance without diagnostics, of "
                         "the gang's precision, after gb_prb_run_begin with at least its step count", q);
            return GB_ERR_INVALID;
        }
    }
    gb_prb_gang *g = new gb_prb_gang();
    g->n = n;
    g->mixed = mixed;
    // block counts per phase and member (the single-instance launch shapes)
    const int tpb[GP_COUNT] = {64, 64, TPB, TPB, 64, 64, TPB, TPB, 256, TPB, TPB, 32};
    for (int q = 0; q < GP_COUNT; ++q) g->threads[q] = tpb[q];
    std::vector<int> off((size_t)GP_COUNT * (n + 1));
    std::vector<PrbDev> devs(n);
    std::vector<GangRec> rec(n);
    std::vector<MgEq> eqs(2 * (size_t)n);
    g->blocks.assign(GP_COUNT, 0);
    for (int q = 0; q < n; ++q) {
        gb_prb *h = members[q];
        prb_refresh_scalars(h);
        const PrbDev &d = h->dev;
        devs[q] = d;
        g->mg_smem = std::max(g->mg_smem, prb_mg_smem(h));
        const size_t nr = d.nr, np = d.np;
        const int nb[GP_COUNT] = {(int)gb_ceil_div(np + 1, 64), (int)gb_ceil_div(nr - 1, 64),
                                  (int)gb_ceil_div((nr - 1) * (np + 1), TPB), (int)gb_ceil_div((nr - 1) * (np + 1), TPB),
                                  (int)gb_ceil_div(np + 1, 64), (int)gb_ceil_div(nr, 64),
                                  (int)gb_ceil_div(nr * (np + 1), TPB), (int)gb_ceil_div(nr * (np + 1), TPB), 1,
                                  (int)gb_ceil_div(nr * (np + 1), TPB), (int)gb_ceil_div((nr + 2) * (np + 1), TPB), 1};
        for (int ph = 0; ph < GP_COUNT; ++ph) {
            off[(size_t)ph * (n + 1) + q] = g->blocks[ph];
            g->blocks[ph] += nb[ph];
        }
        g->heat_smem = std::max(g->heat_smem, 2 * (size_t)(np + 1) * sizeof(double));
        double c1 = h->p.rmax - h->p.r0, c2 = c1, div = h->p.xx;
        if (h->p.variant == GB_PRB_ANNULUS || h->p.variant == GB_PRB_TAYCOU) {
            const double L = log(h->p.r0 / h->p.rmax);
            c1 = -h->p.r0 * L;
            c2 = -h->p.rmax * L;
            div = 2.0 * acos(-1.0);
        }
        rec[q] = {c1, c2, div};
        // the member's current equation descriptors (its settings as prb_launch_mg would use them)
        for (int e = 0; e < 2; ++e) {
            MgEq E = h->eq_host[e];
            E.mode = h->p.smoother;
            E.maxsweeps = h->p.maxsweeps;
            E.tolcon = h->p.tolcon;
            E.sor = h->p.sor;
            eqs[2 * (size_t)q + e] = E;
        }
    }
    for (int ph = 0; ph < GP_COUNT; ++ph) off[(size_t)ph * (n + 1) + n] = g->blocks[ph];
#define GTRY(x)                                                                   \
    do {                                                                          \
        cudaError_t _e = (x);                                                     \
        if (_e != cudaSuccess) {                                                  \
            gb_set_error("gb_prb_gang_create: %s: %s", #x, cudaGetErrorString(_e)); \
            gb_prb_gang_destroy(g);                                               \
            return GB_ERR_CUDA;                                                   \
        }                                                                         \
    } while (0)
    GTRY(cudaMalloc(&g->d_dev, sizeof(PrbDev) * n));
    GTRY(cudaMalloc(&g->d_off, sizeof(int) * off.size()));
    GTRY(cudaMalloc(&g->d_limit, sizeof(int) * n));
    GTRY(cudaMalloc(&g->d_rec, sizeof(GangRec) * n));
    GTRY(cudaMalloc(&g->d_eqs, sizeof(MgEq) * eqs.size()));
    GTRY(cudaMemcpy(g->d_dev, devs.data(), sizeof(PrbDev) * n, cudaMemcpyHostToDevice));
    GTRY(cudaMemcpy(g->d_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice));
    GTRY(cudaMemcpy(g->d_limit, nsteps_total, sizeof(int) * n, cudaMemcpyHostToDevice));
    GTRY(cudaMemcpy(g->d_rec, rec.data(), sizeof(GangRec) * n, cudaMemcpyHostToDevice));
    GTRY(cudaMemcpy(g->d_eqs, eqs.data(), sizeof(MgEq) * eqs.size(), cudaMemcpyHostToDevice));
    // the members' own queued work (their first steps) finishes before the gang's
    for (int q = 0; q < n; ++q) GTRY(cudaStreamSynchronize(members[q]->stream));
    GTRY(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    if (g->heat_smem > 48 * 1024)
        GTRY(cudaFuncSetAttribute(k_prb_gang<GP_HEAT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g->heat_smem));
#undef GTRY
    *out = g;
    return GB_OK;
}

static void prb_gang_enqueue_step(gb_prb_gang *g, cudaStream_t s)
{
    GangTab t{g->d_dev, g->d_off, g->d_rec, g->d_limit, g->n};
#define GL(PH) k_prb_gang<PH><<<g->blocks[PH], g->threads[PH], PH == GP_HEAT ? g->heat_smem : 0, s>>>(t)
    GL(GP_CDR);
    GL(GP_CDX);
    GL(GP_CUPD);
    GL(GP_CROB);
    GL(GP_TDR);
    GL(GP_TDX);
    GL(GP_TUPD);
    GL(GP_TROB);
    GL(GP_HEAT);
    GL(GP_RHS);
    prb_mg_launch_eqs(g->d_eqs, 2 * g->n, g->mixed, g->spread, g->mg_smem, s);
    GL(GP_UPD);
    GL(GP_REC);
#undef GL
    g->launches_per_step = GP_COUNT + 1;
}

// Queues nsteps leapfrog steps (not the first step of a run) of every
// member, one CUDA graph launch per step, on `stream` (NULL: the gang's own).
extern "C" int gb_prb_gang_enqueue(gb_prb_gang *g, int nsteps, void *stream)
{
    if (!g || nsteps < 0) { gb_set_error("gb_prb_gang_enqueue: invalid argument"); return GB_ERR_INVALID; }
    cudaStream_t s = stream ? (cudaStream_t)stream : g->stream;
    if (!g->graph) {
        cudaGraph_t gr;
        GB_CUDA_TRY(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
        prb_gang_enqueue_step(g, g->stream);
        GB_CUDA_TRY(cudaStreamEndCapture(g->stream, &gr));
        GB_CUDA_TRY(cudaGraphInstantiate(&g->graph, gr, 0));
        cudaGraphDestroy(gr);
    }
    for (int k = 0; k < nsteps; ++k) GB_CUDA_TRY(cudaGraphLaunch(g->graph, s));
    return GB_OK;
}

extern "C" int gb_prb_gang_set_solve_spread(gb_prb_gang *g, int ctas)
{
    if (!g || (ctas != 1 && ctas != prb_mg_cluster_ctas())) {
        gb_set_error("gb_prb_gang_set_solve_spread: ctas must be 1 or %d", prb_mg_cluster_ctas());
        return GB_ERR_INVALID;
    }
    if (g->spread != ctas) {
        g->spread = ctas;
        if (g->graph) { cudaGraphExecDestroy(g->graph); g->graph = nullptr; }
    }
    return GB_OK;
}

extern "C" void *gb_prb_gang_stream(gb_prb_gang *g) { return g ? (void *)g->stream : nullptr; }

extern "C" int gb_prb_gang_query(gb_prb_gang *g)
{
    if (!g) return -GB_ERR_INVALID;
    const cudaError_t e = cudaStreamQuery(g->stream);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) { cudaGetLastError(); return 0; }
    gb_set_error("gb_prb_gang_query: %s", cudaGetErrorString(e));
    return -GB_ERR_CUDA;
}
extern "C" long long gb_prb_gang_launches_per_step(const gb_prb_gang *g) { return g ? g->launches_per_step : 0; }
