// Axisymmetric rotating annulus in the (r, z) meridional plane (rotann2.f,
// "AXI") on the device: Dufort-Frankel vorticity, swirl-velocity and
// temperature updates with the Arakawa Jacobian, Thom wall vorticity, the
// inner-wall heat flux, and the streamfunction multigrid.
//
// Numerics: every expression keeps the reference's operation order and the
// translation unit is compiled with -fmad=false, so the FP64 path is
// bit-identical to the reference algorithm (and to the C oracle).
//
// Layout: each field is a column-major (0:ld-1, 0:nz) array with ld = nr+1,
// the ten fields of an instance in one allocation.  The multigrid keeps the
// full-size psif and rc arrays, per level the packed v / f slots, the
// factored r-line matrix (one per level: its coefficients vary with r only)
// and one factored z-line matrix per r-row (its diagonal holds -1/r^2).
//
// The multigrid solve is one persistent block: the sweep loop, every level
// and the convergence test run in one launch.  LEX orders the lines as the
// reference does (rows j = 1..n2-1, then columns i = 1..n1-1, rotann2.f:
// 698-725) and one thread marches them; ZEBRA solves odd lines, then even
// lines, one thread per line.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "banded.cuh"
#include "gbcommon.cuh"
#include "str_internal.cuh"

#define AXI_THREADS 512
#define AXI_MAXLEV 8
#define AX(i, j) ((size_t)(i) + (size_t)ld * (size_t)(j))

struct AxiLevel {
    int n1, n2, lf;           // sizes; lf = 2^l / 2 scales i into rval
    double hr, hz, hhr, hhz;
    double *v, *f;            // packed (n1+1)*(n2+1)
    double *fac_r;            // r-line factors, 3 (n1-1)
    double *fac_z;            // z-line factors, 3 (n2-1) for each i = 1..n1-1
    // mixed precision: FP32 correction cycle (pivots stored as reciprocals)
    float *v32, *f32, *fac_r32, *fac_z32;
};

// Stretched grid (gb_axi_create_stretched): level-1 positions, grid.f's
// finite-difference weights and the inner-wall d/dr weights of the heat flux.
struct AxsTab {
    const double *r, *z;      // r(0..nr), z(0..nz)
    const double *cr, *crr;   // rows i = 1..nr-1: [3(i-1) + k], [4(i-1) + k]
    const double *cz, *czz;   // rows j = 1..nz-1: [3(j-1) + k], [4(j-1) + k]
    double hw[5];             // d/dr at r(0) on r(0..4)
};

struct AxiDev {
    int nr, nz, ld, nlev, mode, maxsweeps, nrel;
    int stretched;            // 1: the transport uses st (and the stretched multigrid)
    AxsTab st;
    double dt, dr, dz, r0, rmax, zmax, Ra, Re, Ptl;
    double cf1, cf2, cf3, cf4, tolcon;
    double *f[GB_A_COUNT];
    double *rval;             // rotann2.f:626: rval(i) = i hr(1) + r0
    double *psif, *rc;
    float *psif32, *rc32, *rval32;
    AxiLevel lev[AXI_MAXLEV];
    double *heat;
    unsigned long long *errmax;   // bit patterns of the step's max |x - x_p|, x = omega, v, T
    int *abort;               // 1: a solve failed; 2: the run reached the steady state
    int *status;              // [0] poisson status, [1] sweeps
    int *step_index;
    double *nu_hist;
    int *sweep_hist;
    int hist_cap;
    double nu_c, nu_d;        // httrans = trans * nu_c / nu_d
};

// ---------------------------------------------------------------------------
// Transport
// ---------------------------------------------------------------------------

// arakawa, rotann2.f:432-459, at one interior point.
__device__ __forceinline__ double arakawa_at(const double *psi, const double *th, int ld, int i, int j, double hx,
                                             double hy)
{
    const int ip = i + 1, im = i - 1;
    const double a = (psi[AX(ip, j)] - psi[AX(im, j)]) * (th[AX(i, j + 1)] - th[AX(i, j - 1)]) -
                     (psi[AX(i, j + 1)] - psi[AX(i, j - 1)]) * (th[AX(ip, j)] - th[AX(im, j)]) +
                     psi[AX(ip, j)] * (th[AX(ip, j + 1)] - th[AX(ip, j - 1)]) -
                     psi[AX(im, j)] * (th[AX(im, j + 1)] - th[AX(im, j - 1)]) -
                     psi[AX(i, j + 1)] * (th[AX(ip, j + 1)] - th[AX(im, j + 1)]) +
                     psi[AX(i, j - 1)] * (th[AX(ip, j - 1)] - th[AX(im, j - 1)]) +
                     th[AX(i, j + 1)] * (psi[AX(ip, j + 1)] - psi[AX(im, j + 1)]) -
                     th[AX(i, j - 1)] * (psi[AX(ip, j - 1)] - psi[AX(im, j - 1)]) -
                     th[AX(ip, j)] * (psi[AX(ip, j + 1)] - psi[AX(ip, j - 1)]) +
                     th[AX(im, j)] * (psi[AX(im, j + 1)] - psi[AX(im, j - 1)]);
    return a / (12.0 * hx * hy);
}

// ---------------------------------------------------------------------------
// Stretched-grid forms: every derivative of rotann2.f's transport taken with
// grid.f's weights, each sum in the order written here (the oracle's
// orc_axi_set_stretched states them and performs the same operations).
// ---------------------------------------------------------------------------
#define SCR(i, k) T.cr[3 * ((i) - 1) + (k) - 1]
#define SCRR(i, k) T.crr[4 * ((i) - 1) + (k) - 1]
#define SCZ(j, k) T.cz[3 * ((j) - 1) + (k) - 1]
#define SCZZ(j, k) T.czz[4 * ((j) - 1) + (k) - 1]

__device__ __forceinline__ double axs_dr_off(const AxsTab &T, const double *x, int ld, int i, int j)
{
    return SCR(i, 1) * x[AX(i - 1, j)] + SCR(i, 3) * x[AX(i + 1, j)];
}
__device__ __forceinline__ double axs_drr_off(const AxsTab &T, const double *x, int ld, int i, int j, int nr)
{
    if (i <= nr / 2) return SCRR(i, 1) * x[AX(i - 1, j)] + SCRR(i, 3) * x[AX(i + 1, j)] + SCRR(i, 4) * x[AX(i + 2, j)];
    return SCRR(i, 1) * x[AX(i - 2, j)] + SCRR(i, 2) * x[AX(i - 1, j)] + SCRR(i, 4) * x[AX(i + 1, j)];
}
__device__ __forceinline__ double axs_crrc(const AxsTab &T, int i, int nr) { return i <= nr / 2 ? SCRR(i, 2) : SCRR(i, 3); }
__device__ __forceinline__ double axs_dz(const AxsTab &T, const double *x, int ld, int i, int j)
{
    return SCZ(j, 1) * x[AX(i, j - 1)] + SCZ(j, 2) * x[AX(i, j)] + SCZ(j, 3) * x[AX(i, j + 1)];
}
__device__ __forceinline__ double axs_dzz_off(const AxsTab &T, const double *x, int ld, int i, int j, int nz)
{
    if (j <= nz / 2) return SCZZ(j, 1) * x[AX(i, j - 1)] + SCZZ(j, 3) * x[AX(i, j + 1)] + SCZZ(j, 4) * x[AX(i, j + 2)];
    return SCZZ(j, 1) * x[AX(i, j - 2)] + SCZZ(j, 2) * x[AX(i, j - 1)] + SCZZ(j, 4) * x[AX(i, j + 1)];
}
__device__ __forceinline__ double axs_czzc(const AxsTab &T, int j, int nz) { return j <= nz / 2 ? SCZZ(j, 2) : SCZZ(j, 3); }

// the Arakawa sum over the local metric 3 (r(i+1) - r(i-1)) (z(j+1) - z(j-1))
__device__ __forceinline__ double axs_arakawa(const AxsTab &T, const double *psi, const double *th, int ld, int i, int j)
{
    const int ip = i + 1, im = i - 1;
    const double a = (psi[AX(ip, j)] - psi[AX(im, j)]) * (th[AX(i, j + 1)] - th[AX(i, j - 1)]) -
                     (psi[AX(i, j + 1)] - psi[AX(i, j - 1)]) * (th[AX(ip, j)] - th[AX(im, j)]) +
                     psi[AX(ip, j)] * (th[AX(ip, j + 1)] - th[AX(ip, j - 1)]) -
                     psi[AX(im, j)] * (th[AX(im, j + 1)] - th[AX(im, j - 1)]) -
                     psi[AX(i, j + 1)] * (th[AX(ip, j + 1)] - th[AX(im, j + 1)]) +
                     psi[AX(i, j - 1)] * (th[AX(ip, j - 1)] - th[AX(im, j - 1)]) +
                     th[AX(i, j + 1)] * (psi[AX(ip, j + 1)] - psi[AX(im, j + 1)]) -
                     th[AX(i, j - 1)] * (psi[AX(ip, j - 1)] - psi[AX(im, j - 1)]) -
                     th[AX(ip, j)] * (psi[AX(ip, j + 1)] - psi[AX(ip, j - 1)]) +
                     th[AX(im, j)] * (psi[AX(im, j + 1)] - psi[AX(im, j - 1)]);
    return a / (3.0 * (T.r[ip] - T.r[im]) * (T.z[j + 1] - T.z[j - 1]));
}

// vorticity and velocity of the stretched state at interior point (i, j)
__device__ __forceinline__ void axs_vort_vel_at(const AxiDev &d, int what, int i, int j)
{
    const AxsTab &T = d.st;
    const int ld = d.ld, nr = d.nr, nz = d.nz;
    const double Ptl = d.Ptl, Ra = d.Ra, Re = d.Re, dt = d.dt;
    const double *phi = d.f[GB_A_phi], *omeg = d.f[GB_A_omeg], *vel = d.f[GB_A_vel], *theta = d.f[GB_A_theta];
    const double RRP = Ra / Re / Ptl;
    const double r = T.r[i];
    const double sigma = axs_crrc(T, i, nr) + SCR(i, 2) / r + axs_czzc(T, j, nz);
    const double A = 1.0 / (2.0 * Ptl * dt) - sigma / 2.0 + 1.0 / (2.0 * (r * r));
    const double AA = 1.0 / (2.0 * Ptl * dt) + sigma / 2.0 - 1.0 / (2.0 * (r * r));
    const double dz_phi = axs_dz(T, phi, ld, i, j), dz_v = axs_dz(T, vel, ld, i, j);
    if (what & 1) {
        const double arak = axs_arakawa(T, phi, omeg, ld, i, j);
        const double dz_om = axs_dz(T, omeg, ld, i, j), dz_th = axs_dz(T, theta, ld, i, j);
        const double B = (phi[AX(i, j)] * dz_om + omeg[AX(i, j)] * dz_phi) / (Ptl * r);
        const double C = 2.0 * vel[AX(i, j)] * dz_v / (Ptl * r);
        const double D = 2.0 * Re * dz_v;
        const double E = r * Ra * dz_th;
        const double EE = 2.0 * RRP * vel[AX(i, j)] * dz_th + 2.0 * RRP * theta[AX(i, j)] * dz_v;
        const double F = axs_drr_off(T, omeg, ld, i, j, nr);
        const double G = axs_dr_off(T, omeg, ld, i, j) / r;
        const double H = axs_dzz_off(T, omeg, ld, i, j, nz);
        d.f[GB_A_omegn][AX(i, j)] = (AA * d.f[GB_A_omegp][AX(i, j)] + arak / Ptl + B + C + D - E - EE + F + G + H) / A;
    }
    if (what & 2) {
        const double arak = axs_arakawa(T, phi, vel, ld, i, j);
        const double B = (vel[AX(i, j)] * dz_phi - phi[AX(i, j)] * dz_v) / (Ptl * r);
        const double C = 2.0 * Re * dz_phi;
        const double CC = -2.0 * RRP * theta[AX(i, j)] * dz_phi;
        const double D = axs_drr_off(T, vel, ld, i, j, nr);
        const double E = axs_dr_off(T, vel, ld, i, j) / r;
        const double F = axs_dzz_off(T, vel, ld, i, j, nz);
        d.f[GB_A_veln][AX(i, j)] = (AA * d.f[GB_A_velp][AX(i, j)] + arak / Ptl - B - C - CC + D + E + F) / A;
    }
}

// temperature of the stretched state at (i, j), j = 0..nz (rows 0 and nz
// mirrored: d/dz = 0, d2/dz2 from the wall spacing)
__device__ __forceinline__ void axs_temperature_at(const AxiDev &d, int i, int j)
{
    const AxsTab &T = d.st;
    const int ld = d.ld, nr = d.nr, nz = d.nz;
    const double dt = d.dt;
    const double *phi = d.f[GB_A_phi], *theta = d.f[GB_A_theta];
    const double r = T.r[i];
    double arak, B, E, czzc;
    if (j == 0) {
        const double h1 = T.z[1] - T.z[0];
        arak = 0.0;
        B = 0.0;
        E = 2.0 * theta[AX(i, 1)] / (h1 * h1);
        czzc = -2.0 / (h1 * h1);
    } else if (j == nz) {
        const double hn = T.z[nz] - T.z[nz - 1];
        arak = 0.0;
        B = 0.0;
        E = 2.0 * theta[AX(i, nz - 1)] / (hn * hn);
        czzc = -2.0 / (hn * hn);
    } else {
        arak = axs_arakawa(T, phi, theta, ld, i, j);
        B = phi[AX(i, j)] * axs_dz(T, theta, ld, i, j) / r;
        E = axs_dzz_off(T, theta, ld, i, j, nz);
        czzc = axs_czzc(T, j, nz);
    }
    const double sigma = axs_crrc(T, i, nr) + SCR(i, 2) / r + czzc;
    const double cf3 = 1.0 / (2.0 * dt) - sigma / 2.0;
    const double cf4 = 1.0 / (2.0 * dt) + sigma / 2.0;
    const double C = axs_drr_off(T, theta, ld, i, j, nr);
    const double D = axs_dr_off(T, theta, ld, i, j) / r;
    d.f[GB_A_thetan][AX(i, j)] = (cf4 * d.f[GB_A_thetap][AX(i, j)] + arak + B + C + D + E) / cf3;
}

#undef SCR
#undef SCRR
#undef SCZ
#undef SCZZ

// vorticity (rotann2.f:268-316, what & 1) and velocity (rotann2.f:324-370,
// what & 2) on the interior, one thread per point (S: the stretched forms).
template <bool S>
__device__ __forceinline__ void k_axi_vort_vel_body(const AxiDev &d, int what, int bidx)
{
    const int t = bidx * blockDim.x + threadIdx.x;
    const int ni = d.nr - 1, nj = d.nz - 1;
    if (t >= ni * nj || *d.abort) return;
    const int i = t % ni + 1, j = t / ni + 1;
    if constexpr (S) {
        axs_vort_vel_at(d, what, i, j);
        return;
    }
    const int ld = d.ld;
    const int ip = i + 1, im = i - 1, jp = j + 1, jm = j - 1;
    const double dr = d.dr, dz = d.dz, Ptl = d.Ptl;
    const double *phi = d.f[GB_A_phi], *omeg = d.f[GB_A_omeg], *vel = d.f[GB_A_vel], *theta = d.f[GB_A_theta];
    const double RRP = d.Ra / d.Re / Ptl;
    const double r = d.r0 + (double)i * dr;
    const double A = d.cf1 + 1.0 / (2.0 * (r * r));
    const double AA = d.cf2 - 1.0 / (2.0 * (r * r));
    if (what & 1) {
        const double arak = arakawa_at(phi, omeg, ld, i, j, dr, dz);
        const double B = (1.0 / (2.0 * Ptl * r * dz)) *
                         (phi[AX(i, j)] * (omeg[AX(i, jp)] - omeg[AX(i, jm)]) +
                          omeg[AX(i, j)] * (phi[AX(i, jp)] - phi[AX(i, jm)]));
        const double C = (1.0 / (Ptl * r * dz)) * vel[AX(i, j)] * (vel[AX(i, jp)] - vel[AX(i, jm)]);
        const double D = d.Re * (vel[AX(i, jp)] - vel[AX(i, jm)]) / dz;
        const double E = r * d.Ra * (theta[AX(i, jp)] - theta[AX(i, jm)]) / (2.0 * dz);
        const double EE = RRP * vel[AX(i, j)] * (theta[AX(i, jp)] - theta[AX(i, jm)]) / dz +
                          RRP * theta[AX(i, j)] * (vel[AX(i, jp)] - vel[AX(i, jm)]) / dz;
        const double F = (omeg[AX(ip, j)] + omeg[AX(im, j)]) / (dr * dr);
        const double G = (1.0 / (2.0 * r * dr)) * (omeg[AX(ip, j)] - omeg[AX(im, j)]);
        const double H = (omeg[AX(i, jp)] + omeg[AX(i, jm)]) / (dz * dz);
        d.f[GB_A_omegn][AX(i, j)] =
            (AA * d.f[GB_A_omegp][AX(i, j)] + arak / Ptl + B + C + D - E - EE + F + G + H) / A;
    }
    if (what & 2) {
        const double arak = arakawa_at(phi, vel, ld, i, j, dr, dz);
        const double B = (1.0 / (2.0 * Ptl * r * dz)) *
                         (vel[AX(i, j)] * (phi[AX(i, jp)] - phi[AX(i, jm)]) -
                          phi[AX(i, j)] * (vel[AX(i, jp)] - vel[AX(i, jm)]));
        const double C = d.Re * (phi[AX(i, jp)] - phi[AX(i, jm)]) / dz;
        const double CC = -RRP * theta[AX(i, j)] * (phi[AX(i, jp)] - phi[AX(i, jm)]) / dz;
        const double D = (vel[AX(ip, j)] + vel[AX(im, j)]) / (dr * dr);
        const double E = (1.0 / (2.0 * r * dr)) * (vel[AX(ip, j)] - vel[AX(im, j)]);
        const double F = (vel[AX(i, jp)] + vel[AX(i, jm)]) / (dz * dz);
        d.f[GB_A_veln][AX(i, j)] = (AA * d.f[GB_A_velp][AX(i, j)] + arak / Ptl - B - C - CC + D + E + F) / A;
    }
}

template <bool S>
__global__ void k_axi_vort_vel(AxiDev d, int what) { k_axi_vort_vel_body<S>(d, what, blockIdx.x); }

// temperature, rotann2.f:379-424: rows j = 0 and nz mirror their neighbour
// and take no Jacobian.
template <bool S>
__device__ __forceinline__ void k_axi_temperature_body(const AxiDev &d, int bidx)
{
    const int t = bidx * blockDim.x + threadIdx.x;
    const int ni = d.nr - 1, nj = d.nz + 1;
    if (t >= ni * nj || *d.abort) return;
    const int i = t % ni + 1, j = t / ni;
    if constexpr (S) {
        axs_temperature_at(d, i, j);
        return;
    }
    const int ld = d.ld, nz = d.nz;
    const double dr = d.dr, dz = d.dz;
    const double *phi = d.f[GB_A_phi], *theta = d.f[GB_A_theta];
    const int ip = i + 1, im = i - 1;
    int jp = j + 1, jm = j - 1;
    double arak;
    if (j == 0) {
        jm = jp;
        arak = 0.0;
    } else if (j == nz) {
        jp = jm;
        arak = 0.0;
    } else {
        arak = arakawa_at(phi, theta, ld, i, j, dr, dz);
    }
    const double r = d.r0 + (double)i * dr;
    const double B = (1.0 / (2.0 * r * dz)) * phi[AX(i, j)] * (theta[AX(i, jp)] - theta[AX(i, jm)]);
    const double C = (theta[AX(ip, j)] + theta[AX(im, j)]) / (dr * dr);
    const double D = (1.0 / (2.0 * r * dr)) * (theta[AX(ip, j)] - theta[AX(im, j)]);
    const double E = (theta[AX(i, jp)] + theta[AX(i, jm)]) / (dz * dz);
    d.f[GB_A_thetan][AX(i, j)] = (d.cf4 * d.f[GB_A_thetap][AX(i, j)] + arak + B + C + D + E) / d.cf3;
}

template <bool S>
__global__ void k_axi_temperature(AxiDev d) { k_axi_temperature_body<S>(d, blockIdx.x); }

// update, rotann2.f:497-539, one thread per point: Thom wall vorticity (the
// r-walls written last own the corners), v = 0 on the walls, T = 0 / 1 on
// the inner / outer wall, then the time levels rotate.  The steady-state
// test's maxima of |x - x_p| (rotann2.f:162-180) are gathered here.
// S: the stretched grid's wall spacings in the Thom wall vorticity (rcsc.f
// update, :706-751).
template <bool S>
__device__ __forceinline__ void k_axi_update_body(const AxiDev &d, int bidx)
{
    const int t = bidx * blockDim.x + threadIdx.x;
    const int nr = d.nr, nz = d.nz, ld = d.ld;
    if (*d.abort) return;   // uniform over the grid
    const bool live = t < (nr + 1) * (nz + 1);
    double e[3] = {0.0, 0.0, 0.0};
    if (live) {
        const int i = t % (nr + 1), j = t / (nr + 1);
        const size_t c = AX(i, j);
        double *const *f = d.f;
        const double *phi = f[GB_A_phi];
        double hr0 = d.dr, hrn = d.dr, hz0 = d.dz, hzn = d.dz;
        if constexpr (S) {
            hr0 = d.st.r[1] - d.st.r[0];
            hrn = d.st.r[nr] - d.st.r[nr - 1];
            hz0 = d.st.z[1] - d.st.z[0];
            hzn = d.st.z[nz] - d.st.z[nz - 1];
        }
        double on = f[GB_A_omegn][c], vn = f[GB_A_veln][c], tn = f[GB_A_thetan][c];
        if (i == 0) {
            on = 2.0 * phi[AX(1, j)] / (hr0 * hr0);
            vn = 0.0;
            tn = 0.0;
        } else if (i == nr) {
            on = 2.0 * phi[AX(nr - 1, j)] / (hrn * hrn);
            vn = 0.0;
            tn = 1.0;
        } else if (j == 0) {
            on = 2.0 * phi[AX(i, 1)] / (hz0 * hz0);
            vn = 0.0;
        } else if (j == nz) {
            on = 2.0 * phi[AX(i, nz - 1)] / (hzn * hzn);
            vn = 0.0;
        }
        f[GB_A_omegn][c] = on;
        f[GB_A_veln][c] = vn;
        f[GB_A_thetan][c] = tn;
        const double o = f[GB_A_omeg][c], v = f[GB_A_vel][c], th = f[GB_A_theta][c];
        f[GB_A_omegp][c] = o;
        f[GB_A_omeg][c] = on;
        f[GB_A_velp][c] = v;
        f[GB_A_vel][c] = vn;
        f[GB_A_thetap][c] = th;
        f[GB_A_theta][c] = tn;
        e[0] = fabs(on - o);
        e[1] = fabs(vn - v);
        e[2] = fabs(tn - th);
    }
    // non-negative doubles order like their bit patterns: warp maximum, then
    // one atomic per warp
    for (int q = 0; q < 3; ++q) {
        unsigned long long m = (unsigned long long)__double_as_longlong(e[q]);
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long w = __shfl_down_sync(0xffffffffu, m, o);
            m = w > m ? w : m;
        }
        if ((threadIdx.x & 31) == 0) atomicMax(&d.errmax[q], m);
    }
}

template <bool S>
__global__ void k_axi_update(AxiDev d) { k_axi_update_body<S>(d, blockIdx.x); }

// heat, rotann2.f:468-487: the per-row terms in parallel, summed by one
// thread in the reference's order.
// S: the five-point one-sided weights of the stretched grid and the
// trapezoid rule on its z positions.
template <bool S>
__device__ __forceinline__ void k_axi_heat_body(const AxiDev &d, int bidx)
{
    extern __shared__ double sh[];
    if (*d.abort == 1) return;
    const int ld = d.ld, nz = d.nz;
    const double dr = d.dr, dz = d.dz;
    const double *th = d.f[GB_A_theta];
    for (int j = threadIdx.x; j <= nz; j += blockDim.x) {
        if constexpr (S) {
            const AxsTab &T = d.st;
            const double *w = T.hw;
            const double wz = j == 0 ? (T.z[1] - T.z[0]) / 2.0
                                     : (j == nz ? (T.z[nz] - T.z[nz - 1]) / 2.0 : (T.z[j + 1] - T.z[j - 1]) / 2.0);
            sh[j] = wz * (w[0] * th[AX(0, j)] + w[1] * th[AX(1, j)] + w[2] * th[AX(2, j)] + w[3] * th[AX(3, j)] +
                          w[4] * th[AX(4, j)]);
        } else {
            const double div = (j == 0 || j == nz) ? 24.0 * dr : 12.0 * dr;
            sh[j] = dz * (-25.0 * th[AX(0, j)] + 48.0 * th[AX(1, j)] - 36.0 * th[AX(2, j)] + 16.0 * th[AX(3, j)] -
                          3.0 * th[AX(4, j)]) / div;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double trans = sh[0];
        trans = trans + sh[nz];
        for (int j = 1; j <= nz - 1; ++j) trans = trans + sh[j];
        d.heat[0] = trans;
    }
}

template <bool S>
__global__ void k_axi_heat(AxiDev d) { k_axi_heat_body<S>(d, blockIdx.x); }

// Per-step bookkeeping: Nu and sweeps into the history, the steady-state
// test (REAL*4 threshold 1e-6, rotann2.f:191) and its reset.
__device__ __forceinline__ void k_axi_record_body(const AxiDev &d, int bidx)
{
    if (threadIdx.x != 0 || bidx != 0) return;
    if (*d.abort) return;
    const int s = *d.step_index;
    if (s < d.hist_cap) {
        d.nu_hist[s] = d.heat[0] * d.nu_c / d.nu_d;
        d.sweep_hist[s] = d.status[1];
    }
    *d.step_index = s + 1;
    const double tol = (double)1e-6f;
    const double e1 = __longlong_as_double((long long)d.errmax[0]), e2 = __longlong_as_double((long long)d.errmax[1]),
                 e3 = __longlong_as_double((long long)d.errmax[2]);
    if (e1 < tol && e2 < tol && e3 < tol) *d.abort = 2;
    d.errmax[0] = d.errmax[1] = d.errmax[2] = 0ull;
}

__global__ void k_axi_record(AxiDev d) { k_axi_record_body(d, blockIdx.x); }

// ---------------------------------------------------------------------------
// Streamfunction multigrid (rotann2.f:543-854)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double axi_blk_max(double v, double *s_red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = (lane < nw) ? s_red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
        if (lane == 0) s_red[32] = v;
    }
    __syncthreads();
    const double r = s_red[32];
    __syncthreads();
    return r;
}

// r-line j of relax (rotann2.f:698-710).
__device__ __forceinline__ void axi_rline(const AxiDev &d, const AxiLevel &L, int j)
{
    const int ld = d.ld, n1 = L.n1;
    double *psif = d.psif;
    const double *f = L.f;
    const double hhz = L.hhz;
    auto rhs = [&](int q) -> double {
        const int i = q + 1;
        return -(psif[AX(i, j + 1)] + psif[AX(i, j - 1)]) / hhz + f[(size_t)j * (n1 + 1) + i];
    };
    apply_tdma_rhs(L.fac_r, n1 - 1, psif + AX(1, j), 1, rhs);
}

// z-line i of relax (rotann2.f:712-725).
__device__ __forceinline__ void axi_zline(const AxiDev &d, const AxiLevel &L, int i)
{
    const int ld = d.ld, n1 = L.n1, n2 = L.n2;
    double *psif = d.psif;
    const double *f = L.f;
    const double hhr = L.hhr, hr = L.hr, rv = d.rval[i * L.lf];
    auto rhs = [&](int q) -> double {
        const int j = q + 1;
        return -(psif[AX(i + 1, j)] + psif[AX(i - 1, j)]) / hhr + f[(size_t)j * (n1 + 1) + i] -
               (psif[AX(i + 1, j)] - psif[AX(i - 1, j)]) * 0.5 / rv / hr;
    };
    apply_tdma_rhs(L.fac_z + (size_t)(i - 1) * tdma_fac_len(n2 - 1), n2 - 1, psif + AX(i, 1), ld, rhs);
}

// relax (rotann2.f:668-753): psif from v, nrel sweeps of r-lines then
// z-lines with the residual after each, psif back into v.  Returns the last
// residual max norm; *nan_out is set (block-uniform) on a NaN residual.
__device__ double axi_relax(const AxiDev &d, int klev, double *s_red, int *nan_out)
{
    const AxiLevel &L = d.lev[klev];
    const int ld = d.ld, n1 = L.n1, n2 = L.n2;
    const double hhr = L.hhr, hhz = L.hhz, hr = L.hr;
    double *psif = d.psif, *rc = d.rc;
    const int tp = (n1 + 1) * (n2 + 1);
    for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
        const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
        psif[AX(i, j)] = L.v[idx];
    }
    __syncthreads();
    const double drdz = 2.0 * (1.0 / hhr + 1.0 / hhz);
    double m = 0.0;
    int nan = 0;
    for (int irel = 0; irel < d.nrel; ++irel) {
        if (d.mode == GB_SMOOTHER_LEX) {
            if (threadIdx.x == 0)
                for (int j = 1; j <= n2 - 1; ++j) axi_rline(d, L, j);
            __syncthreads();
            if (threadIdx.x == 0)
                for (int i = 1; i <= n1 - 1; ++i) axi_zline(d, L, i);
            __syncthreads();
        } else {
            for (int par = 1; par >= 0; --par) {
                for (int t = threadIdx.x; 2 * t + 2 - par <= n2 - 1; t += blockDim.x) axi_rline(d, L, 2 * t + 2 - par);
                __syncthreads();
            }
            for (int par = 1; par >= 0; --par) {
                for (int t = threadIdx.x; 2 * t + 2 - par <= n1 - 1; t += blockDim.x) axi_zline(d, L, 2 * t + 2 - par);
                __syncthreads();
            }
        }
        m = 0.0;
        nan = 0;
        const int ni = n1 - 1, tot = ni * (n2 - 1);
        for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
            const int j = idx / ni + 1, i = idx - (j - 1) * ni + 1;
            const double rv = d.rval[i * L.lf];
            double temp = (psif[AX(i + 1, j)] + psif[AX(i - 1, j)]) / hhr +
                          (psif[AX(i + 1, j)] - psif[AX(i - 1, j)]) * 0.5 / hr / rv -
                          psif[AX(i, j)] / (rv * rv) + (psif[AX(i, j + 1)] + psif[AX(i, j - 1)]) / hhz -
                          psif[AX(i, j)] * drdz;
            temp = L.f[(size_t)j * (n1 + 1) + i] - temp;
            rc[AX(i, j)] = temp;
            temp = fabs(temp);
            if (temp != temp) nan = 1;
            if (temp > m) m = temp;
        }
        nan = __syncthreads_or(nan);
        m = axi_blk_max(m, s_red);
    }
    for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
        const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
        L.v[idx] = psif[AX(i, j)];
    }
    __syncthreads();
    *nan_out = nan;
    return m;
}

// corser (rotann2.f:755-801): the nine-point restriction of rc into the
// packed coarse right-hand side; the rows and columns the reference clears
// (i = 0, n1c and j = 0, n1c: n1 of the coarse level in both directions)
// are zero, and the coarse solution slot is cleared.
__device__ void axi_corser(const AxiDev &d, int klev)
{
    const int ld = d.ld;
    const int n1c = d.lev[klev + 1].n1, n2c = d.lev[klev + 1].n2;
    const double *rf = d.rc;
    double *fc = d.lev[klev + 1].f, *vc = d.lev[klev + 1].v;
    const int tot = (n1c + 1) * (n2c + 1);
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int j = idx / (n1c + 1), i = idx - j * (n1c + 1);
        double temp = 0.0;
        if (i >= 1 && i <= n1c - 1 && j >= 1 && j <= n2c - 1 && j != n1c) {
            const int ii = i + i, jj = j + j;
            temp = rf[AX(ii, jj)];
            temp = temp * 2.0 + rf[AX(ii + 1, jj)] + rf[AX(ii - 1, jj)];
            temp = temp + rf[AX(ii, jj + 1)] + rf[AX(ii, jj - 1)];
            temp = temp * 2.0 + rf[AX(ii + 1, jj + 1)] + rf[AX(ii - 1, jj - 1)];
            temp = temp + rf[AX(ii + 1, jj - 1)] + rf[AX(ii - 1, jj + 1)];
            temp = temp / 16.0;
        }
        fc[idx] = temp;
        vc[idx] = 0.0;
    }
    __syncthreads();
}

// finer (rotann2.f:803-854): bilinear prolongation of the coarse solution
// plus the saved fine solution into psif, the coarse slot cleared, psif
// packed into the fine slot.
__device__ void axi_finer(const AxiDev &d, int klev)
{
    const int ld = d.ld;
    const int n1c = d.lev[klev].n1;
    const int n1f = d.lev[klev - 1].n1, n2f = d.lev[klev - 1].n2;
    const double *vc = d.lev[klev].v;
    double *vf = d.lev[klev - 1].v, *psif = d.psif;
    const int tot = (n1f + 1) * (n2f + 1);
#define PC(ii, jj) vc[(size_t)(jj) * (n1c + 1) + (ii)]
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int j = idx / (n1f + 1), i = idx - j * (n1f + 1);
        const int i1 = i / 2, j1 = j / 2;
        double p;
        if (i1 * 2 == i) {
            if (j1 * 2 == j) p = PC(i1, j1);
            else p = (PC(i1, j1) + PC(i1, j1 + 1)) * 0.5;
        } else {
            if (j1 * 2 == j) {
                p = (PC(i1, j1) + PC(i1 + 1, j1)) * 0.5;
            } else {
                double temp = PC(i1, j1) + PC(i1 + 1, j1 + 1);
                temp = temp + PC(i1, j1 + 1) + PC(i1 + 1, j1);
                p = temp * 0.25;
            }
        }
        psif[AX(i, j)] = p + vf[idx];
    }
#undef PC
    __syncthreads();
    const int tc = (n1c + 1) * (d.lev[klev].n2 + 1);
    for (int idx = threadIdx.x; idx < tc; idx += blockDim.x) d.lev[klev].v[idx] = 0.0;
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int j = idx / (n1f + 1), i = idx - j * (n1f + 1);
        vf[idx] = psif[AX(i, j)];
    }
    __syncthreads();
}

// poisson (rotann2.f:598-666): phi from omegn.
__device__ __forceinline__ void k_axi_mg_solve_body(const AxiDev &d, int bidx)
{
    __shared__ double s_red[33];
    if (*d.abort) return;
    const int ld = d.ld, nlev = d.nlev;
    const AxiLevel &L1 = d.lev[1];
    const int n1 = L1.n1, n2 = L1.n2;
    double *psi = d.f[GB_A_phi];
    const double *rhs = d.f[GB_A_omegn];
    const int tp = (n1 + 1) * (n2 + 1);
    for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
        const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
        L1.f[idx] = rhs[AX(i, j)];
        L1.v[idx] = psi[AX(i, j)];
        d.rc[AX(i, j)] = 0.0;
    }
    __syncthreads();
    int status = GB_MAXSWEEPS, sweeps = d.maxsweeps, nan1 = 0, nn = 0;
    double res1 = 0.0;
    for (int sweep = 1; sweep <= d.maxsweeps; ++sweep) {
        if (sweep == 1 || nlev == 1) res1 = axi_relax(d, 1, s_red, &nan1);
        if (nlev > 1) {
            for (int l = 1; l <= nlev - 1; ++l) {
                axi_corser(d, l);
                axi_relax(d, l + 1, s_red, &nn);
            }
            for (int l = nlev; l >= 2; --l) {
                axi_finer(d, l);
                const double r = axi_relax(d, l - 1, s_red, &nn);
                if (l - 1 == 1) { res1 = r; nan1 = nn; }
            }
        }
        if (nan1) { status = GB_NAN; sweeps = sweep; break; }
        if (res1 < d.tolcon) {
            for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
                const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
                psi[AX(i, j)] = d.psif[AX(i, j)];
            }
            status = GB_OK;
            sweeps = sweep;
            break;
        }
    }
    if (threadIdx.x == 0) {
        d.status[0] = status;
        d.status[1] = sweeps;
        if (status == GB_NAN) *d.abort = 1;
    }
}

__global__ void __maxnreg__(128) k_axi_mg_solve(AxiDev d) { k_axi_mg_solve_body(d, blockIdx.x); }

// ---------------------------------------------------------------------------
// Mixed precision: FP64 defect correction around one FP32 V-cycle of the
// reference's schedule (relax on the finest level, down, up) on A e = r from
// e = 0; psi += e in FP64 (AXI has no over-relaxation).  Zebra colours stage
// their lines in shared memory ([row][line], odd pitch) for the elimination.
// ---------------------------------------------------------------------------
#define AX32_LINE_FLOATS 24576
#define AX32_SMEM_BYTES (AX32_LINE_FLOATS * 4)

__device__ __forceinline__ void tdma32_pitch(const float *fac, int n, float *x, int pitch)
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

// right-hand side of r-line j (dir 0) or z-line i (dir 1) at row q+1
__device__ __forceinline__ float axi_rhs32(const AxiDev &d, const AxiLevel &L, int dir, int line, int q)
{
    const int ld = d.ld, n1 = L.n1;
    const float *psif = d.psif32;
    if (dir == 0) {
        const int i = q + 1, j = line;
        return -(psif[AX(i, j + 1)] + psif[AX(i, j - 1)]) / (float)L.hhz + L.f32[(size_t)j * (n1 + 1) + i];
    }
    const int i = line, j = q + 1;
    const float rv = d.rval32[i * L.lf];
    return -(psif[AX(i + 1, j)] + psif[AX(i - 1, j)]) / (float)L.hhr + L.f32[(size_t)j * (n1 + 1) + i] -
           (psif[AX(i + 1, j)] - psif[AX(i - 1, j)]) * 0.5f / rv / (float)L.hr;
}

// one colour of zebra lines in direction dir, staged in shared memory
__device__ void axi_colour32(const AxiDev &d, const AxiLevel &L, int dir, int parity)
{
    extern __shared__ float s_ax32[];
    const int ld = d.ld;
    const int nlen = dir == 0 ? L.n1 - 1 : L.n2 - 1;       // rows of a line
    const int nl_all = dir == 0 ? L.n2 - 1 : L.n1 - 1;     // lines 1..nl_all
    const int nlines = (nl_all + parity) / 2;              // lines 2t + 2 - parity
    int B = AX32_LINE_FLOATS / nlen - 1;
    if (B > nlines) B = nlines;
    for (int b0 = 0; b0 < nlines; b0 += B) {
        const int nb = (nlines - b0 < B) ? nlines - b0 : B;
        const int pitch = nb | 1;
        for (int t = threadIdx.x >> 5; t < nb; t += blockDim.x >> 5) {
            const int line = 2 * (b0 + t) + 2 - parity;
            for (int q = threadIdx.x & 31; q < nlen; q += 32) s_ax32[q * pitch + t] = axi_rhs32(d, L, dir, line, q);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < nb; t += blockDim.x) {
            const int line = 2 * (b0 + t) + 2 - parity;
            const float *fac = dir == 0 ? L.fac_r32 : L.fac_z32 + (size_t)(line - 1) * 3 * nlen;
            tdma32_pitch(fac, nlen, s_ax32 + t, pitch);
        }
        __syncthreads();
        for (int t = threadIdx.x >> 5; t < nb; t += blockDim.x >> 5) {
            const int line = 2 * (b0 + t) + 2 - parity;
            for (int q = threadIdx.x & 31; q < nlen; q += 32) {
                const float v = s_ax32[q * pitch + t];
                if (dir == 0) d.psif32[AX(q + 1, line)] = v;
                else d.psif32[AX(line, q + 1)] = v;
            }
        }
        __syncthreads();
    }
}

// one line of the lexicographic order, marched by one thread
__device__ void axi_line32_lex(const AxiDev &d, const AxiLevel &L, int dir, int line)
{
    const int ld = d.ld;
    const int nlen = dir == 0 ? L.n1 - 1 : L.n2 - 1;
    const float *fac = dir == 0 ? L.fac_r32 : L.fac_z32 + (size_t)(line - 1) * 3 * nlen;
    float *x = dir == 0 ? d.psif32 + AX(1, line) : d.psif32 + AX(line, 1);
    const int stride = dir == 0 ? 1 : ld;
    const float *fact = fac, *ibp = fac + nlen, *c = fac + 2 * nlen;
    float prev = axi_rhs32(d, L, dir, line, 0);
    x[0] = prev;
    for (int q = 1; q < nlen; ++q) {
        prev = axi_rhs32(d, L, dir, line, q) - fact[q] * prev;
        x[(size_t)q * stride] = prev;
    }
    float y = prev * ibp[nlen - 1];
    x[(size_t)(nlen - 1) * stride] = y;
    for (int q = nlen - 2; q >= 0; --q) {
        y = (x[(size_t)q * stride] - c[q] * y) * ibp[q];
        x[(size_t)q * stride] = y;
    }
}

__device__ void axi_relax32(const AxiDev &d, int klev)
{
    const AxiLevel &L = d.lev[klev];
    const int ld = d.ld, n1 = L.n1, n2 = L.n2;
    for (int j = threadIdx.x >> 5; j <= n2; j += blockDim.x >> 5)
        for (int i = threadIdx.x & 31; i <= n1; i += 32) d.psif32[AX(i, j)] = L.v32[(size_t)j * (n1 + 1) + i];
    __syncthreads();
    const float hhr = (float)L.hhr, hhz = (float)L.hhz, hr = (float)L.hr;
    const float drdz = 2.0f * (1.0f / hhr + 1.0f / hhz);
    for (int irel = 0; irel < d.nrel; ++irel) {
        if (d.mode == GB_SMOOTHER_LEX) {
            if (threadIdx.x == 0)
                for (int j = 1; j <= n2 - 1; ++j) axi_line32_lex(d, L, 0, j);
            __syncthreads();
            if (threadIdx.x == 0)
                for (int i = 1; i <= n1 - 1; ++i) axi_line32_lex(d, L, 1, i);
            __syncthreads();
        } else {
            for (int par = 1; par >= 0; --par) axi_colour32(d, L, 0, par);
            for (int par = 1; par >= 0; --par) axi_colour32(d, L, 1, par);
        }
    }
    const float *psif = d.psif32;
    for (int j = 1 + (threadIdx.x >> 5); j <= n2 - 1; j += blockDim.x >> 5)
        for (int i = 1 + (threadIdx.x & 31); i <= n1 - 1; i += 32) {
            const float rv = d.rval32[i * L.lf];
            const float a = (psif[AX(i + 1, j)] + psif[AX(i - 1, j)]) / hhr +
                            (psif[AX(i + 1, j)] - psif[AX(i - 1, j)]) * 0.5f / hr / rv - psif[AX(i, j)] / (rv * rv) +
                            (psif[AX(i, j + 1)] + psif[AX(i, j - 1)]) / hhz - psif[AX(i, j)] * drdz;
            d.rc32[AX(i, j)] = L.f32[(size_t)j * (n1 + 1) + i] - a;
        }
    for (int j = threadIdx.x >> 5; j <= n2; j += blockDim.x >> 5)
        for (int i = threadIdx.x & 31; i <= n1; i += 32) L.v32[(size_t)j * (n1 + 1) + i] = psif[AX(i, j)];
    __syncthreads();
}

__device__ void axi_corser32(const AxiDev &d, int klev)
{
    const int ld = d.ld;
    const int n1c = d.lev[klev + 1].n1, n2c = d.lev[klev + 1].n2;
    const float *rf = d.rc32;
    float *fc = d.lev[klev + 1].f32, *vc = d.lev[klev + 1].v32;
    for (int j = threadIdx.x >> 5; j <= n2c; j += blockDim.x >> 5)
        for (int i = threadIdx.x & 31; i <= n1c; i += 32) {
            float t = 0.f;
            if (i >= 1 && i <= n1c - 1 && j >= 1 && j <= n2c - 1 && j != n1c) {
                const int ii = i + i, jj = j + j;
                t = 0.25f * rf[AX(ii, jj)] +
                    0.125f * (rf[AX(ii + 1, jj)] + rf[AX(ii - 1, jj)] + rf[AX(ii, jj + 1)] + rf[AX(ii, jj - 1)]) +
                    0.0625f * (rf[AX(ii + 1, jj + 1)] + rf[AX(ii - 1, jj - 1)] + rf[AX(ii + 1, jj - 1)] +
                               rf[AX(ii - 1, jj + 1)]);
            }
            fc[(size_t)j * (n1c + 1) + i] = t;
            vc[(size_t)j * (n1c + 1) + i] = 0.f;
        }
    __syncthreads();
}

__device__ void axi_finer32(const AxiDev &d, int klev)
{
    const int ld = d.ld;
    const int n1c = d.lev[klev].n1, n2c = d.lev[klev].n2;
    const int n1f = d.lev[klev - 1].n1, n2f = d.lev[klev - 1].n2;
    const float *vc = d.lev[klev].v32;
    float *vf = d.lev[klev - 1].v32, *psif = d.psif32;
#define PC32(ii, jj) vc[(size_t)(jj) * (n1c + 1) + (ii)]
    for (int j = threadIdx.x >> 5; j <= n2f; j += blockDim.x >> 5)
        for (int i = threadIdx.x & 31; i <= n1f; i += 32) {
            const int i1 = i / 2, j1 = j / 2;
            float p;
            if (i1 * 2 == i) p = (j1 * 2 == j) ? PC32(i1, j1) : (PC32(i1, j1) + PC32(i1, j1 + 1)) * 0.5f;
            else if (j1 * 2 == j) p = (PC32(i1, j1) + PC32(i1 + 1, j1)) * 0.5f;
            else p = (PC32(i1, j1) + PC32(i1 + 1, j1 + 1) + PC32(i1, j1 + 1) + PC32(i1 + 1, j1)) * 0.25f;
            psif[AX(i, j)] = p + vf[(size_t)j * (n1f + 1) + i];
        }
#undef PC32
    __syncthreads();
    for (int q = threadIdx.x; q < (n1c + 1) * (n2c + 1); q += blockDim.x) d.lev[klev].v32[q] = 0.f;
    for (int j = threadIdx.x >> 5; j <= n2f; j += blockDim.x >> 5)
        for (int i = threadIdx.x & 31; i <= n1f; i += 32) vf[(size_t)j * (n1f + 1) + i] = psif[AX(i, j)];
    __syncthreads();
}

__device__ __forceinline__ void k_axi_mg_solve_mixed_body(const AxiDev &d, int bidx)
{
    __shared__ double s_red[33];
    if (*d.abort) return;
    const int ld = d.ld, nlev = d.nlev;
    const AxiLevel &L1 = d.lev[1];
    const int n1 = L1.n1, n2 = L1.n2;
    double *psi = d.f[GB_A_phi], *psif = d.psif;
    const double *rhs = d.f[GB_A_omegn];
    for (int idx = threadIdx.x; idx < (n1 + 1) * (n2 + 1); idx += blockDim.x) {
        const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
        L1.f[idx] = rhs[AX(i, j)];
        psif[AX(i, j)] = psi[AX(i, j)];
    }
    __syncthreads();
    const double hhr = L1.hhr, hhz = L1.hhz, hr = L1.hr;
    const double drdz = 2.0 * (1.0 / hhr + 1.0 / hhz);
    const int ni = n1 - 1, tot = ni * (n2 - 1);
    int status = GB_MAXSWEEPS, cycles = 0;
    for (int it = 0;; ++it) {
        // FP64 residual of the iterate (the relax residual, rotann2.f:727-741)
        double m = 0.0;
        int nan = 0;
        for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
            const int j = idx / ni + 1, i = idx - (j - 1) * ni + 1;
            const double rv = d.rval[i];
            double temp = (psif[AX(i + 1, j)] + psif[AX(i - 1, j)]) / hhr +
                          (psif[AX(i + 1, j)] - psif[AX(i - 1, j)]) * 0.5 / hr / rv - psif[AX(i, j)] / (rv * rv) +
                          (psif[AX(i, j + 1)] + psif[AX(i, j - 1)]) / hhz - psif[AX(i, j)] * drdz;
            temp = L1.f[(size_t)j * (n1 + 1) + i] - temp;
            L1.f32[(size_t)j * (n1 + 1) + i] = (float)temp;
            temp = fabs(temp);
            if (temp != temp) nan = 1;
            if (temp > m) m = temp;
        }
        nan = __syncthreads_or(nan);
        const double res = axi_blk_max(m, s_red);
        if (nan) { status = GB_NAN; break; }
        if (res < d.tolcon) { status = GB_OK; break; }
        if (it == d.maxsweeps) break;
        for (int q = threadIdx.x; q < (n1 + 1) * (n2 + 1); q += blockDim.x) L1.v32[q] = 0.f;
        __syncthreads();
        axi_relax32(d, 1);
        if (nlev > 1) {
            for (int l = 1; l <= nlev - 1; ++l) {
                axi_corser32(d, l);
                axi_relax32(d, l + 1);
            }
            for (int l = nlev; l >= 2; --l) {
                axi_finer32(d, l);
                axi_relax32(d, l - 1);
            }
        }
        for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
            const int j = idx / ni + 1, i = idx - (j - 1) * ni + 1;
            psif[AX(i, j)] += (double)L1.v32[(size_t)j * (n1 + 1) + i];
        }
        __syncthreads();
        cycles = it + 1;
    }
    if (status == GB_OK)
        for (int idx = threadIdx.x; idx < (n1 + 1) * (n2 + 1); idx += blockDim.x) {
            const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
            psi[AX(i, j)] = psif[AX(i, j)];
        }
    if (threadIdx.x == 0) {
        d.status[0] = status;
        d.status[1] = cycles;
        if (status == GB_NAN) *d.abort = 1;
    }
}

__global__ void __maxnreg__(128) k_axi_mg_solve_mixed(AxiDev d) { k_axi_mg_solve_mixed_body(d, blockIdx.x); }

// FP32 copies of rval and the factors (pivots as reciprocals).
// FP32 copies of the factors (pivots as reciprocals): block l - 1 converts
// level l, its threads the level's lines (thread 0 also the r-line table).
__global__ void k_axi_factors32(AxiDev d)
{
    const int l = 1 + blockIdx.x;
    if (l == 1)
        for (int i = threadIdx.x; i <= d.lev[1].n1; i += blockDim.x) d.rval32[i] = (float)d.rval[i];
    const AxiLevel &L = d.lev[l];
    auto conv = [](const double *f, float *g, int n) {
        for (int j = 0; j < n; ++j) {
            g[j] = (float)f[j];
            g[n + j] = (float)(1.0 / f[n + j]);
            g[2 * n + j] = (float)f[2 * n + j];
        }
    };
    if (threadIdx.x == 0 && L.n1 - 1 >= 1) conv(L.fac_r, L.fac_r32, L.n1 - 1);
    if (L.n2 - 1 >= 1)
        for (int i = 1 + threadIdx.x; i <= L.n1 - 1; i += blockDim.x)
            conv(L.fac_z + (size_t)(i - 1) * tdma_fac_len(L.n2 - 1), L.fac_z32 + (size_t)(i - 1) * 3 * (L.n2 - 1),
                 L.n2 - 1);
}

__global__ void k_axi_rval(AxiDev d)
{
    for (int i = threadIdx.x; i <= d.lev[1].n1; i += blockDim.x) d.rval[i] = (double)i * d.lev[1].hr + d.r0;
}

// The factored line matrices of every level, with the coefficients relax
// forms for each line (rotann2.f:698-721): block l - 1 takes level l; its
// thread 0 the r-line matrix (work: three arrays per level), every thread
// the z-line matrices of its rows, whose coefficients are constant along the
// line (the tdma factorization with scalar a, b, c, the same operations).
__global__ void k_axi_factors(AxiDev d, double *work)
{
    const int l = 1 + blockIdx.x;
    const AxiLevel &L = d.lev[l];
    const int n1 = L.n1, n2 = L.n2;
    const double hhr = L.hhr, hhz = L.hhz, hr = L.hr;
    const int nmax = (d.lev[1].n1 > d.lev[1].n2 ? d.lev[1].n1 : d.lev[1].n2) + 2;
    if (threadIdx.x == 0 && n1 - 1 >= 1) {
        double *a = work + (size_t)blockIdx.x * 3 * nmax, *b = a + nmax, *c = b + nmax;
        for (int i = 1; i <= n1 - 1; ++i) {
            const double rv = d.rval[i * L.lf];
            a[i - 1] = 1.0 / hhr - 0.5 / hr / rv;
            c[i - 1] = 1.0 / hhr + 0.5 / hr / rv;
            b[i - 1] = -2.0 / hhr - 2.0 / hhz - 1.0 / (rv * rv);
        }
        factor_tdma(a, b, c, n1 - 1, L.fac_r);
    }
    const int n = n2 - 1;
    if (n < 1) return;
    for (int i = 1 + threadIdx.x; i <= n1 - 1; i += blockDim.x) {
        const double rv = d.rval[i * L.lf];
        const double av = 1.0 / hhz, cv = 1.0 / hhz;
        const double bv = -2.0 / hhr - 2.0 / hhz - 1.0 / (rv * rv);
        double *fac = L.fac_z + (size_t)(i - 1) * tdma_fac_len(n);
        double *fact = fac, *bp = fac + n, *cc = fac + 2 * n, *ibp = fac + 3 * n;
        bp[0] = bv;
        fact[0] = 0.0;
        for (int j = 0; j < n; ++j) cc[j] = cv;
        for (int j = 1; j < n; ++j) {
            fact[j] = av / bp[j - 1];
            bp[j] = bv - fact[j] * cv;
        }
        for (int j = 0; j < n; ++j) ibp[j] = 1.0 / bp[j];
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct gb_axi {
    gb_axi_params p;
    AxiDev dev;
    gb_str *str = nullptr;              // stretched grid: rcsc.f's multigrid for the streamfunction
    double *stab = nullptr;             // stretched grid: the transport's tables (AxsTab)
    double *fields = nullptr, *pool = nullptr;
    void *small = nullptr, *hist = nullptr;
    int hist_cap = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    gb_axi_params graph_params;
    double dr_set = 0.0, dz_set = 0.0;   // a Fortran caller's /num/ spacings, 0 = derived
};

static int axi_levels(int nr, int nz)
{
    int nlev = 0, it = nr, it2 = nr, jt = nz, jt2 = nz;
    for (int i = 2; i <= 8; ++i) {
        it = it / 2;
        jt = jt / 2;
        if (it * 2 - it2 == 0 && jt * 2 - jt2 == 0) {
            nlev = nlev + 1;
            it2 = it;
            jt2 = jt;
        } else {
            break;
        }
    }
    if (nlev > 6) nlev = 6;
    return nlev;
}

extern "C" void gb_axi_default_params(gb_axi_params *p, int nr, int nz)
{
    memset(p, 0, sizeof(*p));
    p->nr = nr;
    p->nz = nz;
    p->dt = 1e-5;
    p->r0 = 0.5;
    p->rmax = 1.0;
    p->zmax = 0.5;
    p->Ra = 1e5;
    p->Re = 1e2;
    p->Pr = 1.0;
    p->tolcon = 1.0e-6;
    p->maxsweeps = 10000;
    p->nrel = 2;
    p->smoother = GB_SMOOTHER_LEX;
    p->precision = GB_PRB_FP64;
}

static void axi_scalars(gb_axi *h)
{
    AxiDev &d = h->dev;
    const gb_axi_params &p = h->p;
    d.dt = p.dt;
    d.r0 = p.r0;
    d.rmax = p.rmax;
    d.zmax = p.zmax;
    d.Ra = p.Ra;
    d.Re = p.Re;
    d.Ptl = p.Pr;
    d.dr = h->dr_set != 0.0 ? h->dr_set : (p.rmax - p.r0) / (double)p.nr;
    d.dz = h->dz_set != 0.0 ? h->dz_set : p.zmax / (double)p.nz;
    const double dr = d.dr, dz = d.dz, Ptl = p.Pr, dt = p.dt;
    d.cf1 = 1.0 / (2.0 * Ptl * dt) + 1.0 / (dr * dr) + 1.0 / (dz * dz);
    d.cf2 = 1.0 / (2.0 * Ptl * dt) - 1.0 / (dr * dr) - 1.0 / (dz * dz);
    d.cf3 = 1.0 / (2.0 * dt) + 1.0 / (dr * dr) + 1.0 / (dz * dz);
    d.cf4 = 1.0 / (2.0 * dt) - 1.0 / (dr * dr) - 1.0 / (dz * dz);
    d.tolcon = p.tolcon;
    d.maxsweeps = p.maxsweeps;
    d.nrel = p.nrel;
    d.mode = p.smoother;
    d.nu_c = -p.r0 * log(p.r0 / p.rmax);
    d.nu_d = p.zmax * p.rmax;
}

extern "C" int gb_axi_destroy(gb_axi *h)
{
    if (!h) return GB_OK;
    if (h->graph) cudaGraphExecDestroy(h->graph);
    if (h->str) gb_str_destroy(h->str);
    cudaFree(h->stab);
    cudaFree(h->fields);
    cudaFree(h->pool);
    cudaFree(h->small);
    cudaFree(h->hist);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return GB_OK;
}

static int axi_create(const gb_axi_params *p, double dr, double dz, gb_axi **out, int *nlev_out);

extern "C" int gb_axi_create(const gb_axi_params *p, gb_axi **out, int *nlev_out)
{
    return axi_create(p, 0.0, 0.0, out, nlev_out);
}

extern "C" int gb_axi_create_spacing(const gb_axi_params *p, double dr, double dz, gb_axi **out, int *nlev_out)
{
    if (!(dr > 0.0 && dz > 0.0)) {
        gb_set_error("gb_axi_create_spacing: spacings must be positive");
        return GB_ERR_INVALID;
    }
    return axi_create(p, dr, dz, out, nlev_out);
}

static int axi_create(const gb_axi_params *p, double dr, double dz, gb_axi **out, int *nlev_out)
{
    if (!p || !out) { gb_set_error("gb_axi_create: null argument"); return GB_ERR_INVALID; }
    *out = nullptr;
    const int nr = p->nr, nz = p->nz;
    const int nlev = axi_levels(nr, nz);
    if (nlev_out) *nlev_out = nlev;
    if (nr < 4 || nz < 4 || nlev < 1 || nr > 8192 || nz > 8192 || !(p->r0 > 0.0 && p->rmax > p->r0) ||
        !(p->zmax > 0.0) || p->nrel < 1 || p->maxsweeps < 1 || p->Re == 0.0) {
        gb_set_error("gb_axi_create: unsupported parameters (nr=%d nz=%d need both even with >= 1 multigrid level; "
                     "0 < r0 < rmax, zmax > 0, Re != 0)", nr, nz);
        return GB_ERR_INVALID;
    }
    if (p->precision != GB_PRB_FP64 && p->precision != GB_PRB_MIXED) {
        gb_set_error("gb_axi_create: unknown precision %d", p->precision);
        return GB_ERR_INVALID;
    }
    if (2 * (nr > nz ? nr : nz) > AX32_LINE_FLOATS) {
        gb_set_error("gb_axi_create: nr=%d nz=%d exceed the shared-memory line buffer", nr, nz);
        return GB_ERR_INVALID;
    }
    gb_axi *h = new gb_axi();
    h->p = *p;
    h->dr_set = dr;
    h->dz_set = dz;
    AxiDev &d = h->dev;
    memset(&d, 0, sizeof(d));
    d.nr = nr;
    d.nz = nz;
    d.ld = nr + 1;
    d.nlev = nlev;
    axi_scalars(h);
    const size_t fsz = (size_t)d.ld * (size_t)(nz + 1);
    cudaError_t e = cudaMalloc(&h->fields, sizeof(double) * fsz * GB_A_COUNT);
    if (e != cudaSuccess) { gb_set_error("gb_axi_create: %s", cudaGetErrorString(e)); delete h; return GB_ERR_ALLOC; }
    cudaMemset(h->fields, 0, sizeof(double) * fsz * GB_A_COUNT);
    for (int q = 0; q < GB_A_COUNT; ++q) d.f[q] = h->fields + (size_t)q * fsz;
    // pool: rval, psif, rc, then per level v, f, fac_r, fac_z; work for the factors
    size_t need = (size_t)(nr + 2) + 2 * fsz + fsz + (size_t)(nr + 2) / 2 + 8;   // + psif32, rc32, rval32
    for (int l = 1; l <= nlev; ++l) {
        const size_t n1 = (size_t)nr * 2 / ((size_t)1 << l), n2 = (size_t)nz * 2 / ((size_t)1 << l);
        const size_t lv = 2 * (n1 + 1) * (n2 + 1) + 4 * n1 + n1 * 4 * (n2 + 1);
        need += lv + (lv + 1) / 2 + 4;   // FP64 slots, then their FP32 copies
    }
    const size_t work = 3 * (size_t)((nr > nz ? nr : nz) + 2) * (size_t)nlev;   // r-line coefficients, per level
    e = cudaMalloc(&h->pool, sizeof(double) * (need + work));
    if (e != cudaSuccess) { gb_axi_destroy(h); gb_set_error("gb_axi_create: multigrid pool"); return GB_ERR_ALLOC; }
    cudaMemset(h->pool, 0, sizeof(double) * (need + work));
    double *b = h->pool;
    d.rval = b; b += nr + 2;
    d.psif = b; b += fsz;
    d.rc = b; b += fsz;
    {
        float *fb = (float *)b;
        d.psif32 = fb; fb += fsz;
        d.rc32 = fb; fb += fsz;
        d.rval32 = fb; fb += nr + 2;
        b = (double *)(((uintptr_t)fb + 15) & ~(uintptr_t)15);
    }
    for (int l = 1; l <= nlev; ++l) {
        AxiLevel &L = d.lev[l];
        L.n1 = nr * 2 / (1 << l);
        L.n2 = nz * 2 / (1 << l);
        L.lf = (1 << l) / 2;
        L.hr = d.dr * (double)(1 << l) / 2.0;
        L.hz = d.dz * (double)(1 << l) / 2.0;
        L.hhr = L.hr * L.hr;
        L.hhz = L.hz * L.hz;
        const size_t sz = (size_t)(L.n1 + 1) * (L.n2 + 1);
        L.v = b; b += sz;
        L.f = b; b += sz;
        L.fac_r = b; b += 4 * (size_t)L.n1;                          // tdma_fac_len(n1 - 1) and more
        L.fac_z = b; b += (size_t)L.n1 * 4 * (size_t)(L.n2 + 1);
        float *fb = (float *)b;
        L.v32 = fb; fb += sz;
        L.f32 = fb; fb += sz;
        L.fac_r32 = fb; fb += 3 * (size_t)L.n1;
        L.fac_z32 = fb; fb += (size_t)L.n1 * 3 * (size_t)(L.n2 + 1);
        b = (double *)(((uintptr_t)fb + 15) & ~(uintptr_t)15);
    }
    if ((size_t)(b - h->pool) > need) {
        gb_axi_destroy(h);
        gb_set_error("gb_axi_create: multigrid pool layout overflow");
        return GB_ERR_CUDA;
    }
    double *wk = h->pool + need;
    e = cudaMalloc(&h->small, 4096);
    if (e != cudaSuccess) { gb_axi_destroy(h); gb_set_error("gb_axi_create: state"); return GB_ERR_ALLOC; }
    cudaMemset(h->small, 0, 4096);
    char *sm = (char *)h->small;
    d.heat = (double *)(sm + 0);
    d.errmax = (unsigned long long *)(sm + 64);
    d.abort = (int *)(sm + 128);
    d.status = (int *)(sm + 192);
    d.step_index = (int *)(sm + 256);
    k_axi_rval<<<1, 256>>>(d);
    k_axi_factors<<<d.nlev, 128>>>(d, wk);
    k_axi_factors32<<<d.nlev, 128>>>(d);
    e = cudaFuncSetAttribute(k_axi_mg_solve_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, AX32_SMEM_BYTES);
    if (e != cudaSuccess) { gb_axi_destroy(h); gb_set_error("gb_axi_create: %s", cudaGetErrorString(e)); return GB_ERR_CUDA; }
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { gb_axi_destroy(h); gb_set_error("gb_axi_create: stream"); return GB_ERR_CUDA; }
    e = cudaStreamSynchronize(0);   // the creation's kernels and copies, not other instances' streams
    if (e != cudaSuccess) { gb_set_error("gb_axi_create: %s", cudaGetErrorString(e)); gb_axi_destroy(h); return GB_ERR_CUDA; }
    *out = h;
    return GB_OK;
}

// The annulus on a stretched grid: the state, its transport tables and the
// stretched multigrid; no uniform multigrid.
extern "C" int gb_axi_create_stretched(const gb_axi_params *p, const gb_axi_grid *g, gb_axi **out, int *nlev_out)
{
    if (!p || !g || !out || !g->levels || !g->z || !g->cz || !g->hw) {
        gb_set_error("gb_axi_create_stretched: null argument");
        return GB_ERR_INVALID;
    }
    *out = nullptr;
    const int nr = p->nr, nz = p->nz;
    const gb_str_level &L1 = g->levels[0];
    if (g->nlev < 1 || L1.n1 != nr || L1.n2 != nz || nr < 4 || nz < 4 || !L1.r || !L1.cr || !L1.crr || !L1.czz ||
        !(p->zmax > 0.0) || p->nrel < 1 || p->maxsweeps < 1 || p->Re == 0.0 ||
        (p->precision != GB_PRB_FP64 && p->precision != GB_PRB_MIXED)) {
        gb_set_error("gb_axi_create_stretched: level 1 must be %d x %d with all tables (nr, nz >= 4, zmax > 0, "
                     "Re != 0, FP64 or mixed)", nr, nz);
        return GB_ERR_INVALID;
    }
    gb_axi *h = new gb_axi();
    h->p = *p;
    AxiDev &d = h->dev;
    memset(&d, 0, sizeof(d));
    d.nr = nr;
    d.nz = nz;
    d.ld = nr + 1;
    d.nlev = g->nlev;
    d.stretched = 1;
    axi_scalars(h);
    int st = gb_str_create(g->nlev, g->levels, p->tolcon, p->maxsweeps, p->nrel, p->smoother, &h->str);
    if (st != GB_OK) { delete h; return st; }
    const size_t fsz = (size_t)d.ld * (size_t)(nz + 1);
    cudaError_t e = cudaMalloc(&h->fields, sizeof(double) * fsz * GB_A_COUNT);
    if (e != cudaSuccess) { gb_axi_destroy(h); gb_set_error("gb_axi_create_stretched: %s", cudaGetErrorString(e)); return GB_ERR_ALLOC; }
    cudaMemset(h->fields, 0, sizeof(double) * fsz * GB_A_COUNT);
    for (int q = 0; q < GB_A_COUNT; ++q) d.f[q] = h->fields + (size_t)q * fsz;
    const size_t ntab = (size_t)(nr + 1) + (nz + 1) + 3 * (size_t)(nr - 1) + 4 * (size_t)(nr - 1) + 3 * (size_t)(nz - 1) +
                        4 * (size_t)(nz - 1);
    e = cudaMalloc(&h->stab, sizeof(double) * ntab);
    if (e != cudaSuccess) { gb_axi_destroy(h); gb_set_error("gb_axi_create_stretched: tables"); return GB_ERR_ALLOC; }
    double *b = h->stab;
    auto put = [&](const double *src, size_t n) {
        double *dst = b;
        cudaMemcpy(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice);
        b += n;
        return (const double *)dst;
    };
    d.st.r = put(L1.r, (size_t)nr + 1);
    d.st.z = put(g->z, (size_t)nz + 1);
    d.st.cr = put(L1.cr, 3 * (size_t)(nr - 1));
    d.st.crr = put(L1.crr, 4 * (size_t)(nr - 1));
    d.st.cz = put(g->cz, 3 * (size_t)(nz - 1));
    d.st.czz = put(L1.czz, 4 * (size_t)(nz - 1));
    for (int q = 0; q < 5; ++q) d.st.hw[q] = g->hw[q];
    e = cudaMalloc(&h->small, 4096);
    if (e != cudaSuccess) { gb_axi_destroy(h); gb_set_error("gb_axi_create_stretched: state"); return GB_ERR_ALLOC; }
    cudaMemset(h->small, 0, 4096);
    char *sm = (char *)h->small;
    d.heat = (double *)(sm + 0);
    d.errmax = (unsigned long long *)(sm + 64);
    d.abort = (int *)(sm + 128);
    d.status = (int *)(sm + 192);
    d.step_index = (int *)(sm + 256);
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) { gb_axi_destroy(h); gb_set_error("gb_axi_create_stretched: %s", cudaGetErrorString(e)); return GB_ERR_CUDA; }
    if (nlev_out) *nlev_out = g->nlev;
    *out = h;
    return GB_OK;
}

extern "C" int gb_axi_set_field(gb_axi *h, int field, const double *host, int ld)
{
    if (!h || !host || field < 0 || field >= GB_A_COUNT || ld < h->dev.nr + 1) {
        gb_set_error("gb_axi_set_field: invalid argument");
        return GB_ERR_INVALID;
    }
    GB_CUDA_TRY(cudaMemcpy2DAsync(h->dev.f[field], sizeof(double) * h->dev.ld, host, sizeof(double) * (size_t)ld,
                                  sizeof(double) * (h->dev.nr + 1), h->dev.nz + 1, cudaMemcpyHostToDevice, h->stream));
    GB_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return GB_OK;
}

extern "C" int gb_axi_get_field(gb_axi *h, int field, double *host, int ld)
{
    if (!h || !host || field < 0 || field >= GB_A_COUNT || ld < h->dev.nr + 1) {
        gb_set_error("gb_axi_get_field: invalid argument");
        return GB_ERR_INVALID;
    }
    GB_CUDA_TRY(cudaMemcpy2DAsync(host, sizeof(double) * (size_t)ld, h->dev.f[field], sizeof(double) * h->dev.ld,
                                  sizeof(double) * (h->dev.nr + 1), h->dev.nz + 1, cudaMemcpyDeviceToHost, h->stream));
    GB_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return GB_OK;
}

extern "C" void *gb_axi_stream(gb_axi *h) { return h ? (void *)h->stream : nullptr; }

static const int AXI_TPB = 256;

static void axi_launch_vort_vel(gb_axi *h, int what, cudaStream_t s)
{
    const int n = (h->dev.nr - 1) * (h->dev.nz - 1);
    if (h->dev.stretched) k_axi_vort_vel<true><<<gb_ceil_div(n, AXI_TPB), AXI_TPB, 0, s>>>(h->dev, what);
    else k_axi_vort_vel<false><<<gb_ceil_div(n, AXI_TPB), AXI_TPB, 0, s>>>(h->dev, what);
}

static void axi_launch_temperature(gb_axi *h, cudaStream_t s)
{
    const int n = (h->dev.nr - 1) * (h->dev.nz + 1);
    if (h->dev.stretched) k_axi_temperature<true><<<gb_ceil_div(n, AXI_TPB), AXI_TPB, 0, s>>>(h->dev);
    else k_axi_temperature<false><<<gb_ceil_div(n, AXI_TPB), AXI_TPB, 0, s>>>(h->dev);
}

static void axi_launch_update(gb_axi *h, cudaStream_t s)
{
    const int n = (h->dev.nr + 1) * (h->dev.nz + 1);
    if (h->dev.stretched) k_axi_update<true><<<gb_ceil_div(n, AXI_TPB), AXI_TPB, 0, s>>>(h->dev);
    else k_axi_update<false><<<gb_ceil_div(n, AXI_TPB), AXI_TPB, 0, s>>>(h->dev);
}

static void axi_launch_heat(gb_axi *h, cudaStream_t s)
{
    if (h->dev.stretched) k_axi_heat<true><<<1, 256, sizeof(double) * (h->dev.nz + 1), s>>>(h->dev);
    else k_axi_heat<false><<<1, 256, sizeof(double) * (h->dev.nz + 1), s>>>(h->dev);
}

static void axi_launch_mg(gb_axi *h, cudaStream_t s)
{
    const AxiDev &d = h->dev;
    if (d.stretched) {
        gb_str_launch_device(h->str, d.f[GB_A_phi], d.f[GB_A_omegn], d.status, d.abort,
                             h->p.precision == GB_PRB_MIXED, d.tolcon, d.maxsweeps, d.nrel, d.mode, s);
        return;
    }
    if (h->p.precision == GB_PRB_MIXED) k_axi_mg_solve_mixed<<<1, AXI_THREADS, AX32_SMEM_BYTES, s>>>(h->dev);
    else k_axi_mg_solve<<<1, AXI_THREADS, 0, s>>>(h->dev);
}

static int axi_sync(gb_axi *h, const char *what)
{
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) { gb_set_error("%s: %s", what, cudaGetErrorString(e)); return GB_ERR_CUDA; }
    return GB_OK;
}

static void axi_begin(gb_axi *h)
{
    axi_scalars(h);
    cudaMemsetAsync(h->dev.abort, 0, sizeof(int), h->stream);
}

extern "C" int gb_axi_vorticity(gb_axi *h)
{
    if (!h) return GB_ERR_INVALID;
    axi_begin(h);
    axi_launch_vort_vel(h, 1, h->stream);
    return axi_sync(h, "gb_axi_vorticity");
}

extern "C" int gb_axi_velocity(gb_axi *h)
{
    if (!h) return GB_ERR_INVALID;
    axi_begin(h);
    axi_launch_vort_vel(h, 2, h->stream);
    return axi_sync(h, "gb_axi_velocity");
}

extern "C" int gb_axi_temperature(gb_axi *h)
{
    if (!h) return GB_ERR_INVALID;
    axi_begin(h);
    axi_launch_temperature(h, h->stream);
    return axi_sync(h, "gb_axi_temperature");
}

extern "C" int gb_axi_poisson(gb_axi *h, int *sweeps)
{
    if (!h) return GB_ERR_INVALID;
    axi_begin(h);
    axi_launch_mg(h, h->stream);
    int st[2] = {0, 0};
    GB_CUDA_TRY(cudaMemcpyAsync(st, h->dev.status, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    int r = axi_sync(h, "gb_axi_poisson");
    if (r != GB_OK) return r;
    if (sweeps) *sweeps = st[1];
    return st[0];
}

extern "C" int gb_axi_update(gb_axi *h)
{
    if (!h) return GB_ERR_INVALID;
    axi_begin(h);
    axi_launch_update(h, h->stream);
    GB_CUDA_TRY(cudaMemsetAsync(h->dev.errmax, 0, 3 * sizeof(unsigned long long), h->stream));
    return axi_sync(h, "gb_axi_update");
}

extern "C" int gb_axi_heat(gb_axi *h, double *trans)
{
    if (!h) return GB_ERR_INVALID;
    axi_begin(h);
    axi_launch_heat(h, h->stream);
    double t = 0.0;
    GB_CUDA_TRY(cudaMemcpyAsync(&t, h->dev.heat, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    int r = axi_sync(h, "gb_axi_heat");
    if (trans) *trans = t;
    return r;
}

static int axi_build_graph(gb_axi *h)
{
    cudaGraph_t g;
    GB_CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    axi_launch_vort_vel(h, 3, h->stream);
    axi_launch_temperature(h, h->stream);
    axi_launch_mg(h, h->stream);
    axi_launch_update(h, h->stream);
    axi_launch_heat(h, h->stream);
    k_axi_record<<<1, 32, 0, h->stream>>>(h->dev);
    GB_CUDA_TRY(cudaStreamEndCapture(h->stream, &g));
    GB_CUDA_TRY(cudaGraphInstantiate(&h->graph, g, 0));
    cudaGraphDestroy(g);
    return GB_OK;
}

// Asynchronous stepping (as for the 2D drivers).
extern "C" int gb_axi_run_begin(gb_axi *h, int nsteps_total)
{
    if (!h || nsteps_total < 0) { gb_set_error("gb_axi_run_begin: invalid argument"); return GB_ERR_INVALID; }
    AxiDev &d = h->dev;
    const int cap = nsteps_total > 0 ? nsteps_total : 1;
    if (h->hist_cap < cap) {
        cudaFree(h->hist);
        h->hist = nullptr;
        GB_CUDA_TRY(cudaMalloc(&h->hist, (sizeof(double) + sizeof(int)) * (size_t)cap));
        h->hist_cap = cap;
        if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    }
    d.nu_hist = (double *)h->hist;
    d.sweep_hist = (int *)((double *)h->hist + h->hist_cap);
    d.hist_cap = h->hist_cap;
    if (memcmp(&h->graph_params, &h->p, sizeof(gb_axi_params)) != 0) {
        if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
        h->graph_params = h->p;
        axi_scalars(h);
    }
    GB_CUDA_TRY(cudaMemsetAsync(d.abort, 0, sizeof(int), h->stream));
    GB_CUDA_TRY(cudaMemsetAsync(d.step_index, 0, sizeof(int), h->stream));
    GB_CUDA_TRY(cudaMemsetAsync(d.errmax, 0, 3 * sizeof(unsigned long long), h->stream));
    return GB_OK;
}

extern "C" int gb_axi_run_enqueue(gb_axi *h, int nsteps)
{
    if (!h || nsteps < 0) { gb_set_error("gb_axi_run_enqueue: invalid argument"); return GB_ERR_INVALID; }
    int st;
    if (!h->graph && (st = axi_build_graph(h)) != GB_OK) return st;
    for (int s = 0; s < nsteps; ++s) GB_CUDA_TRY(cudaGraphLaunch(h->graph, h->stream));
    return GB_OK;
}

extern "C" int gb_axi_run_query(gb_axi *h)
{
    if (!h) return -GB_ERR_INVALID;
    const cudaError_t e = cudaStreamQuery(h->stream);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) { cudaGetLastError(); return 0; }
    gb_set_error("gb_axi_run_query: %s", cudaGetErrorString(e));
    return -GB_ERR_CUDA;
}

extern "C" int gb_axi_run_end(gb_axi *h, int nsteps, double *nu, int *sweeps, int *steps_done)
{
    if (!h || nsteps < 0 || nsteps > h->hist_cap) { gb_set_error("gb_axi_run_end: invalid argument"); return GB_ERR_INVALID; }
    AxiDev &d = h->dev;
    int info[2] = {0, 0}, stat[2] = {0, 0};
    GB_CUDA_TRY(cudaMemcpyAsync(&info[0], d.step_index, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    GB_CUDA_TRY(cudaMemcpyAsync(&info[1], d.abort, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    GB_CUDA_TRY(cudaMemcpyAsync(stat, d.status, sizeof(stat), cudaMemcpyDeviceToHost, h->stream));
    std::vector<double> nuh((size_t)nsteps + 1);
    std::vector<int> swh((size_t)nsteps + 1);
    if (nsteps > 0) {
        GB_CUDA_TRY(cudaMemcpyAsync(nuh.data(), d.nu_hist, sizeof(double) * nsteps, cudaMemcpyDeviceToHost, h->stream));
        GB_CUDA_TRY(cudaMemcpyAsync(swh.data(), d.sweep_hist, sizeof(int) * nsteps, cudaMemcpyDeviceToHost, h->stream));
    }
    int st = axi_sync(h, "gb_axi_run_end");
    if (st != GB_OK) return st;
    if (nu) memcpy(nu, nuh.data(), sizeof(double) * nsteps);
    if (sweeps) memcpy(sweeps, swh.data(), sizeof(int) * nsteps);
    if (steps_done) *steps_done = info[0];
    if (info[1] == 1) {
        gb_set_error("gb_axi_step: multigrid failed at step %d (status %d)", info[0] + 1, stat[0]);
        return stat[0];
    }
    return GB_OK;
}

extern "C" int gb_axi_step(gb_axi *h, int nsteps, double *nu, int *sweeps, int *steps_done)
{
    if (!h || nsteps < 0) { gb_set_error("gb_axi_step: invalid argument"); return GB_ERR_INVALID; }
    if (steps_done) *steps_done = 0;
    if (nsteps == 0) return GB_OK;
    int st = gb_axi_run_begin(h, nsteps);
    if (st == GB_OK) st = gb_axi_run_enqueue(h, nsteps);
    if (st != GB_OK) return st;
    return gb_axi_run_end(h, nsteps, nu, sweeps, steps_done);
}

// ---------------------------------------------------------------------------
// Gangs of annulus instances of different grid sizes stepped together (as
// the PRB gangs in prb.cu): each phase of a step is one launch over all
// members' blocks, the streamfunction solves one launch of one block per
// member; every member runs its own kernel bodies, so its results are
// bit-identical to stepping it alone.  A member whose step index reaches
// its step count sets its abort flag to GB_RUN_DONE.
// ---------------------------------------------------------------------------
enum AxiGangPhase { AG_VV, AG_T, AG_MG, AG_UPD, AG_HEAT, AG_REC, AG_COUNT };

struct AxiGangTab {
    const AxiDev *dev;    // [n]
    const int *off;       // [AG_COUNT][n + 1]
    const int *limit;     // [n]
    int n;
};

__device__ __forceinline__ int axi_gang_member(const int *off, int n, int b)
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
__global__ void k_axi_gang(AxiGangTab g)
{
    const int *off = g.off + (size_t)PH * (g.n + 1);
    const int m = axi_gang_member(off, g.n, blockIdx.x);
    const AxiDev &d = g.dev[m];
    const int b = blockIdx.x - off[m];
    switch (PH) {
    case AG_VV: k_axi_vort_vel_body<false>(d, 3, b); break;
    case AG_T: k_axi_temperature_body<false>(d, b); break;
    case AG_UPD: k_axi_update_body<false>(d, b); break;
    case AG_HEAT: k_axi_heat_body<false>(d, b); break;
    case AG_REC:
        k_axi_record_body(d, b);
        if (threadIdx.x == 0 && b == 0 && *d.abort == 0 && *d.step_index >= g.limit[m]) *d.abort = GB_RUN_DONE;
        break;
    default: break;
    }
}

// Launched with AXI_THREADS (512) threads; 128 registers keep the solve
// free of spills (a launch bound of 512 threads left it at 40-64 with spills).
template <bool MIXED>
__global__ void __maxnreg__(128) k_axi_gang_mg(AxiGangTab g)
{
    const AxiDev &d = g.dev[blockIdx.x];
    if (MIXED) k_axi_mg_solve_mixed_body(d, 0);
    else k_axi_mg_solve_body(d, 0);
}

struct gb_axi_gang {
    int n = 0, mixed = 0;
    AxiDev *d_dev = nullptr;
    int *d_off = nullptr, *d_limit = nullptr;
    int blocks[AG_COUNT], threads[AG_COUNT];
    size_t heat_smem = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
};

extern "C" int gb_axi_gang_destroy(gb_axi_gang *g)
{
    if (!g) return GB_OK;
    if (g->graph) cudaGraphExecDestroy(g->graph);
    cudaFree(g->d_dev);
    cudaFree(g->d_off);
    cudaFree(g->d_limit);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
    return GB_OK;
}

extern "C" int gb_axi_gang_create(gb_axi *const *members, const int *nsteps_total, int n, gb_axi_gang **out)
{
    if (!members || !nsteps_total || n < 1 || !out) {
        gb_set_error("gb_axi_gang_create: invalid argument");
        return GB_ERR_INVALID;
    }
    *out = nullptr;
    const int mixed = members[0]->p.precision == GB_PRB_MIXED;
    for (int q = 0; q < n; ++q) {
        const gb_axi *h = members[q];
        if (!h || h->dev.stretched || (h->p.precision == GB_PRB_MIXED) != (mixed != 0) || nsteps_total[q] < 0 ||
            nsteps_total[q] > h->hist_cap) {
            gb_set_error("gb_axi_gang_create: member %d must be a uniform-grid instance of the gang's precision, after "
                         "gb_axi_run_begin with at least its step count", q);
            return GB_ERR_INVALID;
        }
    }
    gb_axi_gang *g = new gb_axi_gang();
    g->n = n;
    g->mixed = mixed;
    const int tpb[AG_COUNT] = {AXI_TPB, AXI_TPB, AXI_THREADS, AXI_TPB, 256, 32};
    std::vector<int> off((size_t)AG_COUNT * (n + 1));
    std::vector<AxiDev> devs(n);
    for (int ph = 0; ph < AG_COUNT; ++ph) {
        g->threads[ph] = tpb[ph];
        g->blocks[ph] = 0;
    }
    for (int q = 0; q < n; ++q) {
        gb_axi *h = members[q];
        axi_scalars(h);
        devs[q] = h->dev;
        const size_t nr = h->dev.nr, nz = h->dev.nz;
        const int nb[AG_COUNT] = {(int)gb_ceil_div((nr - 1) * (nz - 1), AXI_TPB), (int)gb_ceil_div((nr - 1) * (nz + 1), AXI_TPB),
                                  1, (int)gb_ceil_div((nr + 1) * (nz + 1), AXI_TPB), 1, 1};
        for (int ph = 0; ph < AG_COUNT; ++ph) {
            off[(size_t)ph * (n + 1) + q] = g->blocks[ph];
            g->blocks[ph] += nb[ph];
        }
        g->heat_smem = std::max(g->heat_smem, sizeof(double) * (nz + 1));
    }
    for (int ph = 0; ph < AG_COUNT; ++ph) off[(size_t)ph * (n + 1) + n] = g->blocks[ph];
#define GTRY(x)                                                                   \
    do {                                                                          \
        cudaError_t _e = (x);                                                     \
        if (_e != cudaSuccess) {                                                  \
            gb_set_error("gb_axi_gang_create: %s: %s", #x, cudaGetErrorString(_e)); \
            gb_axi_gang_destroy(g);                                               \
            return GB_ERR_CUDA;                                                   \
        }                                                                         \
    } while (0)
    GTRY(cudaMalloc(&g->d_dev, sizeof(AxiDev) * n));
    GTRY(cudaMalloc(&g->d_off, sizeof(int) * off.size()));
    GTRY(cudaMalloc(&g->d_limit, sizeof(int) * n));
    GTRY(cudaMemcpy(g->d_dev, devs.data(), sizeof(AxiDev) * n, cudaMemcpyHostToDevice));
    GTRY(cudaMemcpy(g->d_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice));
    GTRY(cudaMemcpy(g->d_limit, nsteps_total, sizeof(int) * n, cudaMemcpyHostToDevice));
    for (int q = 0; q < n; ++q) GTRY(cudaStreamSynchronize(members[q]->stream));
    GTRY(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    GTRY(cudaFuncSetAttribute(k_axi_gang_mg<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, AX32_SMEM_BYTES));
    if (g->heat_smem > 48 * 1024)
        GTRY(cudaFuncSetAttribute(k_axi_gang<AG_HEAT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g->heat_smem));
#undef GTRY
    *out = g;
    return GB_OK;
}

// Queues nsteps steps of every member (one CUDA graph launch per step) on
// `stream` (NULL: the gang's own).
extern "C" int gb_axi_gang_enqueue(gb_axi_gang *g, int nsteps, void *stream)
{
    if (!g || nsteps < 0) { gb_set_error("gb_axi_gang_enqueue: invalid argument"); return GB_ERR_INVALID; }
    cudaStream_t s = stream ? (cudaStream_t)stream : g->stream;
    if (!g->graph) {
        AxiGangTab t{g->d_dev, g->d_off, g->d_limit, g->n};
        cudaGraph_t gr;
        cudaStream_t cs = g->stream;
        GB_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        k_axi_gang<AG_VV><<<g->blocks[AG_VV], g->threads[AG_VV], 0, cs>>>(t);
        k_axi_gang<AG_T><<<g->blocks[AG_T], g->threads[AG_T], 0, cs>>>(t);
        if (g->mixed) k_axi_gang_mg<true><<<g->n, AXI_THREADS, AX32_SMEM_BYTES, cs>>>(t);
        else k_axi_gang_mg<false><<<g->n, AXI_THREADS, 0, cs>>>(t);
        k_axi_gang<AG_UPD><<<g->blocks[AG_UPD], g->threads[AG_UPD], 0, cs>>>(t);
        k_axi_gang<AG_HEAT><<<g->blocks[AG_HEAT], g->threads[AG_HEAT], g->heat_smem, cs>>>(t);
        k_axi_gang<AG_REC><<<g->blocks[AG_REC], g->threads[AG_REC], 0, cs>>>(t);
        GB_CUDA_TRY(cudaStreamEndCapture(cs, &gr));
        GB_CUDA_TRY(cudaGraphInstantiate(&g->graph, gr, 0));
        cudaGraphDestroy(gr);
    }
    for (int k = 0; k < nsteps; ++k) GB_CUDA_TRY(cudaGraphLaunch(g->graph, s));
    return GB_OK;
}

extern "C" void *gb_axi_gang_stream(gb_axi_gang *g) { return g ? (void *)g->stream : nullptr; }

extern "C" int gb_axi_gang_query(gb_axi_gang *g)
{
    if (!g) return -GB_ERR_INVALID;
    const cudaError_t e = cudaStreamQuery(g->stream);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) { cudaGetLastError(); return 0; }
    gb_set_error("gb_axi_gang_query: %s", cudaGetErrorString(e));
    return -GB_ERR_CUDA;
}
