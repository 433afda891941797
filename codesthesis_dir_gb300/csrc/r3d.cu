// 3D rotating annulus of rot3dmg.f on sm_103a: the Dufort-Frankel transport
// of the vorticity components A, B, C and the temperature, the wall
// vorticities, the right-hand sides of the three velocity Poisson equations,
// and their multigrid solves, FP64, bit-identical to the oracle (every
// expression in the reference's order, -fmad=false, IEEE division).
//
// Layout: every field is a (0:nr+1, 0:nz+1, 0:np) column-major array in HBM
// (i fastest), the reference's COMMON arrays cut to the run's size.  Each
// multigrid level holds its correction v, right-hand side f and residual
// res as (0:n1, 0:n2, 0:n3) arrays.
//
// Multigrid: one persistent cooperative launch per Poisson solve runs the
// whole sweep loop of poisson1/2/3.  A relaxation pass in one direction is
// a sequence of phases of independent lines separated by bounded grid
// barriers; each thread solves whole lines in place.  The line matrices
// depend only on the level and the line's radius, so the banded solvers'
// matrix eliminations are done once at creation (k_r3d_factors) and a line
// solve only carries its right-hand side through the recorded multipliers:
// the same operations, in the same order, as the reference's tdma, ptdma
// and pdma (rot3dmg.f:2570-2689).  Phases: GB_SMOOTHER_LEX runs the
// reference's sequential order as anti-diagonal wavefronts (a line reads
// the new values of the lines before it in the reference's order and the old
// values of those after it, and every such neighbour sits on an earlier or
// a later anti-diagonal), GB_SMOOTHER_ZEBRA the two-colour order with the
// one-sided boundary rows last.
#include "gbcommon.cuh"
#include "gridsync.cuh"
#include "divrn.cuh"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <vector>

#define R3_MAXLEV 8
#define R3_THREADS 256
#define R3_SYNC_STRIDE 32           // unsigneds between the components' barriers

// Work arrays of one level of one component's solve (the w and v solves
// of a step run concurrently, each on its own arrays).
struct R3Work {
    double *v, *f, *res;
    float *v32, *f32, *res32;
};

struct R3Lev {
    int n1, n2, n3, L1, L2;
    double hr, hz, hp, hhr, hhz, hhp;
    double *rvc, *rvv;          // r0 + (i - 1/2) hr and i hr + r0, i = 0..n1+1
    double *fac[4][3];          // [component][direction] factor tables
    int *lines[4][3];           // packed p | q << 16, phase by phase
    int *poff[4][3];            // phase offsets (nphase + 1)
    int nphase[4][3];
    // FP32 inner cycles (GB_PRB_MIXED)
    float *irc, *irv, *iqc, *iqv;   // 1/r and 1/r^2 at cell centres and faces, i = 0..n1+1
    float ihr, ihhr, ihhz, ihhp;
    float *fac32[4][3];         // the factor tables with reciprocal pivots
};

struct R3Dev {
    int nr, nz, np, ni, nj, nk, nlev;
    double dt, r0, rmax, zmax, Ra, Re, Gr, Ptl, dr, dz, dp;
    double nu_num, nu_den;      // -r0 ln(r0/rmax) and zmax 2 pi (host libm)
    double tolcon, sor;
    int nrel, maxsweeps;
    double *fld[GB_R_COUNT];
    R3Lev lev[R3_MAXLEV];
    R3Work work[4][R3_MAXLEV];  // [component 1..3][level]
    unsigned long long *resmax; // two slots per component, bit patterns of non-negative doubles
    int *nanflag;               // two slots per component
    int *abort;                 // nonzero: a solve failed, later kernels return
    int *steps_done;
    double *trans;              // per-k heat flux sums (np + 1)
    double *hist_nu;
    int *hist_sw;
    int *solve_status, *solve_sweeps;   // per component
    GridSync gs[4];             // per component (the w and v solves run concurrently)
    // rot3dmghor.f (GB_R3D_HORIZONTAL): gravity across the axis, both walls'
    // heat flux, the inner wall hot, plain V-cycles
    int horizontal;
    const double *sinth, *costh;        // libm sin, cos of 6.283185307/np k, k = 0..np
    double nu2_num;                     // nz/6 rmax ln(r0/rmax); nu_num is nz/6 r0 ln(r0/rmax) there
    double *trans2;                     // outer-wall per-k sums (np + 1)
    double *hist_nu2;
};

#define FX(a, i, j, k) ((a)[(size_t)(i) + (size_t)ni * ((size_t)(j) + (size_t)nj * (size_t)(k))])

// ---------------------------------------------------------------------------
// Transport (rot3dmg.f:341-873): one thread per point
// ---------------------------------------------------------------------------

__global__ void k_r3d_avort(R3Dev d)
{
    if (*(volatile int *)d.abort) return;
    const int nr = d.nr, nz = d.nz, np = d.np, ni = d.ni, nj = d.nj;
    const long long total = (long long)nr * (nz - 1) * (np + 1);
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int i = 1 + (int)(t % nr);
    const long long rest = t / nr;
    const int j = 1 + (int)(rest % (nz - 1));
    const int k = (int)(rest / (nz - 1));
    const double dr = d.dr, dz = d.dz, dp = d.dp, dt = d.dt, Ptl = d.Ptl;
    const double Ra = d.Ra, Re = d.Re, Gr = d.Gr;
    const double *A = d.fld[GB_R_A], *Ap = d.fld[GB_R_Ap], *B = d.fld[GB_R_B], *C = d.fld[GB_R_C];
    const double *th = d.fld[GB_R_th];
    const double *uel = d.fld[GB_R_uel], *vel = d.fld[GB_R_vel], *wel = d.fld[GB_R_wel];
    double *An = d.fld[GB_R_An];
    const int im = i - 1, jp = j + 1;
    const int km = k == 0 ? np - 1 : k - 1;
    const int ka = k == np ? 1 : k + 1;
    const double r = d.r0 + ((double)i - 0.5) * dr;
    const double u = (FX(uel, i, j, k) + FX(uel, i, jp, k) + FX(uel, i, j, ka) + FX(uel, i, jp, ka) +
                      FX(uel, im, j, k) + FX(uel, im, jp, k) + FX(uel, im, j, ka) + FX(uel, im, jp, ka)) *
                     0.125;
    const double v = (FX(vel, i, jp, k) + FX(vel, i, j, k)) * 0.5;
    const double w = (FX(wel, i, j, ka) + FX(wel, i, j, k)) * 0.5;
    const double tem = (FX(th, i, j, k) + FX(th, i, j, ka) + FX(th, i, jp, k) + FX(th, i, jp, ka)) * 0.25;
    const double BB = (FX(B, i, j, k) + FX(B, im, j, k) + FX(B, i, j, ka) + FX(B, im, j, ka)) * 0.25;
    const double CC = (FX(C, i, j, k) + FX(C, i, jp, k) + FX(C, im, j, k) + FX(C, im, jp, k)) * 0.25;
    double Arra, Ara, Ar, cnr;
    if (i == 1) {
        Arra = (3.2 * FX(A, i - 1, j, k) + 2.0 * FX(A, i + 1, j, k) - 0.2 * FX(A, i + 2, j, k)) / (dr * dr);
        Ara = (-4.0 * FX(A, i - 1, j, k) / 3.0 + FX(A, i + 1, j, k) / 3.0) / dr;
        Ar = (-4.0 * FX(A, i - 1, j, k) / 3.0 + FX(A, i, j, k) + FX(A, i + 1, j, k) / 3.0) / dr;
        cnr = -2.5 / (dr * dr) + 0.5 / dr / r;
    } else if (i == nr) {
        Arra = (3.2 * FX(A, i + 1, j, k) + 2.0 * FX(A, i - 1, j, k) - 0.2 * FX(A, i - 2, j, k)) / (dr * dr);
        Ara = (-FX(A, i - 1, j, k) / 3.0 + 4.0 * FX(A, i + 1, j, k) / 3.0) / dr;
        // the inner-wall formula again (rot3dmg.f:390)
        Ar = (-4.0 * FX(A, i - 1, j, k) / 3.0 + FX(A, i, j, k) + FX(A, i + 1, j, k) / 3.0) / dr;
        cnr = -2.5 / (dr * dr) - 0.5 / dr / r;
    } else {
        Arra = (FX(A, i - 1, j, k) + FX(A, i + 1, j, k)) / (dr * dr);
        Ara = (FX(A, i + 1, j, k) - FX(A, i - 1, j, k)) * 0.5 / dr;
        Ar = Ara;
        cnr = -1.0 / (dr * dr);
        const double Pe = fabs(u * dr / Ptl);
        if (Pe > 2.0) {
            if (u > 0.0) Ar = (FX(A, i, j, k) - FX(A, i - 1, j, k)) / dr;
            else if (u < 0.0) Ar = (FX(A, i + 1, j, k) - FX(A, i, j, k)) / dr;
        }
    }
    const double uelr = ((FX(uel, i, j, k) + FX(uel, i, jp, k) + FX(uel, i, j, ka) + FX(uel, i, jp, ka)) * 0.25 -
                         (FX(uel, im, j, k) + FX(uel, im, jp, k) + FX(uel, im, j, ka) + FX(uel, im, jp, ka)) * 0.25) /
                        dr;
    const double Azza = (FX(A, i, j - 1, k) + FX(A, i, j + 1, k)) / (dz * dz);
    double Az = (FX(A, i, j + 1, k) - FX(A, i, j - 1, k)) * 0.5 / dz;
    {
        const double Pe = fabs(w * dz / Ptl);
        if (Pe > 2.0) {
            if (w > 0.0) Az = (FX(A, i, j, k) - FX(A, i, j - 1, k)) / dz;
            else if (w < 0.0) Az = (FX(A, i, j + 1, k) - FX(A, i, j, k)) / dz;
        }
    }
    const double uelz = ((FX(uel, i, jp, k) + FX(uel, i, jp, ka) + FX(uel, im, jp, k) + FX(uel, im, jp, ka)) * 0.25 -
                         (FX(uel, i, j, k) + FX(uel, i, j, ka) + FX(uel, im, j, k) + FX(uel, im, j, ka)) * 0.25) /
                        dz;
    const double thz = (FX(th, i, jp, k) + FX(th, i, jp, ka) - FX(th, i, j, k) - FX(th, i, j, ka)) * 0.5 / dz;
    const double thh = (FX(th, i, j, ka) + FX(th, i, jp, ka) - FX(th, i, j, k) - FX(th, i, jp, k)) * 0.5 / dp;
    const double Ahha = (FX(A, i, j, ka) + FX(A, i, j, km)) / (dp * dp);
    double Ah = (FX(A, i, j, ka) - FX(A, i, j, km)) * 0.5 / dp;
    {
        const double Pe = fabs(v * dp * r / Ptl);
        if (Pe > 2.0) {
            if (v > 0.0) Ah = (FX(A, i, j, k) - FX(A, i, j, km)) / dp;
            else if (v < 0.0) Ah = (FX(A, i, j, ka) - FX(A, i, j, k)) / dp;
        }
    }
    const double Bh = (FX(B, i, j, ka) + FX(B, im, j, ka) - FX(B, i, j, k) - FX(B, im, j, k)) * 0.5 / dp;
    const double uelh = ((FX(uel, i, j, ka) + FX(uel, i, jp, ka) + FX(uel, im, j, ka) + FX(uel, im, jp, ka)) * 0.25 -
                         (FX(uel, i, j, k) + FX(uel, i, jp, k) + FX(uel, im, j, k) + FX(uel, im, jp, k)) * 0.25) /
                        dp;
    const double cnz = -1.0 / (dz * dz);
    const double cnh = -1.0 / (dp * dp) / (r * r);
    const double RHS1 = Arra + Ara / r + Ahha / (r * r) + Azza - 2.0 * Bh / (r * r) + FX(A, i, j, k) / (Ptl * dt);
    const double ULT = (u * Ar + v * Ah / r + w * Az - uelh * BB / r - uelz * CC) / Ptl;
    const double RHS2 = d.horizontal ? d.sinth[k] * Gr * Ptl * thz   // rot3dmghor.f:479
                                     : -2.0 * Re * uelz + 2.0 * Ra * (tem * uelz + thz * u) / Re / Ptl - Gr * Ptl / r * thh;
    const double cf1 = 1.0 / (Ptl * dt) - uelr / (2.0 * Ptl) + 1.0 / (2.0 * (r * r)) - cnr - cnz - cnh;
    const double cf2 = uelr / (2.0 * Ptl) - 1.0 / (2.0 * (r * r)) + cnr + cnz + cnh;
    FX(An, i, j, k) = (cf2 * FX(Ap, i, j, k) - ULT - RHS2 + RHS1) / cf1;
}

__global__ void k_r3d_bvort(R3Dev d)
{
    if (*(volatile int *)d.abort) return;
    const int nr = d.nr, nz = d.nz, np = d.np, ni = d.ni, nj = d.nj;
    const long long total = (long long)(nr - 1) * (nz - 1) * (np + 1);
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int i = 1 + (int)(t % (nr - 1));
    const long long rest = t / (nr - 1);
    const int j = 1 + (int)(rest % (nz - 1));
    const int k = (int)(rest / (nz - 1));
    const double dr = d.dr, dz = d.dz, dp = d.dp, dt = d.dt, Ptl = d.Ptl;
    const double Ra = d.Ra, Re = d.Re, Gr = d.Gr;
    const double *A = d.fld[GB_R_A], *B = d.fld[GB_R_B], *Bp = d.fld[GB_R_Bp], *C = d.fld[GB_R_C];
    const double *th = d.fld[GB_R_th];
    const double *uel = d.fld[GB_R_uel], *vel = d.fld[GB_R_vel], *wel = d.fld[GB_R_wel];
    double *Bn = d.fld[GB_R_Bn];
    const int ip = i + 1, jp = j + 1;
    const int km = k == 0 ? np - 1 : k - 1;
    const int ka = k == np ? 1 : k + 1;
    const double r = d.r0 + (double)i * dr;
    const double u = (FX(uel, i, j, k) + FX(uel, i, jp, k)) * 0.5;
    const double v = (FX(vel, i, j, km) + FX(vel, i, jp, km) + FX(vel, i, j, k) + FX(vel, i, jp, k) +
                      FX(vel, ip, j, km) + FX(vel, ip, jp, km) + FX(vel, ip, j, k) + FX(vel, ip, jp, k)) *
                     0.125;
    const double w = (FX(wel, i, j, k) + FX(wel, ip, j, k)) * 0.5;
    const double tem = (FX(th, i, jp, k) + FX(th, ip, jp, k) + FX(th, i, j, k) + FX(th, ip, j, k)) * 0.25;
    const double AA = (FX(A, i, j, k) + FX(A, ip, j, k) + FX(A, i, j, km) + FX(A, ip, j, km)) * 0.25;
    const double CC = (FX(C, i, j, k) + FX(C, i, jp, k) + FX(C, i, j, km) + FX(C, i, jp, km)) * 0.25;
    const double Brra = (FX(B, i - 1, j, k) + FX(B, i + 1, j, k)) / (dr * dr);
    const double Bra = (FX(B, i + 1, j, k) - FX(B, i - 1, j, k)) * 0.5 / dr;
    double Br = Bra;
    {
        const double Pe = fabs(u * dr / Ptl);
        if (Pe > 2.0) {
            if (u > 0.0) Br = (FX(B, i, j, k) - FX(B, i - 1, j, k)) / dr;
            else if (u < 0.0) Br = (FX(B, i + 1, j, k) - FX(B, i, j, k)) / dr;
        }
    }
    const double velr = ((FX(vel, ip, j, km) + FX(vel, ip, jp, km) + FX(vel, ip, j, k) + FX(vel, ip, jp, k)) * 0.25 -
                         (FX(vel, i, j, km) + FX(vel, i, jp, km) + FX(vel, i, j, k) + FX(vel, i, jp, k)) * 0.25) /
                        dr;
    const double Bzza = (FX(B, i, j - 1, k) + FX(B, i, j + 1, k)) / (dz * dz);
    double Bz = (FX(B, i, j + 1, k) - FX(B, i, j - 1, k)) * 0.5 / dz;
    {
        const double Pe = fabs(w * dz / Ptl);
        if (Pe > 2.0) {
            if (w > 0.0) Bz = (FX(B, i, j, k) - FX(B, i, j - 1, k)) / dz;
            else if (w < 0.0) Bz = (FX(B, i, j + 1, k) - FX(B, i, j, k)) / dz;
        }
    }
    const double velz = ((FX(vel, i, jp, km) + FX(vel, ip, jp, km) + FX(vel, i, jp, k) + FX(vel, ip, jp, k)) * 0.25 -
                         (FX(vel, i, j, km) + FX(vel, ip, j, km) + FX(vel, i, j, k) + FX(vel, ip, j, k)) * 0.25) /
                        dz;
    const double thz = (FX(th, i, jp, k) + FX(th, ip, jp, k) - FX(th, i, j, k) - FX(th, ip, j, k)) * 0.5 / dz;
    const double thr = (FX(th, ip, jp, k) + FX(th, ip, j, k) - FX(th, i, jp, k) - FX(th, i, j, k)) * 0.5 / dr;
    const double Bhha = (FX(B, i, j, ka) + FX(B, i, j, km)) / (dp * dp);
    double Bh = (FX(B, i, j, ka) - FX(B, i, j, km)) * 0.5 / dp;
    {
        const double Pe = fabs(v * dp * r / Ptl);
        if (Pe > 2.0) {
            if (v > 0.0) Bh = (FX(B, i, j, k) - FX(B, i, j, km)) / dp;
            else if (v < 0.0) Bh = (FX(B, i, j, ka) - FX(B, i, j, k)) / dp;
        }
    }
    const double Ah = (FX(A, i, j, k) + FX(A, ip, j, k) - FX(A, i, j, km) - FX(A, ip, j, km)) * 0.5 / dp;
    const double velh = ((FX(vel, i, j, k) + FX(vel, ip, j, k) + FX(vel, i, jp, k) + FX(vel, ip, jp, k)) * 0.25 -
                         (FX(vel, i, j, km) + FX(vel, ip, j, km) + FX(vel, i, jp, km) + FX(vel, ip, jp, km)) * 0.25) /
                        dp;
    const double cnr = -1.0 / (dr * dr);
    const double cnz = -1.0 / (dz * dz);
    const double cnh = -1.0 / (dp * dp) / (r * r);
    const double RHS1 = Brra + Bra / r + Bhha / (r * r) + Bzza + 2.0 * Ah / (r * r) + FX(B, i, j, k) / (Ptl * dt);
    const double ULT = (u * Br + v * Bh / r + w * Bz - (velr - v / r) * AA - velz * CC) / Ptl;
    const double RHS2 = d.horizontal ? d.costh[k] * Gr * Ptl * thz   // rot3dmghor.f:606
                                     : -2.0 * Re * velz + r * Ra * thz + 2.0 * Ra * (tem * velz + thz * v) / Re / Ptl +
                                           Gr * Ptl * thr;
    const double cf1 = 1.0 / (Ptl * dt) - (u / r + velh / r) / (2.0 * Ptl) + 1.0 / (2.0 * (r * r)) - cnr - cnz - cnh;
    const double cf2 = (u / r + velh / r) / (2.0 * Ptl) - 1.0 / (2.0 * (r * r)) + cnr + cnz + cnh;
    FX(Bn, i, j, k) = (cf2 * FX(Bp, i, j, k) - ULT - RHS2 + RHS1) / cf1;
}

__global__ void k_r3d_cvort(R3Dev d)
{
    if (*(volatile int *)d.abort) return;
    const int nr = d.nr, nz = d.nz, np = d.np, ni = d.ni, nj = d.nj;
    const long long total = (long long)(nr - 1) * nz * (np + 1);
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int i = 1 + (int)(t % (nr - 1));
    const long long rest = t / (nr - 1);
    const int j = 1 + (int)(rest % nz);
    const int k = (int)(rest / nz);
    const double dr = d.dr, dz = d.dz, dp = d.dp, dt = d.dt, Ptl = d.Ptl;
    const double Ra = d.Ra, Re = d.Re;
    const double *A = d.fld[GB_R_A], *B = d.fld[GB_R_B], *C = d.fld[GB_R_C], *Cp = d.fld[GB_R_Cp];
    const double *th = d.fld[GB_R_th];
    const double *uel = d.fld[GB_R_uel], *vel = d.fld[GB_R_vel], *wel = d.fld[GB_R_wel];
    double *Cn = d.fld[GB_R_Cn];
    const int ip = i + 1, jm = j - 1;
    const int km = k == 0 ? np - 1 : k - 1;
    const int ka = k == np ? 1 : k + 1;
    const double r = d.r0 + (double)i * dr;
    const double u = (FX(uel, i, j, ka) + FX(uel, i, j, k)) * 0.5;
    const double v = (FX(vel, i, j, k) + FX(vel, ip, j, k)) * 0.5;
    const double w = (FX(wel, i, j, k) + FX(wel, ip, j, k) + FX(wel, i, j, ka) + FX(wel, ip, j, ka) +
                      FX(wel, i, jm, k) + FX(wel, ip, jm, k) + FX(wel, i, jm, ka) + FX(wel, ip, jm, ka)) *
                     0.125;
    const double AA = (FX(A, i, j, k) + FX(A, i, jm, k) + FX(A, ip, j, k) + FX(A, ip, jm, k)) * 0.25;
    const double BB = (FX(B, i, j, k) + FX(B, i, jm, k) + FX(B, i, j, ka) + FX(B, i, jm, ka)) * 0.25;
    const double tem = (FX(th, i, j, k) + FX(th, ip, j, k) + FX(th, ip, j, ka) + FX(th, i, j, ka)) * 0.25;
    const double Crra = (FX(C, i - 1, j, k) + FX(C, i + 1, j, k)) / (dr * dr);
    const double Cra = (FX(C, i + 1, j, k) - FX(C, i - 1, j, k)) * 0.5 / dr;
    double Cr = Cra;
    {
        const double Pe = fabs(u * dr / Ptl);
        if (Pe > 2.0) {
            if (u > 0.0) Cr = (FX(C, i, j, k) - FX(C, i - 1, j, k)) / dr;
            else if (u < 0.0) Cr = (FX(C, i + 1, j, k) - FX(C, i, j, k)) / dr;
        }
    }
    const double welr = ((FX(wel, ip, j, k) + FX(wel, ip, j, ka) + FX(wel, ip, jm, k) + FX(wel, ip, jm, ka)) * 0.25 -
                         (FX(wel, i, j, k) + FX(wel, i, j, ka) + FX(wel, i, jm, k) + FX(wel, i, jm, ka)) * 0.25) /
                        dr;
    const double thr = (FX(th, ip, j, k) + FX(th, ip, j, ka) - FX(th, i, j, k) - FX(th, i, j, ka)) * 0.5 / dr;
    double Czza, Cz, cnz;
    if (j == 1) {
        Czza = (3.2 * FX(C, i, j - 1, k) + 2.0 * FX(C, i, j + 1, k) - 0.2 * FX(C, i, j + 2, k)) / (dz * dz);
        Cz = (-4.0 * FX(C, i, j - 1, k) / 3.0 + FX(C, i, j, k) + FX(C, i, j + 1, k) / 3.0) / dz;
        cnz = -2.5 / (dz * dz);
    } else if (j == nz) {
        Czza = (3.2 * FX(C, i, j + 1, k) + 2.0 * FX(C, i, j - 1, k) - 0.2 * FX(C, i, j - 2, k)) / (dz * dz);
        Cz = (-FX(C, i, j - 1, k) / 3.0 - FX(C, i, j, k) + 4.0 * FX(C, i, j + 1, k) / 3.0) / dz;
        cnz = -2.5 / (dz * dz);
    } else {
        Czza = (FX(C, i, j - 1, k) + FX(C, i, j + 1, k)) / (dz * dz);
        Cz = (FX(C, i, j + 1, k) - FX(C, i, j - 1, k)) * 0.5 / dz;
        const double Pe = fabs(w * dz / Ptl);
        if (Pe > 2.0) {
            if (w > 0.0) Cz = (FX(C, i, j, k) - FX(C, i, j - 1, k)) / dz;
            else if (w < 0.0) Cz = (FX(C, i, j + 1, k) - FX(C, i, j, k)) / dz;
        }
        cnz = -1.0 / (dz * dz);
    }
    const double welz = ((FX(wel, i, j, k) + FX(wel, ip, j, k) + FX(wel, i, j, ka) + FX(wel, ip, j, ka)) * 0.25 -
                         (FX(wel, i, jm, k) + FX(wel, ip, jm, k) + FX(wel, i, jm, ka) + FX(wel, ip, jm, ka)) * 0.25) /
                        dz;
    const double Chha = (FX(C, i, j, ka) + FX(C, i, j, km)) / (dp * dp);
    double Ch = (FX(C, i, j, ka) - FX(C, i, j, km)) * 0.5 / dp;
    {
        const double Pe = fabs(v * dp * r / Ptl);
        if (Pe > 2.0) {
            if (v > 0.0) Ch = (FX(C, i, j, k) - FX(C, i, j, km)) / dp;
            else if (v < 0.0) Ch = (FX(C, i, j, ka) - FX(C, i, j, k)) / dp;
        }
    }
    const double welh = ((FX(wel, i, j, ka) + FX(wel, ip, j, ka) + FX(wel, i, jm, ka) + FX(wel, ip, jm, ka)) * 0.25 -
                         (FX(wel, i, j, k) + FX(wel, ip, j, k) + FX(wel, i, jm, k) + FX(wel, ip, jm, k)) * 0.25) /
                        dp;
    const double thh = (FX(th, i, j, ka) + FX(th, ip, j, ka) - FX(th, i, j, k) - FX(th, ip, j, k)) * 0.5 / dp;
    const double cnr = -1.0 / (dr * dr);
    const double cnh = -1.0 / (dp * dp) / (r * r);
    const double RHS1 = Crra + Cra / r + Chha / (r * r) + Czza + FX(C, i, j, k) / (Ptl * dt);
    const double ULT = (u * Cr + v * Ch / r + w * Cz - welr * AA - welh * BB / r) / Ptl;
    const double RHS2 =
        d.horizontal ? -(1.0 / r * d.Gr * Ptl * d.costh[k] * thh) - d.Gr * Ptl * d.sinth[k] * thr   // rot3dmghor.f:749
                     : -2.0 * Re * welz - Ra * thh + 2.0 * Ra * (tem * welz - thr * u - thh * v / r) / Re / Ptl;
    const double cf1 = 1.0 / (Ptl * dt) - welz / (2.0 * Ptl) - cnr - cnz - cnh;
    const double cf2 = welz / (2.0 * Ptl) + cnr + cnz + cnh;
    FX(Cn, i, j, k) = (cf2 * FX(Cp, i, j, k) - ULT - RHS2 + RHS1) / cf1;
}

__global__ void k_r3d_temp(R3Dev d)
{
    if (*(volatile int *)d.abort) return;
    const int nr = d.nr, nz = d.nz, np = d.np, ni = d.ni, nj = d.nj;
    const long long total = (long long)nr * (nz + 2) * (np + 1);
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int i = 1 + (int)(t % nr);
    const long long rest = t / nr;
    const int j = (int)(rest % (nz + 2));
    const int k = (int)(rest / (nz + 2));
    const double dr = d.dr, dz = d.dz, dp = d.dp, dt = d.dt, Ptl = d.Ptl;
    const double *th = d.fld[GB_R_th], *thp = d.fld[GB_R_thp];
    const double *uel = d.fld[GB_R_uel], *vel = d.fld[GB_R_vel], *wel = d.fld[GB_R_wel];
    double *thn = d.fld[GB_R_thn];
    const int im = i - 1, jm = j - 1;
    const int km = k == 0 ? np - 1 : k - 1;
    const int ka = k == np ? 1 : k + 1;
    const double r = d.r0 + ((double)i - 0.5) * dr;
    double u, v, w;
    if (j == 0 || j == nz + 1) {
        u = 0.0;
        v = 0.0;
        w = 0.0;
    } else {
        u = (FX(uel, i, j, k) + FX(uel, im, j, k)) * 0.5;
        v = (FX(vel, i, j, k) + FX(vel, i, j, km)) * 0.5;
        w = (FX(wel, i, j, k) + FX(wel, i, jm, k)) * 0.5;
    }
    double thrra, thra, thr, cnr;
    if (i == 1) {
        thrra = (3.2 * FX(th, i - 1, j, k) + 2.0 * FX(th, i + 1, j, k) - 0.2 * FX(th, i + 2, j, k)) / (dr * dr);
        thra = (-4.0 * FX(th, i - 1, j, k) / 3.0 + FX(th, i + 1, j, k) / 3.0) / dr;
        thr = (-4.0 * FX(th, i - 1, j, k) / 3.0 + FX(th, i, j, k) + FX(th, i + 1, j, k) / 3.0) / dr;
        cnr = -2.5 / (dr * dr) + 0.5 / dr / r;
    } else if (i == nr) {
        thrra = (3.2 * FX(th, i + 1, j, k) + 2.0 * FX(th, i - 1, j, k) - 0.2 * FX(th, i - 2, j, k)) / (dr * dr);
        thra = (-FX(th, i - 1, j, k) / 3.0 + 4.0 * FX(th, i + 1, j, k) / 3.0) / dr;
        thr = (-FX(th, i - 1, j, k) / 3.0 - FX(th, i, j, k) + 4.0 * FX(th, i + 1, j, k) / 3.0) / dr;
        cnr = -2.5 / (dr * dr) - 0.5 / dr / r;
    } else {
        thrra = (FX(th, i - 1, j, k) + FX(th, i + 1, j, k)) / (dr * dr);
        thra = (FX(th, i + 1, j, k) - FX(th, i - 1, j, k)) * 0.5 / dr;
        thr = thra;
        const double Pe = fabs(u * dr / Ptl);
        if (Pe > 2.0) {
            if (u > 0.0) thr = (FX(th, i, j, k) - FX(th, i - 1, j, k)) / dr;
            else if (u < 0.0) thr = (FX(th, i + 1, j, k) - FX(th, i, j, k)) / dr;
        }
        cnr = -1.0 / (dr * dr);
    }
    double thzza, thz, cnz;
    if (j == 1) {
        thzza = (3.2 * FX(th, i, j - 1, k) + 2.0 * FX(th, i, j + 1, k) - 0.2 * FX(th, i, j + 2, k)) / (dz * dz);
        thz = (-4.0 * FX(th, i, j - 1, k) / 3.0 + FX(th, i, j, k) + FX(th, i, j + 1, k) / 3.0) / dz;
        cnz = -2.5 / (dz * dz);
    } else if (j == nz) {
        thzza = (3.2 * FX(th, i, j + 1, k) + 2.0 * FX(th, i, j - 1, k) - 0.2 * FX(th, i, j - 2, k)) / (dz * dz);
        thz = (-FX(th, i, j - 1, k) / 3.0 - FX(th, i, j, k) + 4.0 * FX(th, i, j + 1, k) / 3.0) / dz;
        cnz = -2.5 / (dz * dz);
    } else if (j == 0) {
        thzza = 8.0 * FX(th, i, j + 1, k) / (dz * dz);
        thz = 0.0;
        cnz = -4.0 / (dz * dz);
    } else if (j == nz + 1) {
        thzza = 8.0 * FX(th, i, j - 1, k) / (dz * dz);
        thz = 0.0;
        cnz = -4.0 / (dz * dz);
    } else {
        thzza = (FX(th, i, j - 1, k) + FX(th, i, j + 1, k)) / (dz * dz);
        thz = (FX(th, i, j + 1, k) - FX(th, i, j - 1, k)) * 0.5 / dz;
        const double Pe = fabs(w * dz / Ptl);
        if (Pe > 2.0) {
            if (w > 0.0) thz = (FX(th, i, j, k) - FX(th, i, j - 1, k)) / dz;
            else if (w < 0.0) thz = (FX(th, i, j + 1, k) - FX(th, i, j, k)) / dz;
        }
        cnz = -1.0 / (dz * dz);
    }
    const double thhha = (FX(th, i, j, ka) + FX(th, i, j, km)) / (dp * dp);
    double thh = (FX(th, i, j, ka) - FX(th, i, j, km)) * 0.5 / dp;
    {
        const double Pe = fabs(v * dp * r / Ptl);
        if (Pe > 2.0) {
            if (v > 0.0) thh = (FX(th, i, j, k) - FX(th, i, j, km)) / dp;
            else if (v < 0.0) thh = (FX(th, i, j, ka) - FX(th, i, j, k)) / dp;
        }
    }
    const double cnp = -1.0 / (dp * dp) / (r * r);
    const double RHS1 = thrra + thra / r + thhha / (r * r) + thzza + FX(th, i, j, k) / dt;
    const double ULT = u * thr + v * thh / r + w * thz;
    const double cf1 = 1.0 / dt - cnr - cnz - cnp;
    const double cf2 = cnr + cnz + cnp;
    FX(thn, i, j, k) = (cf2 * FX(thp, i, j, k) - ULT + RHS1) / cf1;
}

// heat (rot3dmg.f:882-909): one thread per k sums its z column in the
// reference's order; k_r3d_heat_sum adds the columns k = 1..np in order.
__global__ void k_r3d_heat_k(R3Dev d)
{
    if (*(volatile int *)d.abort) return;
    const int k = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (k > d.np) return;
    const int ni = d.ni, nj = d.nj, nz = d.nz;
    const double dr = d.dr, dz = d.dz;
    const double *th = d.fld[GB_R_th];
#define HT(j, k) ((-184.0 * FX(th, 0, j, k) + 225.0 * FX(th, 1, j, k) - 50.0 * FX(th, 2, j, k) + 9.0 * FX(th, 3, j, k)))
    if (d.horizontal) {
        // rot3dmghor.f:913-945: both cylinders over j = nz/2-3 .. nz/2+3
        const int nr = d.nr, nza = nz / 2 - 3, nzb = nz / 2 + 3;
#define HB(j, k) ((184.0 * FX(th, nr + 1, j, k) - 225.0 * FX(th, nr, j, k) + 50.0 * FX(th, nr - 1, j, k) - \
                   9.0 * FX(th, nr - 2, j, k)))
        double ta = dz * HT(nza, k) / (120.0 * dr);
        double tb = dz * HB(nza, k) / (120.0 * dr);
        ta = ta + dz * HT(nzb, k) / (120.0 * dr);
        tb = tb + dz * HB(nzb, k) / (120.0 * dr);
        for (int j = nza + 1; j <= nzb - 1; ++j) {
            ta = ta + dz * HT(j, k) / (60.0 * dr);
            tb = tb + dz * HB(j, k) / (60.0 * dr);
        }
#undef HB
        d.trans[k] = ta;
        d.trans2[k] = tb;
        return;
    }
    double trans = dz * HT(0, k) / (240.0 * dr);
    trans = trans + dz * HT(1, k) / (80.0 * dr);
    trans = trans + dz * HT(nz, k) / (80.0 * dr);
    trans = trans + dz * HT(nz + 1, k) / (240.0 * dr);
    for (int j = 2; j <= nz - 1; ++j) trans = trans + dz * HT(j, k) / (60.0 * dr);
#undef HT
    d.trans[k] = trans;
}

__global__ void k_r3d_heat_sum(R3Dev d, int step)
{
    if (*(volatile int *)d.abort) return;
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double trans1 = 0.0, trans2 = 0.0;
    for (int k = 1; k <= d.np; ++k) trans1 = trans1 + d.trans[k] * d.dp;
    if (d.horizontal)
        for (int k = 1; k <= d.np; ++k) trans2 = trans2 + d.trans2[k] * d.dp;
    d.trans[0] = trans1;
    d.trans2[0] = trans2;
    if (step >= 0) {
        d.hist_nu[step] = d.nu_num * trans1 / d.nu_den;
        d.hist_nu2[step] = d.horizontal ? d.nu2_num * trans2 / d.nu_den : 0.0;
    }
}

// rhsw / rhsv / rhsu (rot3dmg.f:1026-1150)
template <int COMP>
__global__ void k_r3d_rhs(R3Dev d)
{
    if (*(volatile int *)d.abort) return;
    const int nr = d.nr, nz = d.nz, np = d.np, ni = d.ni, nj = d.nj;
    const int I = COMP == 3 ? nr - 1 : nr, J = COMP == 1 ? nz - 1 : nz;
    const long long total = (long long)I * J * (np + 1);
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int i = 1 + (int)(t % I);
    const long long rest = t / I;
    const int j = 1 + (int)(rest % J);
    const int k = (int)(rest / J);
    const double dr = d.dr, dz = d.dz, dp = d.dp;
    const double *An = d.fld[GB_R_An], *Bn = d.fld[GB_R_Bn], *Cn = d.fld[GB_R_Cn], *wel = d.fld[GB_R_wel];
    const int km = k == 0 ? np - 1 : k - 1;
    if (COMP == 1) {
        const double r = d.r0 + ((double)i - 0.5) * dr;
        const double Ah = (FX(An, i, j, k) - FX(An, i, j, km)) / dp;
        double w;
        if (i == 1) w = Ah / r - FX(Bn, 1, j, k) / dr - 0.5 * FX(Bn, 1, j, k) / r;
        else if (i == nr) w = Ah / r + FX(Bn, nr - 1, j, k) / dr - 0.5 * FX(Bn, nr - 1, j, k) / r;
        else {
            const double Br = (FX(Bn, i, j, k) - FX(Bn, i - 1, j, k)) / dr;
            w = Ah / r - Br - 0.5 * (FX(Bn, i, j, k) + FX(Bn, i - 1, j, k)) / r;
        }
        FX(d.fld[GB_R_wrh], i, j, k) = w;
    } else if (COMP == 2) {
        const double r = d.r0 + ((double)i - 0.5) * dr;
        double v;
        if (i == 1) v = FX(Cn, 1, j, k) / dr + FX(Cn, 1, j, k) / r;
        else if (i == nr) v = -FX(Cn, nr - 1, j, k) / dr + FX(Cn, nr - 1, j, k) / r;
        else {
            const double Cr = (FX(Cn, i, j, k) - FX(Cn, i - 1, j, k)) / dr;
            v = Cr + (FX(Cn, i, j, k) + FX(Cn, i - 1, j, k)) / r;
        }
        if (j == 1) v = v - FX(An, i, 1, k) / dz;
        else if (j == nz) v = v + FX(An, i, nz - 1, k) / dz;
        else {
            const double Az = (FX(An, i, j, k) - FX(An, i, j - 1, k)) / dz;
            v = v - Az;
        }
        FX(d.fld[GB_R_vrh], i, j, k) = v;
    } else {
        const double r = d.r0 + (double)i * dr;
        const double welz =
            0.5 * (FX(wel, i, j, k) + FX(wel, i + 1, j, k) - FX(wel, i, j - 1, k) - FX(wel, i + 1, j - 1, k)) / dz;
        const double Ch = (FX(Cn, i, j, k) - FX(Cn, i, j, km)) / dp;
        double u;
        if (j == 1) u = FX(Bn, i, 1, k) / dz - Ch / r - 2.0 * welz / r;
        else if (j == nz) u = -FX(Bn, i, nz - 1, k) / dz - Ch / r - 2.0 * welz / r;
        else {
            const double Bz = (FX(Bn, i, j, k) - FX(Bn, i, j - 1, k)) / dz;
            u = Bz - Ch / r - 2.0 * welz / r;
        }
        FX(d.fld[GB_R_urh], i, j, k) = u;
    }
}

// update (rot3dmg.f:964-1023): each thread sets the wall values of its own
// point (they depend on the velocities only) and moves its time levels.
__global__ void k_r3d_update(R3Dev d, int step)
{
    if (*(volatile int *)d.abort) return;
    const int nr = d.nr, nz = d.nz, ni = d.ni, nj = d.nj;
    const long long total = (long long)ni * nj * d.nk;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0 && step >= 0) atomicAdd(d.steps_done, 1);
    if (t >= total) return;
    const int i = (int)(t % ni);
    const long long rest = t / ni;
    const int j = (int)(rest % nj);
    const int k = (int)(rest / nj);
    const double dr = d.dr, dz = d.dz;
    const double *uel = d.fld[GB_R_uel], *vel = d.fld[GB_R_vel], *wel = d.fld[GB_R_wel];
    double *An = d.fld[GB_R_An], *Bn = d.fld[GB_R_Bn], *Cn = d.fld[GB_R_Cn], *thn = d.fld[GB_R_thn];
    if (i >= 1 && i <= nr) {
        if (j == 0) FX(An, i, 0, k) = -(3.0 * FX(vel, i, 1, k) - FX(vel, i, 2, k) / 3.0) / dz;
        else if (j == nz) FX(An, i, nz, k) = -(FX(vel, i, nz - 1, k) / 3.0 - 3.0 * FX(vel, i, nz, k)) / dz;
    }
    if (i >= 1 && i <= nr - 1) {
        if (j == 0) FX(Bn, i, 0, k) = (3.0 * FX(uel, i, 1, k) - FX(uel, i, 2, k) / 3.0) / dz;
        else if (j == nz) FX(Bn, i, nz, k) = (-3.0 * FX(uel, i, nz, k) + FX(uel, i, nz - 1, k) / 3.0) / dz;
    }
    if (j >= 1 && j <= nz - 1) {
        if (i == 0) FX(Bn, 0, j, k) = -(3.0 * FX(wel, 1, j, k) - FX(wel, 2, j, k) / 3.0) / dr;
        else if (i == nr) FX(Bn, nr, j, k) = -(FX(wel, nr - 1, j, k) / 3.0 - 3.0 * FX(wel, nr, j, k)) / dr;
    }
    if (j >= 1 && j <= nz) {
        if (i == 0) FX(Cn, 0, j, k) = (3.0 * FX(vel, 1, j, k) - FX(vel, 2, j, k) / 3.0) / dr;
        else if (i == nr) FX(Cn, nr, j, k) = (FX(vel, nr - 1, j, k) / 3.0 - 3.0 * FX(vel, nr, j, k)) / dr;
    }
    // wall temperatures: inner 0, outer 1 (the horizontal annulus: inner 1, outer 0)
    if (i == 0) FX(thn, 0, j, k) = d.horizontal ? 1.0 : 0.0;
    else if (i == nr + 1) FX(thn, nr + 1, j, k) = d.horizontal ? 0.0 : 1.0;
    const size_t p = (size_t)t;
    d.fld[GB_R_Ap][p] = d.fld[GB_R_A][p];
    d.fld[GB_R_A][p] = An[p];
    d.fld[GB_R_Bp][p] = d.fld[GB_R_B][p];
    d.fld[GB_R_B][p] = Bn[p];
    d.fld[GB_R_Cp][p] = d.fld[GB_R_C][p];
    d.fld[GB_R_C][p] = Cn[p];
    d.fld[GB_R_thp][p] = d.fld[GB_R_th][p];
    d.fld[GB_R_th][p] = thn[p];
}

// ---------------------------------------------------------------------------
// Multigrid line relaxation (rot3dmg.f:1543-2173)
// ---------------------------------------------------------------------------

// Solver of each (component, direction): 0 pdma, 1 tdma, 2 ptdma.
__host__ __device__ __forceinline__ int r3_kind(int comp, int dir)
{
    if (dir == 2) return 2;
    if (dir == 0) return comp == 3 ? 1 : 0;
    return comp == 1 ? 1 : 0;
}
__host__ __device__ __forceinline__ int r3_len(int comp, int dir, int n1, int n2, int n3)
{
    if (dir == 0) return comp == 3 ? n1 - 1 : n1;
    if (dir == 1) return comp == 1 ? n2 - 1 : n2;
    return n3;
}
__host__ __device__ __forceinline__ int r3_tabsize(int kind, int n)
{
    return kind == 0 ? 6 * n : kind == 1 ? 4 * n : 7 * n;   // the last n: reciprocals of the pivots
}
__host__ __device__ __forceinline__ int r3_imax(int comp, int n1) { return comp == 3 ? n1 - 1 : n1; }
__host__ __device__ __forceinline__ int r3_jmax(int comp, int n2) { return comp == 1 ? n2 - 1 : n2; }

// Matrix row e (0-based) of a line of component comp in direction dir on
// level L (ti: the line's i for z- and phi-lines), as the reference builds
// it: relax1 :1576-1598, :1614-1643, :1652-1683; relax2 :1776-1799,
// :1830-1878, :1890-1926; relax3 :2022-2026, :2060-2081, :2094-2120.
__device__ void r3_coef(const R3Lev &L, int comp, int dir, int ti, int e, double &a, double &b, double &c, double &dd,
                        double &ee)
{
    const int n1 = L.n1, n2 = L.n2;
    const double hr = L.hr, hhr = L.hhr, hhz = L.hhz, hhp = L.hhp;
    dd = 0.0;
    ee = 0.0;
    if (dir == 0) {
        const int i = e + 1;
        if (comp == 1) {
            const double rval = L.rvc[i];
            if (i == 1) {
                a = 0.0;
                b = 0.0;
                c = -2.0 / hhr - 1.0 / hr / rval * 0.5 - 2.0 / hhz - 2.0 / hhp / (rval * rval);
                dd = 5.0 / hhr / 3.0 + 1.0 / hr / rval * 0.5;
                ee = -0.2 / hhr;
            } else if (i == n1) {
                a = -0.2 / hhr;
                b = 5.0 / hhr / 3.0 - 1.0 / hr / rval * 0.5;
                c = -2.0 / hhr + 1.0 / hr / rval * 0.5 - 2.0 / hhz - 2.0 / hhp / (rval * rval);
            } else {
                a = 0.0;
                b = 1.0 / hhr - 0.5 / hr / rval;
                c = -(2.0 / hhr + 2.0 / hhz + 2.0 / hhp / (rval * rval));
                dd = 1.0 / hhr + 0.5 / hr / rval;
            }
        } else if (comp == 2) {
            const double rval = L.rvc[i];
            const double rq = rval * rval;
            if (i == 1) {
                a = 0.0;
                b = 0.0;
                c = -2.0 / hhr - 2.0 / hhp / rq + 1.0 / rq;
                dd = 5.0 / 3.0 / hhr + 4.0 / 3.0 / hr / rval;
                ee = -0.2 / hhr;
            } else if (i == n1) {
                a = -0.2 / hhr;
                b = 5.0 / 3.0 / hhr - 4.0 / 3.0 / hr / rval;
                c = -2.0 / hhr - 2.0 / hhp / rq + 1.0 / rq;
            } else {
                a = 0.0;
                b = 1.0 / hhr - 1.5 / hr / rval;
                c = -(2.0 / hhr + 2.0 / hhp / rq) + 1.0 / rq;
                dd = 1.0 / hhr + 1.5 / hr / rval;
            }
            c = c - 2.0 / hhz;
        } else {
            const double rval = L.rvv[i];
            const double rq = rval * rval;
            a = 1.0 / hhr - 1.5 / hr / rval;
            b = -(2.0 / hhr - 1.0 / rq + 2.0 / hhp / rq);
            c = 1.0 / hhr + 1.5 / hr / rval;
            b = b - 2.0 / hhz;
        }
    } else if (dir == 1) {
        const int i = ti, j = e + 1;
        if (comp == 1) {
            const double rval = L.rvc[i];
            a = 1.0 / hhz;
            b = -(2.0 / hhz + 2.0 / hhp / (rval * rval));
            c = 1.0 / hhz;
            if (i == 1) b = b - 2.0 / hhr - 1.0 / hr / rval * 0.5;
            else if (i == n1) b = b - 2.0 / hhr + 1.0 / hr / rval * 0.5;
            else b = b - 2.0 / hhr;
        } else if (comp == 2) {
            const double rval = L.rvc[i];
            const double rq = rval * rval;
            if (j == 1) {
                a = 0.0;
                b = 0.0;
                c = -2.0 / hhz - 2.0 / hhp / rq + 1.0 / rq;
                dd = 5.0 / 3.0 / hhz;
                ee = -0.2 / hhz;
            } else if (j == n2) {
                a = -0.2 / hhz;
                b = 5.0 / 3.0 / hhz;
                c = -2.0 / hhz - 2.0 / hhp / rq + 1.0 / rq;
            } else {
                a = 0.0;
                b = 1.0 / hhz;
                c = -(2.0 / hhz + 2.0 / hhp / rq) + 1.0 / rq;
                dd = 1.0 / hhz;
            }
            c = c - 2.0 / hhr;
        } else {
            const double rval = L.rvv[i];
            const double rq = rval * rval;
            if (j == 1) {
                a = 0.0;
                b = 0.0;
                c = -2.0 / hhz - 2.0 / hhr + 1.0 / rq - 2.0 / hhp / rq;
                dd = 5.0 / hhz / 3.0;
                ee = -0.2 / hhz;
            } else if (j == n2) {
                a = -0.2 / hhz;
                b = 5.0 / hhz / 3.0;
                c = -2.0 / hhz - 2.0 / hhr + 1.0 / rq - 2.0 / hhp / rq;
            } else {
                a = 0.0;
                b = 1.0 / hhz;
                c = -(2.0 / hhz + 2.0 / hhr + 2.0 / hhp / rq) + 1.0 / rq;
                dd = 1.0 / hhz;
            }
        }
    } else {
        const int i = ti;
        if (comp == 1) {
            const double rval = L.rvc[i];
            a = 1.0 / hhp / (rval * rval);
            b = -(2.0 / hhz + 2.0 / hhp / (rval * rval));
            c = 1.0 / hhp / (rval * rval);
            if (i == 1) b = b - 2.0 / hhr - 1.0 / hr / rval * 0.5;
            else if (i == n1) b = b - 2.0 / hhr + 1.0 / hr / rval * 0.5;
            else b = b - 2.0 / hhr;
        } else if (comp == 2) {
            const double rval = L.rvc[i];
            const double rq = rval * rval;
            a = 1.0 / hhp / rq;
            c = 1.0 / hhp / rq;
            b = -(2.0 / hhp / rq) + 1.0 / rq;
            b = b - 2.0 / hhr;
            b = b - 2.0 / hhz;
        } else {
            const double rval = L.rvv[i];
            const double rq = rval * rval;
            a = 1.0 / hhp / rq;
            b = -(2.0 / hhr - 1.0 / rq + 2.0 / hhp / rq);
            c = 1.0 / hhp / rq;
            b = b - 2.0 / hhz;
        }
    }
}

struct FacJob {
    int lev, comp, dir, ti;
    double *tab;
};

// Runs the matrix half of the reference's eliminations once per line class
// and records what the right-hand-side half needs (one thread per class).
//   pdma  [C | B | A | D | E]: divisor c(k) at step k, b(k) as used at step
//         k-1, a(k), the normalised d(k), e(k); C(n) is the last divisor.
//   tdma  [F | B | C]: multipliers a(j)/b(j-1), eliminated diagonal, c.
//   ptdma [A | B | C | F1 | F2 | F3]: eliminated a (fill-in column), b, c;
//         multipliers of row j and of row n at step j; the last multiplier.
__global__ void k_r3d_factors(const __grid_constant__ R3Dev d, const FacJob *jobs, int njobs)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= njobs) return;
    const FacJob J = jobs[q];
    const R3Lev &L = d.lev[J.lev];
    const int kind = r3_kind(J.comp, J.dir);
    const int n = r3_len(J.comp, J.dir, L.n1, L.n2, L.n3);
    double *T = J.tab;
    if (kind == 0) {
        double *Cc = T, *Bb = T + n, *Aa = T + 2 * n, *Dd = T + 3 * n, *Ee = T + 4 * n;
        for (int e = 0; e < n; ++e) r3_coef(L, J.comp, J.dir, J.ti, e, Aa[e], Bb[e], Cc[e], Dd[e], Ee[e]);
        for (int k = 0; k <= n - 2; ++k) {
            const double ck = Cc[k];
            Dd[k] = Dd[k] / ck;
            Ee[k] = Ee[k] / ck;
            Cc[k + 1] = Cc[k + 1] - Bb[k + 1] * Dd[k];
            if (k != n - 2) Dd[k + 1] = Dd[k + 1] - Bb[k + 1] * Ee[k];
            if (k != n - 2) {
                Bb[k + 2] = Bb[k + 2] - Aa[k + 2] * Dd[k];
                Cc[k + 2] = Cc[k + 2] - Aa[k + 2] * Ee[k];
            }
        }
        for (int k = 0; k < n; ++k) T[5 * n + k] = 1.0 / Cc[k];
    } else if (kind == 1) {
        double *F = T, *Bb = T + n, *Cc = T + 2 * n;
        double dummy_d, dummy_e;
        for (int e = 0; e < n; ++e) r3_coef(L, J.comp, J.dir, J.ti, e, F[e], Bb[e], Cc[e], dummy_d, dummy_e);
        F[0] = 0.0;
        for (int j = 1; j < n; ++j) {
            const double fact = F[j] / Bb[j - 1];
            Bb[j] = Bb[j] - fact * Cc[j - 1];
            F[j] = fact;
        }
        for (int j = 0; j < n; ++j) T[3 * n + j] = 1.0 / Bb[j];
    } else {
        double *a = T, *b = T + n, *c = T + 2 * n, *F1 = T + 3 * n, *F2 = T + 4 * n, *F3 = T + 5 * n;
        double dummy_d, dummy_e;
        for (int e = 0; e < n; ++e) {
            r3_coef(L, J.comp, J.dir, J.ti, e, a[e], b[e], c[e], dummy_d, dummy_e);
            F1[e] = 0.0;
            F2[e] = 0.0;
        }
        const int N = n - 1;
        double fact;
        for (int j = 1; j <= n - 3; ++j) {
            fact = a[j] / b[j - 1];
            b[j] = b[j] - fact * c[j - 1];
            a[j] = -fact * a[j - 1];
            F1[j] = fact;
            fact = c[N] / b[j - 1];
            c[N] = -fact * c[j - 1];
            b[N] = b[N] - fact * a[j - 1];
            F2[j] = fact;
        }
        fact = a[n - 2] / b[n - 3];
        b[n - 2] = b[n - 2] - fact * c[n - 3];
        c[n - 2] = c[n - 2] - fact * a[n - 3];
        F1[n - 2] = fact;
        fact = c[N] / b[n - 3];
        a[N] = a[N] - fact * c[n - 3];
        b[N] = b[N] - fact * a[n - 3];
        F2[n - 2] = fact;
        fact = a[N] / b[n - 2];
        b[N] = b[N] - fact * c[n - 2];
        F3[0] = fact;
        for (int j = 0; j < n; ++j) T[6 * n + j] = 1.0 / b[j];
    }
}

static const double F02 = (double)0.2f;   // REAL*4 literal 0.2 (rot3dmg.f:1626, 1800, 2029, 2106 ...)

#define PV(i, j, k) v[(size_t)(i) + (size_t)L1 * ((size_t)(j) + (size_t)L2 * (size_t)(k))]
#define RF(i, j, k) f[(size_t)(i) + (size_t)L1 * ((size_t)(j) + (size_t)L2 * (size_t)(k))]

// Right-hand side of row e of line (p, q): relax1 :1599-1601, :1616-1640,
// :1655-1681; relax2 :1798-1816, :1858-1876, :1891-1922; relax3 :2027-2041,
// :2082-2085, :2096-2118.
template <int COMP>
__device__ __forceinline__ double r3_rhs(const R3Lev &L, const R3Work &W, int dir, int p, int q, int e)
{
    const int n1 = L.n1, n2 = L.n2, n3 = L.n3, L1 = L.L1, L2 = L.L2;
    const double hr = L.hr, hhr = L.hhr, hhz = L.hhz, hhp = L.hhp;
    const double *v = W.v, *f = W.f;
    if (dir == 0) {
        const int i = e + 1, j = p, k = q;
        const int ka = k == n3 ? 1 : k + 1, km = k - 1;
        if (COMP == 1) {
            const double rval = L.rvc[i];
            return -(PV(i, j + 1, k) + PV(i, j - 1, k)) / hhz - (PV(i, j, ka) + PV(i, j, km)) / hhp / (rval * rval) +
                   RF(i, j, k);
        } else if (COMP == 2) {
            const double rval = L.rvc[i];
            const double rq = rval * rval;
            if (j == 1)
                return -(5.0 / 3.0 * PV(i, j + 1, k) - F02 * PV(i, j + 2, k)) / hhz -
                       (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
            if (j == n2)
                return -(5.0 / 3.0 * PV(i, j - 1, k) - F02 * PV(i, j - 2, k)) / hhz -
                       (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
            return -(PV(i, j - 1, k) + PV(i, j + 1, k)) / hhz - (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
        } else {
            const double rval = L.rvv[i];
            const double rq = rval * rval;
            if (j == 1)
                return -(5.0 * PV(i, j + 1, k) / 3.0 - F02 * PV(i, j + 2, k)) / hhz -
                       (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
            if (j == n2)
                return -(5.0 * PV(i, j - 1, k) / 3.0 - F02 * PV(i, j - 2, k)) / hhz -
                       (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
            return -(PV(i, j - 1, k) + PV(i, j + 1, k)) / hhz - (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
        }
    } else if (dir == 1) {
        const int i = p, j = e + 1, k = q;
        const int ka = k == n3 ? 1 : k + 1, km = k - 1;
        if (COMP == 1) {
            const double rval = L.rvc[i];
            if (i == 1)
                return -(5.0 * PV(i + 1, j, k) / 3.0 - F02 * PV(i + 2, j, k)) / hhr - 1.0 * PV(i + 1, j, k) / hr / rval * 0.5 -
                       (PV(i, j, ka) + PV(i, j, km)) / hhp / (rval * rval) + RF(i, j, k);
            if (i == n1)
                return -(5.0 * PV(i - 1, j, k) / 3.0 - F02 * PV(i - 2, j, k)) / hhr + 1.0 * PV(i - 1, j, k) / hr / rval * 0.5 -
                       (PV(i, j, ka) + PV(i, j, km)) / hhp / (rval * rval) + RF(i, j, k);
            return -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 0.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                   (PV(i, j, ka) + PV(i, j, km)) / hhp / (rval * rval) + RF(i, j, k);
        } else if (COMP == 2) {
            const double rval = L.rvc[i];
            const double rq = rval * rval;
            if (i == 1)
                return -(5.0 / 3.0 * PV(i + 1, j, k) - 0.2 * PV(i + 2, j, k)) / hhr - 4.0 / 3.0 * PV(i + 1, j, k) / hr / rval -
                       (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
            if (i == n1)
                return -(5.0 / 3.0 * PV(i - 1, j, k) - 0.2 * PV(i - 2, j, k)) / hhr + 4.0 / 3.0 * PV(i - 1, j, k) / hr / rval -
                       (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
            return -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                   (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
        } else {
            const double rval = L.rvv[i];
            const double rq = rval * rval;
            return -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                   (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
        }
    } else {
        const int i = p, j = q, k = e + 1;
        if (COMP == 1) {
            const double rval = L.rvc[i];
            if (i == 1)
                return -(5.0 * PV(i + 1, j, k) / 3.0 - F02 * PV(i + 2, j, k)) / hhr - PV(i + 1, j, k) / hr / rval * 0.5 -
                       (PV(i, j + 1, k) + PV(i, j - 1, k)) / hhz + RF(i, j, k);
            if (i == n1)
                return -(5.0 * PV(i - 1, j, k) / 3.0 - F02 * PV(i - 2, j, k)) / hhr + PV(i - 1, j, k) / hr / rval * 0.5 -
                       (PV(i, j + 1, k) + PV(i, j - 1, k)) / hhz + RF(i, j, k);
            return -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 0.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                   (PV(i, j + 1, k) + PV(i, j - 1, k)) / hhz + RF(i, j, k);
        } else if (COMP == 2) {
            const double rval = L.rvc[i];
            double rr;
            if (i == 1)
                rr = -(5.0 / 3.0 * PV(i + 1, j, k) - 0.2 * PV(i + 2, j, k)) / hhr - 4.0 / 3.0 * PV(i + 1, j, k) / hr / rval;
            else if (i == n1)
                rr = -(5.0 / 3.0 * PV(i - 1, j, k) - 0.2 * PV(i - 2, j, k)) / hhr + 4.0 / 3.0 * PV(i - 1, j, k) / hr / rval;
            else
                rr = -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval;
            if (j == 1) return rr - (5.0 / 3.0 * PV(i, j + 1, k) - 0.2 * PV(i, j + 2, k)) / hhz + RF(i, j, k);
            if (j == n2) return rr - (5.0 / 3.0 * PV(i, j - 1, k) - 0.2 * PV(i, j - 2, k)) / hhz + RF(i, j, k);
            return rr - (PV(i, j - 1, k) + PV(i, j + 1, k)) / hhz + RF(i, j, k);
        } else {
            const double rval = L.rvv[i];
            if (j == 1)
                return -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                       (5.0 * PV(i, j + 1, k) / 3.0 - F02 * PV(i, j + 2, k)) / hhz + RF(i, j, k);
            if (j == n2)
                return -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                       (5.0 * PV(i, j - 1, k) / 3.0 - F02 * PV(i, j - 2, k)) / hhz + RF(i, j, k);
            return -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                   (PV(i, j + 1, k) + PV(i, j - 1, k)) / hhz + RF(i, j, k);
        }
    }
}

// Solves line (p, q) of direction dir whose right-hand side s[0..n-1] a
// block formed beforehand in shared memory: the elimination runs in s and
// the solution goes to the level's correction v.  Lines along r and z on
// plane k = n3 also write plane 0; phi-lines write plane 0 from plane n3.
template <int COMP>
__device__ void r3_line(const R3Lev &L, const R3Work &W, int dir, int p, int q, double *s)
{
    const int n1 = L.n1, n2 = L.n2, n3 = L.n3, L1 = L.L1, L2 = L.L2;
    const int kind = r3_kind(COMP, dir);
    const int n = r3_len(COMP, dir, n1, n2, n3);
    double *v = W.v;
    size_t base;
    long long step;
    if (dir == 0) {
        base = (size_t)1 + (size_t)L1 * ((size_t)p + (size_t)L2 * (size_t)q);
        step = 1;
    } else if (dir == 1) {
        base = (size_t)p + (size_t)L1 * ((size_t)1 + (size_t)L2 * (size_t)q);
        step = L1;
    } else {
        base = (size_t)p + (size_t)L1 * ((size_t)q + (size_t)L2);
        step = (long long)L1 * L2;
    }
    const long long plane = (long long)L1 * L2 * n3;
    const bool seam = dir != 2 && q == n3;
    const double *T = L.fac[COMP][dir];
    if (dir != 0) T += (size_t)(p - 1) * r3_tabsize(kind, n);
#define PUT(e, x)                                                                     \
    do {                                                                              \
        const double _x = (x);                                                        \
        v[base + (size_t)((long long)(e) * step)] = _x;                               \
        if (seam) v[base + (size_t)((long long)(e) * step) - plane] = _x;             \
    } while (0)
    if (kind == 0) {
        const double *Cc = T, *Bb = T + n, *Aa = T + 2 * n, *Dd = T + 3 * n, *Ee = T + 4 * n, *iC = T + 5 * n;
        double r0 = s[0], r1 = s[1];
#pragma unroll 4
        for (int k = 0; k <= n - 2; ++k) {
            const double rk = div_by_rcp(r0, Cc[k], iC[k]);
            s[k] = rk;
            const double rk1 = r1 - Bb[k + 1] * rk;
            double rk2 = 0.0;
            if (k != n - 2) rk2 = s[k + 2] - Aa[k + 2] * rk;
            r0 = rk1;
            r1 = rk2;
        }
        double x1 = div_by_rcp(r0, Cc[n - 1], iC[n - 1]);
        PUT(n - 1, x1);
        double x0 = s[n - 2] - Dd[n - 2] * x1;
        PUT(n - 2, x0);
        double x2 = x1;
        x1 = x0;
#pragma unroll 4
        for (int j = n - 3; j >= 0; --j) {
            const double x = s[j] - Dd[j] * x1 - Ee[j] * x2;
            PUT(j, x);
            x2 = x1;
            x1 = x;
        }
    } else if (kind == 1) {
        const double *F = T, *Bb = T + n, *Cc = T + 2 * n, *iB = T + 3 * n;
        double rprev = s[0];
#pragma unroll 4
        for (int j = 1; j < n; ++j) {
            const double rj = s[j] - F[j] * rprev;
            s[j] = rj;
            rprev = rj;
        }
        double y = div_by_rcp(rprev, Bb[n - 1], iB[n - 1]);
        PUT(n - 1, y);
#pragma unroll 4
        for (int j = n - 2; j >= 0; --j) {
            y = div_by_rcp(s[j] - Cc[j] * y, Bb[j], iB[j]);
            PUT(j, y);
        }
    } else {
        const double *Aa = T, *Bb = T + n, *Cc = T + 2 * n, *F1 = T + 3 * n, *F2 = T + 4 * n, *F3 = T + 5 * n;
        const double *iB = T + 6 * n;
        const int N = n - 1;
        double rN = s[N];
        double rprev = s[0];
#pragma unroll 4
        for (int j = 1; j <= n - 3; ++j) {
            const double rj = s[j] - F1[j] * rprev;
            rN = rN - F2[j] * rprev;
            s[j] = rj;
            rprev = rj;
        }
        const double rn2 = s[n - 2] - F1[n - 2] * rprev;
        rN = rN - F2[n - 2] * rprev;
        rN = rN - F3[0] * rn2;
        const double yN = div_by_rcp(rN, Bb[N], iB[N]);
        PUT(N, yN);
        double y = div_by_rcp(rn2 - Cc[n - 2] * yN, Bb[n - 2], iB[n - 2]);
        PUT(n - 2, y);
#pragma unroll 4
        for (int j = n - 3; j >= 0; --j) {
            y = div_by_rcp(s[j] - Cc[j] * y - Aa[j] * yN, Bb[j], iB[j]);
            PUT(j, y);
        }
        v[base - (size_t)step] = yN;   // plane 0 = plane n3
    }
#undef PUT
}

// Shared memory of a solve block: right-hand sides of up to R3_SMEM_DOUBLES
// line elements (each line padded to an odd pitch against bank conflicts).
#define R3_SMEM_DOUBLES 6144

// One phase of independent lines [a, b) of the list: each block takes a
// contiguous share, forms the right-hand sides of a chunk of its lines with
// all its threads (every element independently, so the loads and divisions
// overlap), then one thread per line runs the elimination.
// A block's share of a phase's entries [a, b) starts at x moved forward
// past the rest of a group that x would split (entries marked as continued
// belong with the next one); every block moves its two ends the same way,
// so the shares still partition [a, b).
__device__ __forceinline__ int r3_group_start(const int *lines, int a, int b, int x)
{
    if (x >= b) return b;
    while (x > a && (lines[x - 1] & 0x80000000)) ++x;
    return x;
}

// End of a chunk [c0, c1): moved back to the end of the last whole group
// (groups never exceed a chunk; the phase lists are built so).
__device__ __forceinline__ int r3_chunk_end(const int *lines, int c0, int c1)
{
    int e = c1;
    while (e > c0 + 1 && (lines[e - 1] & 0x80000000)) --e;
    return e;
}

template <int COMP>
__device__ void r3_phase(const R3Lev &L, const R3Work &W, int dir, const int *lines, int a, int b, double *sm)
{
    const int n = r3_len(COMP, dir, L.n1, L.n2, L.n3);
    const int pitch = n | 1;
    const int per = (b - a + (int)gridDim.x - 1) / (int)gridDim.x;
    const int my0 = r3_group_start(lines, a, b, a + (int)blockIdx.x * per);
    const int my1 = r3_group_start(lines, a, b, a + ((int)blockIdx.x + 1) * per);
    const int chunk = max(1, min((int)blockDim.x, R3_SMEM_DOUBLES / pitch));
    for (int c0 = my0; c0 < my1;) {
        const int c1 = r3_chunk_end(lines, c0, min(my1, c0 + chunk));
        const int nl = c1 - c0;
        for (int t = threadIdx.x; t < nl * n; t += blockDim.x) {
            const int li = t / n, e = t - li * n;
            const int pk = lines[c0 + li] & 0x7fffffff;
            sm[li * pitch + e] = r3_rhs<COMP>(L, W, dir, pk & 0xffff, pk >> 16, e);
        }
        __syncthreads();
        if ((int)threadIdx.x < nl) {
            const int pk = lines[c0 + threadIdx.x] & 0x7fffffff;
            r3_line<COMP>(L, W, dir, pk & 0xffff, pk >> 16, sm + threadIdx.x * pitch);
        }
        __syncthreads();
        c0 = c1;
    }
}

// Residual rc = rf - A psif at the level's unknowns (relax1 :1688-1720,
// relax2 :1935-1977, relax3 :2129-2160), one point per call.
template <int COMP>
__device__ __forceinline__ double r3_resid(const R3Lev &L, const R3Work &W, int i, int j, int k)
{
    const int n1 = L.n1, n2 = L.n2, n3 = L.n3, L1 = L.L1, L2 = L.L2;
    const double hr = L.hr, hhr = L.hhr, hhz = L.hhz, hhp = L.hhp;
    const double *v = W.v, *f = W.f;
    const int ka = k == n3 ? 1 : k + 1, km = k - 1;
    double temp;
    if (COMP == 1) {
        const double rval = L.rvc[i];
        temp = (PV(i, j + 1, k) + PV(i, j - 1, k)) / hhz + (PV(i, j, ka) + PV(i, j, km)) / hhp / (rval * rval) -
               PV(i, j, k) * (2.0 / hhz + 2.0 / hhp / (rval * rval));
        if (i == 1)
            temp = temp + (-2.0 * PV(i, j, k) + 5.0 * PV(i + 1, j, k) / 3.0 - 0.2 * PV(i + 2, j, k)) / hhr +
                   0.5 * (-PV(i, j, k) + PV(i + 1, j, k)) / hr / rval;
        else if (i == n1)
            temp = temp + (-2.0 * PV(i, j, k) + 5.0 * PV(i - 1, j, k) / 3.0 - 0.2 * PV(i - 2, j, k)) / hhr +
                   0.5 * (PV(i, j, k) - PV(i - 1, j, k)) / hr / rval;
        else
            temp = temp + (PV(i - 1, j, k) - 2.0 * PV(i, j, k) + PV(i + 1, j, k)) / hhr +
                   0.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval;
    } else if (COMP == 2) {
        const double rval = L.rvc[i];
        const double rq = rval * rval;
        temp = (PV(i, j, ka) - 2.0 * PV(i, j, k) + PV(i, j, km)) / hhp / rq + PV(i, j, k) / rq;
        if (i == 1)
            temp = temp + (-2.0 * PV(i, j, k) + 5.0 / 3.0 * PV(i + 1, j, k) - 0.2 * PV(i + 2, j, k)) / hhr +
                   4.0 / 3.0 * PV(i + 1, j, k) / hr / rval;
        else if (i == n1)
            temp = temp + (-2.0 * PV(i, j, k) + 5.0 / 3.0 * PV(i - 1, j, k) - 0.2 * PV(i - 2, j, k)) / hhr -
                   4.0 / 3.0 * PV(i - 1, j, k) / hr / rval;
        else
            temp = temp + (PV(i - 1, j, k) - 2.0 * PV(i, j, k) + PV(i + 1, j, k)) / hhr +
                   1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval;
        if (j == 1)
            temp = temp + (-2.0 * PV(i, j, k) + 5.0 / 3.0 * PV(i, j + 1, k) - 0.2 * PV(i, j + 2, k)) / hhz;
        else if (j == n2)
            temp = temp + (-2.0 * PV(i, j, k) + 5.0 / 3.0 * PV(i, j - 1, k) - 0.2 * PV(i, j - 2, k)) / hhz;
        else
            temp = temp + (PV(i, j + 1, k) - 2.0 * PV(i, j, k) + PV(i, j - 1, k)) / hhz;
    } else {
        const double rval = L.rvv[i];
        const double rq = rval * rval;
        temp = (PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr + 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval +
               PV(i, j, k) / rq + (PV(i, j, ka) + PV(i, j, km)) / hhp / rq - PV(i, j, k) * (2.0 / hhr + 2.0 / hhp / rq);
        if (j == 1)
            temp = temp + (-2.0 * PV(i, j, k) + 5.0 * PV(i, j + 1, k) / 3.0 - 0.2 * PV(i, j + 2, k)) / hhz;
        else if (j == n2)
            temp = temp + (-2.0 * PV(i, j, k) + 5.0 * PV(i, j - 1, k) / 3.0 - 0.2 * PV(i, j - 2, k)) / hhz;
        else
            temp = temp + (PV(i, j + 1, k) - 2.0 * PV(i, j, k) + PV(i, j - 1, k)) / hhz;
    }
    return RF(i, j, k) - temp;
}

#undef PV
#undef RF

struct SolveCtx {
    int m;              // residual evaluations so far (selects the max slot)
};

// One relaxation call relax<COMP>(nrel, klev); returns false when a grid
// barrier timed out.
template <int COMP>
__device__ bool r3_relax(const R3Dev &d, int klev, SolveCtx &cx, double *sm)
{
    const R3Lev &L = d.lev[klev];
    const R3Work &W = d.work[COMP][klev];
    const GridSync &gs = d.gs[COMP];
    unsigned long long *resmax = d.resmax + 2 * COMP;
    int *nanflag = d.nanflag + 2 * COMP;
    const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long T = (long long)gridDim.x * blockDim.x;
    const int im = r3_imax(COMP, L.n1), jm = r3_jmax(COMP, L.n2), n3 = L.n3;
    for (int irel = 1; irel <= d.nrel; ++irel) {
        for (int dir = 0; dir < 3; ++dir) {
            const int *lines = L.lines[COMP][dir];
            const int *off = L.poff[COMP][dir];
            for (int ph = 0; ph < L.nphase[COMP][dir]; ++ph) {
                r3_phase<COMP>(L, W, dir, lines, off[ph], off[ph + 1], sm);
                if (!grid_sync(gs)) return false;
            }
        }
        // residual and its max norm into slot m & 1; the other slot is
        // cleared for the next evaluation (nobody reads it before then)
        const int slot = cx.m & 1;
        if (gt == 0) {
            resmax[slot ^ 1] = 0ull;
            nanflag[slot ^ 1] = 0;
        }
        const long long npts = (long long)im * jm * n3;
        double lmax = 0.0;
        int lnan = 0;
        for (long long t = gt; t < npts; t += T) {
            const int i = 1 + (int)(t % im);
            const long long rest = t / im;
            const int j = 1 + (int)(rest % jm);
            const int k = 1 + (int)(rest / jm);
            const double r = r3_resid<COMP>(L, W, i, j, k);
            W.res[(size_t)i + (size_t)L.L1 * ((size_t)j + (size_t)L.L2 * (size_t)k)] = r;
            const double a = fabs(r);
            if (a != a) lnan = 1;
            if (a > lmax) lmax = a;
        }
        for (int o = 16; o > 0; o >>= 1) {
            lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
            lnan |= __shfl_xor_sync(0xffffffffu, lnan, o);
        }
        if ((threadIdx.x & 31) == 0) {
            if (lmax > 0.0) atomicMax(&resmax[slot], (unsigned long long)__double_as_longlong(lmax));
            if (lnan) atomicOr(&nanflag[slot], 1);
        }
        cx.m++;
        if (!grid_sync(gs)) return false;
    }
    return true;
}

// corser (rot3dmg.f:2176-2265): coarse right-hand side and zero correction.
__device__ void r3_corser(const R3Dev &d, int comp, int klev)
{
    const R3Lev &F = d.lev[klev], &Cl = d.lev[klev + 1];
    const R3Work &FW = d.work[comp][klev], &CW = d.work[comp][klev + 1];
    const int n1c = Cl.n1, n2c = Cl.n2, n3c = Cl.n3;
    const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long T = (long long)gridDim.x * blockDim.x;
    const long long npts = (long long)Cl.L1 * Cl.L2 * (n3c + 1);
    const double *rf = FW.res;
    const size_t F1 = (size_t)F.L1, F2 = (size_t)F.L2;
#define R(i, j, k) rf[(size_t)(i) + F1 * ((size_t)(j) + F2 * (size_t)(k))]
    for (long long t = gt; t < npts; t += T) {
        const int i = (int)(t % Cl.L1);
        const long long rest = t / Cl.L1;
        const int j = (int)(rest % Cl.L2);
        const int k = (int)(rest / Cl.L2);
        double val;
        if (i == 0 || i == n1c || j == 0 || j == n2c) {
            val = 0.0;
        } else if (k == 0 || k == n3c) {
            val = R(i, j, k);
        } else {
            const int ii = i + i, jj = j + j, kk = k + k;
            const int iip = ii + 1, iim = ii - 1, jjp = jj + 1, jjm = jj - 1, kkp = kk + 1, kkm = kk - 1;
            double temp = R(ii, jj, kk);
            temp = temp + temp + R(iip, jj, kk) + R(iim, jj, kk) + R(ii, jjp, kk) + R(ii, jjm, kk) + R(ii, jj, kkp) +
                   R(ii, jj, kkm);
            temp = temp + temp + R(iip, jjp, kk) + R(iip, jjm, kk) + R(iim, jjp, kk) + R(iim, jjm, kk) + R(iip, jj, kkp) +
                   R(iip, jj, kkm) + R(iim, jj, kkp) + R(iim, jj, kkm) + R(ii, jjp, kkp) + R(ii, jjp, kkm) +
                   R(ii, jjm, kkp) + R(ii, jjm, kkm);
            temp = temp + temp + R(iip, jjp, kkp) + R(iip, jjp, kkm) + R(iip, jjm, kkp) + R(iip, jjm, kkm) +
                   R(iim, jjm, kkp) + R(iim, jjm, kkm) + R(iim, jjp, kkp) + R(iim, jjp, kkm);
            val = temp * 0.015625;
        }
        CW.f[t] = val;
        CW.v[t] = 0.0;
    }
#undef R
}

// finer (rot3dmg.f:2268-2344): trilinear prolongation added to the fine
// level.  The coarse correction is cleared by the next corser.
__device__ void r3_finer(const R3Dev &d, int comp, int klev)
{
    const R3Lev &Cl = d.lev[klev], &F = d.lev[klev - 1];
    const R3Work &CW = d.work[comp][klev], &FW = d.work[comp][klev - 1];
    const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long T = (long long)gridDim.x * blockDim.x;
    const long long npts = (long long)F.L1 * F.L2 * (F.n3 + 1);
    const double *pc = CW.v;
    const size_t C1 = (size_t)Cl.L1, C2 = (size_t)Cl.L2;
#define PC(i, j, k) pc[(size_t)(i) + C1 * ((size_t)(j) + C2 * (size_t)(k))]
    for (long long t = gt; t < npts; t += T) {
        const int i = (int)(t % F.L1);
        const long long rest = t / F.L1;
        const int j = (int)(rest % F.L2);
        const int k = (int)(rest / F.L2);
        const int i1 = i / 2, j1 = j / 2, k1 = k / 2;
        const bool ie = i1 * 2 == i, je = j1 * 2 == j, ke = k1 * 2 == k;
        double p;
        if (ie) {
            if (je) {
                if (ke) p = PC(i1, j1, k1);
                else p = (PC(i1, j1, k1) + PC(i1, j1, k1 + 1)) * 0.5;
            } else {
                if (ke) p = (PC(i1, j1, k1) + PC(i1, j1 + 1, k1)) * 0.5;
                else p = (PC(i1, j1, k1) + PC(i1, j1 + 1, k1) + PC(i1, j1, k1 + 1) + PC(i1, j1 + 1, k1 + 1)) * 0.25;
            }
        } else {
            if (je) {
                if (ke) p = (PC(i1, j1, k1) + PC(i1 + 1, j1, k1)) * 0.5;
                else p = (PC(i1, j1, k1) + PC(i1 + 1, j1, k1) + PC(i1, j1, k1 + 1) + PC(i1 + 1, j1, k1 + 1)) * 0.25;
            } else {
                if (ke)
                    p = (PC(i1, j1, k1) + PC(i1 + 1, j1, k1) + PC(i1, j1 + 1, k1) + PC(i1 + 1, j1 + 1, k1)) * 0.25;
                else
                    p = (PC(i1, j1, k1) + PC(i1 + 1, j1, k1) + PC(i1, j1 + 1, k1) + PC(i1 + 1, j1 + 1, k1) +
                         PC(i1, j1, k1 + 1) + PC(i1 + 1, j1, k1 + 1) + PC(i1, j1 + 1, k1 + 1) +
                         PC(i1 + 1, j1 + 1, k1 + 1)) *
                        0.125;
            }
        }
        FW.v[t] = p + FW.v[t];
    }
#undef PC
}

// poisson1/2/3 (rot3dmg.f:1216-1540) in one cooperative launch.
template <int COMP>
__global__ void __launch_bounds__(R3_THREADS, 2) k_r3d_solve(const __grid_constant__ R3Dev d, int step)
{
    __shared__ double sm[R3_SMEM_DOUBLES];
    if (*(volatile int *)d.abort) return;
    const int ni = d.ni, nj = d.nj;
    const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long T = (long long)gridDim.x * blockDim.x;
    double *psi = d.fld[COMP == 1 ? GB_R_wel : COMP == 2 ? GB_R_vel : GB_R_uel];
    double *psip = d.fld[COMP == 1 ? GB_R_welp : COMP == 2 ? GB_R_velp : GB_R_uelp];
    const double *rhs = d.fld[COMP == 1 ? GB_R_wrh : COMP == 2 ? GB_R_vrh : GB_R_urh];
    const R3Lev &L = d.lev[1];
    const R3Work &W = d.work[COMP][1];
    const GridSync &gs = d.gs[COMP];
    const long long n1p = L.L1, n2p = L.L2;
    const long long nlvl = n1p * n2p * (L.n3 + 1);
    for (long long t = gt; t < nlvl; t += T) {
        const int i = (int)(t % n1p);
        const long long rest = t / n1p;
        const int j = (int)(rest % n2p);
        const int k = (int)(rest / n2p);
        W.f[t] = FX(rhs, i, j, k);
        W.v[t] = 2.0 * FX(psi, i, j, k) - FX(psip, i, j, k);
    }
    if (!grid_sync(gs)) return;
    SolveCtx cx;
    cx.m = 0;
    int status = GB_MAXSWEEPS, sweeps = d.maxsweeps;
    const int nlev = d.nlev;
    for (int sweep = 1; sweep <= d.maxsweeps; ++sweep) {
        if (sweep != 1 && !d.horizontal) {
            for (long long t = gt; t < nlvl; t += T) {
                const int i = (int)(t % n1p);
                const long long rest = t / n1p;
                const int j = (int)(rest % n2p);
                const int k = (int)(rest / n2p);
                const double pp = FX(psip, i, j, k);
                const double nv = pp + d.sor * (W.v[t] - pp);
                W.v[t] = nv;
                FX(psip, i, j, k) = nv;
            }
            if (!grid_sync(gs)) return;
        }
        if (sweep == 1 || nlev == 1) {
            if (!r3_relax<COMP>(d, 1, cx, sm)) return;
            if (!d.horizontal) {
                for (long long t = gt; t < nlvl; t += T) {
                    const int i = (int)(t % n1p);
                    const long long rest = t / n1p;
                    const int j = (int)(rest % n2p);
                    const int k = (int)(rest / n2p);
                    FX(psip, i, j, k) = W.v[t];
                }
                if (!grid_sync(gs)) return;
            }
        }
        if (nlev > 1) {
            for (int l = 1; l <= nlev - 1; ++l) {
                r3_corser(d, COMP, l);
                if (!grid_sync(gs)) return;
                if (!r3_relax<COMP>(d, l + 1, cx, sm)) return;
            }
            for (int l = nlev; l >= 2; --l) {
                r3_finer(d, COMP, l);
                if (!grid_sync(gs)) return;
                if (!r3_relax<COMP>(d, l - 1, cx, sm)) return;
            }
        }
        const int slot = (cx.m - 1) & 1;
        const double resmax =
            __longlong_as_double((long long)*(volatile unsigned long long *)&d.resmax[2 * COMP + slot]);
        if (*(volatile int *)&d.nanflag[2 * COMP + slot]) {
            status = GB_NAN;
            sweeps = sweep;
            break;
        }
        if (resmax < d.tolcon) {
            status = GB_OK;
            sweeps = sweep;
            break;
        }
    }
    if (status == GB_OK) {
        const int imax = COMP == 3 ? d.nr : d.nr + 1;
        const int jmax = COMP == 1 ? d.nz : d.nz + 1;
        const int ii1 = COMP == 3 ? d.nr - 1 : d.nr;
        const int jj1 = COMP == 1 ? d.nz - 1 : d.nz;
        const long long npts = (long long)(imax + 1) * (jmax + 1) * (d.np + 1);
        for (long long t = gt; t < npts; t += T) {
            const int i = (int)(t % (imax + 1));
            const long long rest = t / (imax + 1);
            const int j = (int)(rest % (jmax + 1));
            const int k = (int)(rest / (jmax + 1));
            const double old = FX(psi, i, j, k);
            FX(psip, i, j, k) = old;
            const bool inner = i >= 1 && i <= ii1 && j >= 1 && j <= jj1;
            FX(psi, i, j, k) = inner ? W.v[(size_t)i + (size_t)n1p * ((size_t)j + (size_t)n2p * (size_t)k)] : 0.0;
        }
    }
    if (gt == 0) {
        d.solve_status[COMP] = status;
        d.solve_sweeps[COMP] = sweeps;
        if (step >= 0) d.hist_sw[3 * step + COMP - 1] = sweeps;
        if (status != GB_OK) atomicExch(d.abort, status);
    }
}

// ---------------------------------------------------------------------------
// Mixed precision (GB_PRB_MIXED): FP32 V-cycles on the residual equation
// inside an FP64 defect correction.  The FP32 operator is the reference's
// operator with every division by a level constant or a radius replaced by
// a multiplication with its reciprocal; pivots of the factor tables are
// stored as reciprocals.
// ---------------------------------------------------------------------------

// FP32 copies of the factor tables (one thread per line class).
__global__ void k_r3d_factors32(const __grid_constant__ R3Dev d, const FacJob *jobs, int njobs, float *const *dst)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= njobs) return;
    const FacJob J = jobs[q];
    const R3Lev &L = d.lev[J.lev];
    const int kind = r3_kind(J.comp, J.dir);
    const int n = r3_len(J.comp, J.dir, L.n1, L.n2, L.n3);
    const double *T = J.tab;
    float *o = dst[q];
    const int m = r3_tabsize(kind, n);
    for (int t = 0; t < m; ++t) o[t] = (float)T[t];
    if (kind == 0)
        for (int t = 0; t < n; ++t) o[t] = (float)(1.0 / T[t]);            // divisors c(k)
    else
        for (int t = 0; t < n; ++t) o[n + t] = (float)(1.0 / T[n + t]);    // eliminated diagonal b
}

#define PV(i, j, k) v[(size_t)(i) + (size_t)L1 * ((size_t)(j) + (size_t)L2 * (size_t)(k))]
#define RF(i, j, k) f[(size_t)(i) + (size_t)L1 * ((size_t)(j) + (size_t)L2 * (size_t)(k))]

template <int COMP>
__device__ __forceinline__ float r3_rhs32(const R3Lev &L, const R3Work &W, int dir, int p, int q, int e)
{
    const int n1 = L.n1, n2 = L.n2, n3 = L.n3, L1 = L.L1, L2 = L.L2;
    const float ihr = L.ihr, ihhr = L.ihhr, ihhz = L.ihhz, ihhp = L.ihhp;
    const float c53 = 5.0f / 3.0f, c43 = 4.0f / 3.0f;
    const float *v = W.v32, *f = W.f32;
    if (dir == 0) {
        const int i = e + 1, j = p, k = q;
        const int ka = k == n3 ? 1 : k + 1, km = k - 1;
        const float iq = COMP == 3 ? L.iqv[i] : L.iqc[i];
        const float ph = (PV(i, j, ka) + PV(i, j, km)) * ihhp * iq;
        float zz;
        if (COMP == 1) zz = (PV(i, j + 1, k) + PV(i, j - 1, k)) * ihhz;
        else if (j == 1) zz = (c53 * PV(i, j + 1, k) - 0.2f * PV(i, j + 2, k)) * ihhz;
        else if (j == n2) zz = (c53 * PV(i, j - 1, k) - 0.2f * PV(i, j - 2, k)) * ihhz;
        else zz = (PV(i, j - 1, k) + PV(i, j + 1, k)) * ihhz;
        return RF(i, j, k) - zz - ph;
    } else if (dir == 1) {
        const int i = p, j = e + 1, k = q;
        const int ka = k == n3 ? 1 : k + 1, km = k - 1;
        const float iq = COMP == 3 ? L.iqv[i] : L.iqc[i];
        const float ir = COMP == 3 ? L.irv[i] : L.irc[i];
        const float ph = (PV(i, j, ka) + PV(i, j, km)) * ihhp * iq;
        float rr;
        if (COMP == 1) {
            if (i == 1) rr = -(c53 * PV(i + 1, j, k) - 0.2f * PV(i + 2, j, k)) * ihhr - 0.5f * PV(i + 1, j, k) * ihr * ir;
            else if (i == n1) rr = -(c53 * PV(i - 1, j, k) - 0.2f * PV(i - 2, j, k)) * ihhr + 0.5f * PV(i - 1, j, k) * ihr * ir;
            else rr = -(PV(i + 1, j, k) + PV(i - 1, j, k)) * ihhr - 0.5f * (PV(i + 1, j, k) - PV(i - 1, j, k)) * ihr * ir;
        } else if (COMP == 2) {
            if (i == 1) rr = -(c53 * PV(i + 1, j, k) - 0.2f * PV(i + 2, j, k)) * ihhr - c43 * PV(i + 1, j, k) * ihr * ir;
            else if (i == n1) rr = -(c53 * PV(i - 1, j, k) - 0.2f * PV(i - 2, j, k)) * ihhr + c43 * PV(i - 1, j, k) * ihr * ir;
            else rr = -(PV(i + 1, j, k) + PV(i - 1, j, k)) * ihhr - 1.5f * (PV(i + 1, j, k) - PV(i - 1, j, k)) * ihr * ir;
        } else {
            rr = -(PV(i + 1, j, k) + PV(i - 1, j, k)) * ihhr - 1.5f * (PV(i + 1, j, k) - PV(i - 1, j, k)) * ihr * ir;
        }
        return rr - ph + RF(i, j, k);
    } else {
        const int i = p, j = q, k = e + 1;
        const float ir = COMP == 3 ? L.irv[i] : L.irc[i];
        float rr;
        if (COMP == 1) {
            if (i == 1) rr = -(c53 * PV(i + 1, j, k) - 0.2f * PV(i + 2, j, k)) * ihhr - 0.5f * PV(i + 1, j, k) * ihr * ir;
            else if (i == n1) rr = -(c53 * PV(i - 1, j, k) - 0.2f * PV(i - 2, j, k)) * ihhr + 0.5f * PV(i - 1, j, k) * ihr * ir;
            else rr = -(PV(i + 1, j, k) + PV(i - 1, j, k)) * ihhr - 0.5f * (PV(i + 1, j, k) - PV(i - 1, j, k)) * ihr * ir;
        } else if (COMP == 2) {
            if (i == 1) rr = -(c53 * PV(i + 1, j, k) - 0.2f * PV(i + 2, j, k)) * ihhr - c43 * PV(i + 1, j, k) * ihr * ir;
            else if (i == n1) rr = -(c53 * PV(i - 1, j, k) - 0.2f * PV(i - 2, j, k)) * ihhr + c43 * PV(i - 1, j, k) * ihr * ir;
            else rr = -(PV(i + 1, j, k) + PV(i - 1, j, k)) * ihhr - 1.5f * (PV(i + 1, j, k) - PV(i - 1, j, k)) * ihr * ir;
        } else {
            rr = -(PV(i + 1, j, k) + PV(i - 1, j, k)) * ihhr - 1.5f * (PV(i + 1, j, k) - PV(i - 1, j, k)) * ihr * ir;
        }
        float zz;
        if (COMP == 1) zz = (PV(i, j + 1, k) + PV(i, j - 1, k)) * ihhz;
        else if (j == 1) zz = (c53 * PV(i, j + 1, k) - 0.2f * PV(i, j + 2, k)) * ihhz;
        else if (j == n2) zz = (c53 * PV(i, j - 1, k) - 0.2f * PV(i, j - 2, k)) * ihhz;
        else zz = (PV(i, j - 1, k) + PV(i, j + 1, k)) * ihhz;
        return rr - zz + RF(i, j, k);
    }
}

// FP32 residual (only where a restriction follows).
template <int COMP>
__device__ __forceinline__ float r3_resid32(const R3Lev &L, const R3Work &W, int i, int j, int k)
{
    const int n1 = L.n1, n2 = L.n2, n3 = L.n3, L1 = L.L1, L2 = L.L2;
    const float ihr = L.ihr, ihhr = L.ihhr, ihhz = L.ihhz, ihhp = L.ihhp;
    const float c53 = 5.0f / 3.0f, c43 = 4.0f / 3.0f;
    const float *v = W.v32, *f = W.f32;
    const int ka = k == n3 ? 1 : k + 1, km = k - 1;
    const float p0 = PV(i, j, k);
    const float iq = COMP == 3 ? L.iqv[i] : L.iqc[i];
    const float ir = COMP == 3 ? L.irv[i] : L.irc[i];
    float t = (PV(i, j, ka) - 2.0f * p0 + PV(i, j, km)) * ihhp * iq;
    if (COMP == 1) {
        t += (PV(i, j + 1, k) - 2.0f * p0 + PV(i, j - 1, k)) * ihhz;
        if (i == 1) t += (-2.0f * p0 + c53 * PV(i + 1, j, k) - 0.2f * PV(i + 2, j, k)) * ihhr + 0.5f * (PV(i + 1, j, k) - p0) * ihr * ir;
        else if (i == n1) t += (-2.0f * p0 + c53 * PV(i - 1, j, k) - 0.2f * PV(i - 2, j, k)) * ihhr + 0.5f * (p0 - PV(i - 1, j, k)) * ihr * ir;
        else t += (PV(i - 1, j, k) - 2.0f * p0 + PV(i + 1, j, k)) * ihhr + 0.5f * (PV(i + 1, j, k) - PV(i - 1, j, k)) * ihr * ir;
    } else {
        t += p0 * iq;
        if (COMP == 2) {
            if (i == 1) t += (-2.0f * p0 + c53 * PV(i + 1, j, k) - 0.2f * PV(i + 2, j, k)) * ihhr + c43 * PV(i + 1, j, k) * ihr * ir;
            else if (i == n1) t += (-2.0f * p0 + c53 * PV(i - 1, j, k) - 0.2f * PV(i - 2, j, k)) * ihhr - c43 * PV(i - 1, j, k) * ihr * ir;
            else t += (PV(i - 1, j, k) - 2.0f * p0 + PV(i + 1, j, k)) * ihhr + 1.5f * (PV(i + 1, j, k) - PV(i - 1, j, k)) * ihr * ir;
        } else {
            t += (PV(i - 1, j, k) - 2.0f * p0 + PV(i + 1, j, k)) * ihhr + 1.5f * (PV(i + 1, j, k) - PV(i - 1, j, k)) * ihr * ir;
        }
        if (j == 1) t += (-2.0f * p0 + c53 * PV(i, j + 1, k) - 0.2f * PV(i, j + 2, k)) * ihhz;
        else if (j == n2) t += (-2.0f * p0 + c53 * PV(i, j - 1, k) - 0.2f * PV(i, j - 2, k)) * ihhz;
        else t += (PV(i, j + 1, k) - 2.0f * p0 + PV(i, j - 1, k)) * ihhz;
    }
    return RF(i, j, k) - t;
}

#undef PV
#undef RF

template <int COMP>
__device__ void r3_line32(const R3Lev &L, const R3Work &W, int dir, int p, int q, float *s)
{
    const int n1 = L.n1, n2 = L.n2, n3 = L.n3, L1 = L.L1, L2 = L.L2;
    const int kind = r3_kind(COMP, dir);
    const int n = r3_len(COMP, dir, n1, n2, n3);
    float *v = W.v32;
    size_t base;
    long long step;
    if (dir == 0) {
        base = (size_t)1 + (size_t)L1 * ((size_t)p + (size_t)L2 * (size_t)q);
        step = 1;
    } else if (dir == 1) {
        base = (size_t)p + (size_t)L1 * ((size_t)1 + (size_t)L2 * (size_t)q);
        step = L1;
    } else {
        base = (size_t)p + (size_t)L1 * ((size_t)q + (size_t)L2);
        step = (long long)L1 * L2;
    }
    const long long plane = (long long)L1 * L2 * n3;
    const bool seam = dir != 2 && q == n3;
    const float *T = L.fac32[COMP][dir];
    if (dir != 0) T += (size_t)(p - 1) * r3_tabsize(kind, n);
#define PUT(e, x)                                                                     \
    do {                                                                              \
        const float _x = (x);                                                         \
        v[base + (size_t)((long long)(e) * step)] = _x;                               \
        if (seam) v[base + (size_t)((long long)(e) * step) - plane] = _x;             \
    } while (0)
    if (kind == 0) {
        const float *Ci = T, *Bb = T + n, *Aa = T + 2 * n, *Dd = T + 3 * n, *Ee = T + 4 * n;
        float r0 = s[0], r1 = s[1];
#pragma unroll 4
        for (int k = 0; k <= n - 2; ++k) {
            const float rk = r0 * Ci[k];
            s[k] = rk;
            const float rk1 = __fmaf_rn(-Bb[k + 1], rk, r1);
            float rk2 = 0.f;
            if (k != n - 2) rk2 = __fmaf_rn(-Aa[k + 2], rk, s[k + 2]);
            r0 = rk1;
            r1 = rk2;
        }
        float x1 = r0 * Ci[n - 1];
        PUT(n - 1, x1);
        float x0 = __fmaf_rn(-Dd[n - 2], x1, s[n - 2]);
        PUT(n - 2, x0);
        float x2 = x1;
        x1 = x0;
#pragma unroll 4
        for (int j = n - 3; j >= 0; --j) {
            const float x = __fmaf_rn(-Ee[j], x2, __fmaf_rn(-Dd[j], x1, s[j]));
            PUT(j, x);
            x2 = x1;
            x1 = x;
        }
    } else if (kind == 1) {
        const float *F = T, *Bi = T + n, *Cc = T + 2 * n;
        float rprev = s[0];
#pragma unroll 4
        for (int j = 1; j < n; ++j) {
            const float rj = __fmaf_rn(-F[j], rprev, s[j]);
            s[j] = rj;
            rprev = rj;
        }
        float y = rprev * Bi[n - 1];
        PUT(n - 1, y);
#pragma unroll 4
        for (int j = n - 2; j >= 0; --j) {
            y = __fmaf_rn(-Cc[j], y, s[j]) * Bi[j];
            PUT(j, y);
        }
    } else {
        const float *Aa = T, *Bi = T + n, *Cc = T + 2 * n, *F1 = T + 3 * n, *F2 = T + 4 * n, *F3 = T + 5 * n;
        const int N = n - 1;
        float rN = s[N];
        float rprev = s[0];
#pragma unroll 4
        for (int j = 1; j <= n - 3; ++j) {
            const float rj = __fmaf_rn(-F1[j], rprev, s[j]);
            rN = __fmaf_rn(-F2[j], rprev, rN);
            s[j] = rj;
            rprev = rj;
        }
        const float rn2 = __fmaf_rn(-F1[n - 2], rprev, s[n - 2]);
        rN = __fmaf_rn(-F2[n - 2], rprev, rN);
        rN = __fmaf_rn(-F3[0], rn2, rN);
        const float yN = rN * Bi[N];
        PUT(N, yN);
        float y = __fmaf_rn(-Cc[n - 2], yN, rn2) * Bi[n - 2];
        PUT(n - 2, y);
#pragma unroll 4
        for (int j = n - 3; j >= 0; --j) {
            y = __fmaf_rn(-Aa[j], yN, __fmaf_rn(-Cc[j], y, s[j])) * Bi[j];
            PUT(j, y);
        }
        v[base - (size_t)step] = yN;
    }
#undef PUT
}

template <int COMP>
__device__ void r3_phase32(const R3Lev &L, const R3Work &W, int dir, const int *lines, int a, int b, float *sm)
{
    const int n = r3_len(COMP, dir, L.n1, L.n2, L.n3);
    const int pitch = n | 1;
    const int per = (b - a + (int)gridDim.x - 1) / (int)gridDim.x;
    const int my0 = r3_group_start(lines, a, b, a + (int)blockIdx.x * per);
    const int my1 = r3_group_start(lines, a, b, a + ((int)blockIdx.x + 1) * per);
    const int chunk = max(1, min((int)blockDim.x, (2 * R3_SMEM_DOUBLES) / pitch));
    for (int c0 = my0; c0 < my1;) {
        const int c1 = r3_chunk_end(lines, c0, min(my1, c0 + chunk));
        const int nl = c1 - c0;
        for (int t = threadIdx.x; t < nl * n; t += blockDim.x) {
            const int li = t / n, e = t - li * n;
            const int pk = lines[c0 + li] & 0x7fffffff;
            sm[li * pitch + e] = r3_rhs32<COMP>(L, W, dir, pk & 0xffff, pk >> 16, e);
        }
        __syncthreads();
        if ((int)threadIdx.x < nl) {
            const int pk = lines[c0 + threadIdx.x] & 0x7fffffff;
            r3_line32<COMP>(L, W, dir, pk & 0xffff, pk >> 16, sm + threadIdx.x * pitch);
        }
        __syncthreads();
        c0 = c1;
    }
}

// relax in FP32; the residual only when a restriction follows.
template <int COMP>
__device__ bool r3_relax32(const R3Dev &d, int klev, bool residual, float *sm)
{
    const R3Lev &L = d.lev[klev];
    const R3Work &W = d.work[COMP][klev];
    const GridSync &gs = d.gs[COMP];
    const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long T = (long long)gridDim.x * blockDim.x;
    const int im = r3_imax(COMP, L.n1), jm = r3_jmax(COMP, L.n2), n3 = L.n3;
    for (int irel = 1; irel <= d.nrel; ++irel)
        for (int dir = 0; dir < 3; ++dir) {
            const int *lines = L.lines[COMP][dir];
            const int *off = L.poff[COMP][dir];
            for (int ph = 0; ph < L.nphase[COMP][dir]; ++ph) {
                r3_phase32<COMP>(L, W, dir, lines, off[ph], off[ph + 1], sm);
                if (!grid_sync(gs)) return false;
            }
        }
    if (residual) {
        const long long npts = (long long)im * jm * n3;
        for (long long t = gt; t < npts; t += T) {
            const int i = 1 + (int)(t % im);
            const long long rest = t / im;
            const int j = 1 + (int)(rest % jm);
            const int k = 1 + (int)(rest / jm);
            W.res32[(size_t)i + (size_t)L.L1 * ((size_t)j + (size_t)L.L2 * (size_t)k)] = r3_resid32<COMP>(L, W, i, j, k);
        }
        if (!grid_sync(gs)) return false;
    }
    return true;
}

__device__ void r3_corser32(const R3Dev &d, int comp, int klev)
{
    const R3Lev &F = d.lev[klev], &Cl = d.lev[klev + 1];
    const R3Work &WF = d.work[comp][klev], &WC = d.work[comp][klev + 1];
    const int n1c = Cl.n1, n2c = Cl.n2, n3c = Cl.n3;
    const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long T = (long long)gridDim.x * blockDim.x;
    const long long npts = (long long)Cl.L1 * Cl.L2 * (n3c + 1);
    const float *rf = WF.res32;
    const size_t F1 = (size_t)F.L1, F2 = (size_t)F.L2;
#define R(i, j, k) rf[(size_t)(i) + F1 * ((size_t)(j) + F2 * (size_t)(k))]
    for (long long t = gt; t < npts; t += T) {
        const int i = (int)(t % Cl.L1);
        const long long rest = t / Cl.L1;
        const int j = (int)(rest % Cl.L2);
        const int k = (int)(rest / Cl.L2);
        float val;
        if (i == 0 || i == n1c || j == 0 || j == n2c) {
            val = 0.f;
        } else if (k == 0 || k == n3c) {
            val = k == 0 ? 0.f : R(i, j, k);
        } else {
            const int ii = i + i, jj = j + j, kk = k + k;
            float c = 0.f;
#pragma unroll
            for (int dk = -1; dk <= 1; ++dk)
#pragma unroll
                for (int dj = -1; dj <= 1; ++dj)
#pragma unroll
                    for (int di = -1; di <= 1; ++di) {
                        const float w = (di ? 0.5f : 1.f) * (dj ? 0.5f : 1.f) * (dk ? 0.5f : 1.f);
                        c = __fmaf_rn(w, R(ii + di, jj + dj, kk + dk), c);
                    }
            val = c * 0.125f;
        }
        WC.f32[t] = val;
        WC.v32[t] = 0.f;
    }
#undef R
}

__device__ void r3_finer32(const R3Dev &d, int comp, int klev)
{
    const R3Lev &Cl = d.lev[klev], &F = d.lev[klev - 1];
    const R3Work &WC = d.work[comp][klev], &WF = d.work[comp][klev - 1];
    const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long T = (long long)gridDim.x * blockDim.x;
    const long long npts = (long long)F.L1 * F.L2 * (F.n3 + 1);
    const float *pc = WC.v32;
    const size_t C1 = (size_t)Cl.L1, C2 = (size_t)Cl.L2;
#define PC(i, j, k) pc[(size_t)(i) + C1 * ((size_t)(j) + C2 * (size_t)(k))]
    for (long long t = gt; t < npts; t += T) {
        const int i = (int)(t % F.L1);
        const long long rest = t / F.L1;
        const int j = (int)(rest % F.L2);
        const int k = (int)(rest / F.L2);
        const int i1 = i >> 1, j1 = j >> 1, k1 = k >> 1;
        const int i2 = i1 + (i & 1), j2 = j1 + (j & 1), k2 = k1 + (k & 1);
        const float p = 0.125f * (PC(i1, j1, k1) + PC(i2, j1, k1) + PC(i1, j2, k1) + PC(i2, j2, k1) + PC(i1, j1, k2) +
                                  PC(i2, j1, k2) + PC(i1, j2, k2) + PC(i2, j2, k2));
        WF.v32[t] += p;
    }
#undef PC
}

// poisson1/2/3 in mixed precision: the FP64 iterate lives in level 1's v,
// the FP64 right-hand side in level 1's f.
template <int COMP>
__global__ void __launch_bounds__(R3_THREADS, 2) k_r3d_solve_mixed(const __grid_constant__ R3Dev d, int step)
{
    __shared__ float sm[2 * R3_SMEM_DOUBLES];
    if (*(volatile int *)d.abort) return;
    const int ni = d.ni, nj = d.nj;
    const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long T = (long long)gridDim.x * blockDim.x;
    double *psi = d.fld[COMP == 1 ? GB_R_wel : COMP == 2 ? GB_R_vel : GB_R_uel];
    double *psip = d.fld[COMP == 1 ? GB_R_welp : COMP == 2 ? GB_R_velp : GB_R_uelp];
    const double *rhs = d.fld[COMP == 1 ? GB_R_wrh : COMP == 2 ? GB_R_vrh : GB_R_urh];
    const R3Lev &L = d.lev[1];
    const R3Work &W = d.work[COMP][1];
    const GridSync &gs = d.gs[COMP];
    const long long n1p = L.L1, n2p = L.L2;
    const long long nlvl = n1p * n2p * (L.n3 + 1);
    for (long long t = gt; t < nlvl; t += T) {
        const int i = (int)(t % n1p);
        const long long rest = t / n1p;
        const int j = (int)(rest % n2p);
        const int k = (int)(rest / n2p);
        W.f[t] = FX(rhs, i, j, k);
        W.v[t] = 2.0 * FX(psi, i, j, k) - FX(psip, i, j, k);
        W.f32[t] = 0.f;
    }
    if (!grid_sync(gs)) return;
    const int im = r3_imax(COMP, L.n1), jm = r3_jmax(COMP, L.n2), n3 = L.n3;
    const long long nunk = (long long)im * jm * n3;
    int status = GB_MAXSWEEPS, cycles = d.maxsweeps, m = 0;
    const int nlev = d.nlev;
    for (int it = 0;; ++it) {
        // FP64 residual of the iterate, its FP32 copy the cycle's right-hand side
        const int slot = m & 1;
        if (gt == 0) {
            d.resmax[2 * COMP + (slot ^ 1)] = 0ull;
            d.nanflag[2 * COMP + (slot ^ 1)] = 0;
        }
        double lmax = 0.0;
        int lnan = 0;
        for (long long t = gt; t < nunk; t += T) {
            const int i = 1 + (int)(t % im);
            const long long rest = t / im;
            const int j = 1 + (int)(rest % jm);
            const int k = 1 + (int)(rest / jm);
            const double r = r3_resid<COMP>(L, W, i, j, k);
            W.f32[(size_t)i + (size_t)L.L1 * ((size_t)j + (size_t)L.L2 * (size_t)k)] = (float)r;
            const double a = fabs(r);
            if (a != a) lnan = 1;
            if (a > lmax) lmax = a;
        }
        for (int o = 16; o > 0; o >>= 1) {
            lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
            lnan |= __shfl_xor_sync(0xffffffffu, lnan, o);
        }
        if ((threadIdx.x & 31) == 0) {
            if (lmax > 0.0) atomicMax(&d.resmax[2 * COMP + slot], (unsigned long long)__double_as_longlong(lmax));
            if (lnan) atomicOr(&d.nanflag[2 * COMP + slot], 1);
        }
        ++m;
        if (!grid_sync(gs)) return;
        const double res = __longlong_as_double((long long)*(volatile unsigned long long *)&d.resmax[2 * COMP + slot]);
        if (*(volatile int *)&d.nanflag[2 * COMP + slot]) {
            status = GB_NAN;
            cycles = it;
            break;
        }
        if (res < d.tolcon) {
            status = GB_OK;
            cycles = it;
            break;
        }
        if (it == d.maxsweeps) break;
        // e = 0, one FP32 cycle: relax on level 1, descent, ascent
        for (long long t = gt; t < nlvl; t += T) W.v32[t] = 0.f;
        if (!grid_sync(gs)) return;
        if (!r3_relax32<COMP>(d, 1, nlev > 1, sm)) return;
        for (int l = 1; l <= nlev - 1; ++l) {
            r3_corser32(d, COMP, l);
            if (!grid_sync(gs)) return;
            if (!r3_relax32<COMP>(d, l + 1, l + 1 < nlev, sm)) return;
        }
        for (int l = nlev; l >= 2; --l) {
            r3_finer32(d, COMP, l);
            if (!grid_sync(gs)) return;
            if (!r3_relax32<COMP>(d, l - 1, false, sm)) return;
        }
        const double w = (it == 0 || d.horizontal) ? 1.0 : d.sor;
        for (long long t = gt; t < nlvl; t += T) W.v[t] += w * (double)W.v32[t];
        if (!grid_sync(gs)) return;
    }
    if (status == GB_OK) {
        const int imax = COMP == 3 ? d.nr : d.nr + 1;
        const int jmax = COMP == 1 ? d.nz : d.nz + 1;
        const int ii1 = COMP == 3 ? d.nr - 1 : d.nr;
        const int jj1 = COMP == 1 ? d.nz - 1 : d.nz;
        const long long npts = (long long)(imax + 1) * (jmax + 1) * (d.np + 1);
        for (long long t = gt; t < npts; t += T) {
            const int i = (int)(t % (imax + 1));
            const long long rest = t / (imax + 1);
            const int j = (int)(rest % (jmax + 1));
            const int k = (int)(rest / (jmax + 1));
            const double old = FX(psi, i, j, k);
            FX(psip, i, j, k) = old;
            const bool inner = i >= 1 && i <= ii1 && j >= 1 && j <= jj1;
            FX(psi, i, j, k) = inner ? W.v[(size_t)i + (size_t)n1p * ((size_t)j + (size_t)n2p * (size_t)k)] : 0.0;
        }
    }
    if (gt == 0) {
        d.solve_status[COMP] = status;
        d.solve_sweeps[COMP] = cycles;
        if (step >= 0) d.hist_sw[3 * step + COMP - 1] = cycles;
        if (status != GB_OK) atomicExch(d.abort, status);
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct gb_r3d {
    gb_r3d_params p;
    R3Dev dev;
    double *fields = nullptr, *pool = nullptr, *work = nullptr, *tables = nullptr;
    int *itab = nullptr;
    void *small = nullptr;
    double *hist_nu = nullptr;
    int *hist_sw = nullptr;
    int hist_cap = 0;
    unsigned *sync = nullptr;
    int grid = 0;
    cudaStream_t stream = nullptr, side = nullptr;   // side: the v solve, beside the w solve
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

static int r3_levels(int nr, int nz)
{
    int nlev = 0, itest = nr, itest2 = nr, jtest = nz, jtest2 = nz;
    for (int i = 2; i <= 8; ++i) {
        itest /= 2;
        jtest /= 2;
        if (itest * 2 - itest2 == 0 && jtest * 2 - jtest2 == 0) {
            if (itest2 >= 4 && jtest2 >= 4) nlev++;
            itest2 = itest;
            jtest2 = jtest;
        } else {
            break;
        }
    }
    if (nlev > 4) nlev = 4;
    return nlev < 1 ? 1 : nlev;
}

extern "C" void gb_r3d_default_params(gb_r3d_params *p, int nr, int nz, int np)
{
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->nr = nr;
    p->nz = nz;
    p->np = np;
    p->dt = 1e-5;
    p->r0 = 0.5;
    p->rmax = 1.0;
    p->zmax = 0.5;
    p->Ra = 1e6;
    p->Re = 500.0;
    p->Gr = 0.0;
    p->Pr = 7.0;
    p->tolcon = 1e-5;
    p->sor = 1.2;
    p->maxsweeps = 500;
    p->nrel = 2;
    p->smoother = GB_SMOOTHER_LEX;
    p->precision = GB_PRB_FP64;
}

extern "C" int gb_r3d_destroy(gb_r3d *h)
{
    if (!h) return GB_OK;
    cudaFree(h->fields);
    cudaFree(h->pool);
    cudaFree(h->work);
    cudaFree(h->tables);
    cudaFree(h->itab);
    cudaFree(h->small);
    cudaFree(h->hist_nu);
    cudaFree(h->hist_sw);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    delete h;
    return GB_OK;
}

// Phase lists of one (level, component, direction), as packed (p, q);
// R3_CONT marks an entry whose line must be solved in the same chunk as the
// next entry's.
//
// LEX: the anti-diagonals p + q, in the reference's order.
//
// ZEBRA: lines with even p + q, then odd.  A line on a one-sided row (p = 1
// or P where p is one-sided, likewise q) also reads the line two over, of
// its own colour; within a colour such lines are solved before the lines
// they read (corners, then the other one-sided lines, then the rest), so
// every read two lines over sees the value from before the colour's pass.
// On the device a colour is one phase: a line and the lines that read it
// two over form a group of consecutive entries that one block solves in
// one chunk, whose right-hand sides are all formed before any of its
// eliminations writes.  A group larger than a chunk (only on grids far from
// the sizes the solver is built for) makes the classes separate phases in
// the same order.
#define R3_CONT 0x80000000u

static int r3_chunk_lines(int n) { return std::max(1, std::min(R3_THREADS, R3_SMEM_DOUBLES / (n | 1))); }

static void r3_phases(int mode, int comp, int dir, int n1, int n2, int n3, std::vector<int> &lines, std::vector<int> &off)
{
    const int im = r3_imax(comp, n1), jm = r3_jmax(comp, n2);
    int P, Q, p_os, q_os;
    if (dir == 0) {
        P = jm;
        Q = n3;
        p_os = comp != 1;
        q_os = 0;
    } else if (dir == 1) {
        P = im;
        Q = n3;
        p_os = comp != 3;
        q_os = 0;
    } else {
        P = im;
        Q = jm;
        p_os = comp != 3;
        q_os = comp != 1;
    }
    off.clear();
    lines.clear();
    off.push_back(0);
    if (mode == GB_SMOOTHER_LEX) {
        for (int dsum = 2; dsum <= P + Q; ++dsum) {
            for (int p = std::max(1, dsum - Q); p <= std::min(P, dsum - 1); ++p) lines.push_back(p | ((dsum - p) << 16));
            off.push_back((int)lines.size());
        }
        return;
    }
    const int chunk = r3_chunk_lines(r3_len(comp, dir, n1, n2, n3));
    auto cls_of = [&](int p, int q) { return (p_os && (p == 1 || p == P)) + (q_os && (q == 1 || q == Q)); };
    auto id = [&](int p, int q) { return (q - 1) * P + (p - 1); };
    for (int colour = 0; colour < 2; ++colour) {
        // groups: union of each one-sided line with the line it reads two over
        std::vector<int> parent((size_t)P * Q);
        for (size_t t = 0; t < parent.size(); ++t) parent[t] = (int)t;
        std::function<int(int)> root = [&](int x) { return parent[x] == x ? x : (parent[x] = root(parent[x])); };
        auto join = [&](int a, int b) { parent[root(a)] = root(b); };
        for (int q = 1; q <= Q; ++q)
            for (int p = 1; p <= P; ++p) {
                if (((p + q) & 1) != colour) continue;
                if (p_os && p == 1 && P >= 3) join(id(p, q), id(3, q));
                if (p_os && p == P && P >= 3) join(id(p, q), id(P - 2, q));
                if (q_os && q == 1 && Q >= 3) join(id(p, q), id(p, 3));
                if (q_os && q == Q && Q >= 3) join(id(p, q), id(p, Q - 2));
            }
        // members of each group, the group ordered by class (highest first)
        std::vector<std::vector<int>> groups((size_t)P * Q);
        for (int cls = 2; cls >= 0; --cls)
            for (int q = 1; q <= Q; ++q)
                for (int p = 1; p <= P; ++p)
                    if (((p + q) & 1) == colour && cls_of(p, q) == cls) groups[root(id(p, q))].push_back(p | (q << 16));
        size_t biggest = 0;
        for (const auto &g : groups) biggest = std::max(biggest, g.size());
        if ((int)biggest <= chunk) {
            const size_t before = lines.size();
            for (int multi = 1; multi >= 0; --multi)   // groups of several lines first, then single lines
                for (const auto &g : groups) {
                    if (g.empty() || (g.size() > 1) != (multi == 1)) continue;
                    for (size_t t = 0; t < g.size(); ++t)
                        lines.push_back((int)((unsigned)g[t] | (t + 1 < g.size() ? R3_CONT : 0u)));
                }
            if (lines.size() != before) off.push_back((int)lines.size());
        } else {
            for (int cls = 2; cls >= 0; --cls) {
                const size_t before = lines.size();
                for (int q = 1; q <= Q; ++q)
                    for (int p = 1; p <= P; ++p)
                        if (((p + q) & 1) == colour && cls_of(p, q) == cls) lines.push_back(p | (q << 16));
                if (lines.size() != before) off.push_back((int)lines.size());
            }
        }
    }
}

static int r3_create(const gb_r3d_params *p, const double *spacing, gb_r3d **out, int *nlev_out);

extern "C" int gb_r3d_create(const gb_r3d_params *p, gb_r3d **out, int *nlev_out)
{
    return r3_create(p, nullptr, out, nlev_out);
}

extern "C" int gb_r3d_create_spacing(const gb_r3d_params *p, double dr, double dz, double dp, gb_r3d **out,
                                     int *nlev_out)
{
    if (!(dr > 0.0 && dz > 0.0 && dp > 0.0)) {
        gb_set_error("gb_r3d_create_spacing: spacings must be positive");
        return GB_ERR_INVALID;
    }
    const double sp[3] = {dr, dz, dp};
    return r3_create(p, sp, out, nlev_out);
}

static int r3_create(const gb_r3d_params *p, const double *spacing, gb_r3d **out, int *nlev_out)
{
    if (!p || !out) { gb_set_error("gb_r3d_create: null argument"); return GB_ERR_INVALID; }
    *out = nullptr;
    const int nr = p->nr, nz = p->nz, np = p->np;
    const int nlev = r3_levels(nr, nz);
    if (nlev_out) *nlev_out = nlev;
    if (nr < 4 || nz < 4 || np < 4 || nr > 4096 || nz > 4096 || np > 16384 || np % (1 << nlev) != 0 ||
        np / (1 << (nlev - 1)) < 4 || !(p->r0 > 0.0 && p->rmax > p->r0) || !(p->zmax > 0.0) || !(p->dt > 0.0) ||
        p->Pr == 0.0 || (p->Re == 0.0 && p->variant != GB_R3D_HORIZONTAL) || p->nrel < 1 || p->maxsweeps < 1) {
        gb_set_error("gb_r3d_create: unsupported parameters (nr=%d nz=%d np=%d: nr, nz >= 4, np a multiple of 2^%d "
                     "with >= 4 phi intervals on the coarsest level; 0 < r0 < rmax, zmax, dt > 0, Pr != 0, Re != 0 "
                     "unless horizontal)",
                     nr, nz, np, nlev);
        return GB_ERR_INVALID;
    }
    if (p->smoother != GB_SMOOTHER_LEX && p->smoother != GB_SMOOTHER_ZEBRA) {
        gb_set_error("gb_r3d_create: unknown smoother %d", p->smoother);
        return GB_ERR_INVALID;
    }
    if (p->precision != GB_PRB_FP64 && p->precision != GB_PRB_MIXED) {
        gb_set_error("gb_r3d_create: unknown precision %d", p->precision);
        return GB_ERR_INVALID;
    }
    if (p->variant != GB_R3D_VERTICAL && p->variant != GB_R3D_HORIZONTAL) {
        gb_set_error("gb_r3d_create: unknown variant %d", p->variant);
        return GB_ERR_INVALID;
    }
    if (p->variant == GB_R3D_HORIZONTAL && nz < 6) {
        gb_set_error("gb_r3d_create: the horizontal annulus's heat band j = nz/2-3..nz/2+3 needs nz >= 6 (nz=%d)", nz);
        return GB_ERR_INVALID;
    }
    gb_r3d *h = new gb_r3d();
    h->p = *p;
    R3Dev &d = h->dev;
    memset(&d, 0, sizeof(d));
    d.nr = nr;
    d.nz = nz;
    d.np = np;
    d.ni = nr + 2;
    d.nj = nz + 2;
    d.nk = np + 1;
    d.nlev = nlev;
    d.dt = p->dt;
    d.r0 = p->r0;
    d.rmax = p->rmax;
    d.zmax = p->zmax;
    d.Ra = p->Ra;
    d.Re = p->Re;
    d.Gr = p->Gr;
    d.Ptl = p->Pr;
    const double pi = acos(-1.0);
    d.dr = spacing ? spacing[0] : (p->rmax - p->r0) / (double)nr;
    d.dz = spacing ? spacing[1] : p->zmax / (double)nz;
    d.dp = spacing ? spacing[2] : 2.0 * pi / (double)np;
    d.nu_num = -p->r0 * log(p->r0 / p->rmax);
    d.nu_den = p->zmax * 2.0 * pi;
    d.horizontal = p->variant == GB_R3D_HORIZONTAL;
    if (d.horizontal) {
        // httrans1, httrans2 of rot3dmghor.f:264-267, host libm as the Fortran runtime
        d.nu_num = (double)nz / 6.0 * p->r0 * log(p->r0 / p->rmax);
        d.nu2_num = (double)nz / 6.0 * p->rmax * log(p->r0 / p->rmax);
    }
    d.tolcon = p->tolcon;
    d.sor = p->sor;
    d.nrel = p->nrel;
    d.maxsweeps = p->maxsweeps;
    const size_t fsz = (size_t)d.ni * d.nj * d.nk;
    cudaError_t e = cudaMalloc(&h->fields, sizeof(double) * fsz * GB_R_COUNT);
    if (e != cudaSuccess) { gb_set_error("gb_r3d_create: fields: %s", cudaGetErrorString(e)); delete h; return GB_ERR_ALLOC; }
    cudaMemset(h->fields, 0, sizeof(double) * fsz * GB_R_COUNT);
    for (int q = 0; q < GB_R_COUNT; ++q) d.fld[q] = h->fields + (size_t)q * fsz;

    // multigrid pool: per level rvc, rvv and the factor tables (shared by the
    // components); the work pool: per component and level v, f, res and their
    // FP32 twins
    std::vector<FacJob> jobs;
    size_t need = 0, wneed = 0;
    for (int l = 1; l <= nlev; ++l) {
        const int n1 = nr >> (l - 1), n2 = nz >> (l - 1), n3 = np >> (l - 1);
        const size_t sz = (size_t)(n1 + 1) * (n2 + 1) * (n3 + 1);
        wneed += 3 * (3 * sz + (3 * sz + 1) / 2 + 2);
        need += 2 * (size_t)(n1 + 2);
        size_t f32 = 4 * (size_t)(n1 + 2);
        for (int comp = 1; comp <= 3; ++comp)
            for (int dir = 0; dir < 3; ++dir) {
                const int n = r3_len(comp, dir, n1, n2, n3);
                const int inst = dir == 0 ? 1 : r3_imax(comp, n1);
                need += (size_t)inst * r3_tabsize(r3_kind(comp, dir), n);
                f32 += (size_t)inst * r3_tabsize(r3_kind(comp, dir), n);
            }
        need += (f32 + 1) / 2 + 2;
    }
    e = cudaMalloc(&h->pool, sizeof(double) * need);
    if (e != cudaSuccess) { gb_r3d_destroy(h); gb_set_error("gb_r3d_create: multigrid pool"); return GB_ERR_ALLOC; }
    cudaMemset(h->pool, 0, sizeof(double) * need);
    e = cudaMalloc(&h->work, sizeof(double) * wneed);
    if (e != cudaSuccess) { gb_r3d_destroy(h); gb_set_error("gb_r3d_create: multigrid work arrays"); return GB_ERR_ALLOC; }
    cudaMemset(h->work, 0, sizeof(double) * wneed);
    double *b = h->pool, *wb = h->work;
    std::vector<int> itab;
    struct TabRef { int l, comp, dir; size_t lines, off; int nphase; };
    std::vector<TabRef> refs;
    std::vector<double> rv_host;
    for (int l = 1; l <= nlev; ++l) {
        R3Lev &L = d.lev[l];
        L.n1 = nr >> (l - 1);
        L.n2 = nz >> (l - 1);
        L.n3 = np >> (l - 1);
        L.L1 = L.n1 + 1;
        L.L2 = L.n2 + 1;
        const int p2 = 1 << l;
        L.hr = d.dr * (double)p2 * 0.5;
        L.hz = d.dz * (double)p2 * 0.5;
        L.hp = d.dp * (double)p2 * 0.5;
        L.hhr = L.hr * L.hr;
        L.hhz = L.hz * L.hz;
        L.hhp = L.hp * L.hp;
        const size_t sz = (size_t)L.L1 * L.L2 * (L.n3 + 1);
        for (int comp = 1; comp <= 3; ++comp) {
            R3Work &W = d.work[comp][l];
            W.v = wb; wb += sz;
            W.f = wb; wb += sz;
            W.res = wb; wb += sz;
            float *fw = (float *)wb;
            W.v32 = fw; fw += sz;
            W.f32 = fw; fw += sz;
            W.res32 = fw; fw += sz;
            wb = (double *)(((uintptr_t)fw + 15) & ~(uintptr_t)15);
        }
        L.rvc = b; b += L.n1 + 2;
        L.rvv = b; b += L.n1 + 2;
        rv_host.assign(2 * (size_t)(L.n1 + 2), 0.0);
        for (int i = 0; i <= L.n1 + 1; ++i) {
            rv_host[i] = d.r0 + ((double)i - 0.5) * L.hr;
            rv_host[L.n1 + 2 + i] = (double)i * L.hr + d.r0;
        }
        cudaMemcpy(L.rvc, rv_host.data(), sizeof(double) * rv_host.size(), cudaMemcpyHostToDevice);
        for (int comp = 1; comp <= 3; ++comp)
            for (int dir = 0; dir < 3; ++dir) {
                const int kind = r3_kind(comp, dir);
                const int n = r3_len(comp, dir, L.n1, L.n2, L.n3);
                const int inst = dir == 0 ? 1 : r3_imax(comp, L.n1);
                L.fac[comp][dir] = b;
                for (int q = 0; q < inst; ++q) jobs.push_back({l, comp, dir, dir == 0 ? 0 : q + 1, b + (size_t)q * r3_tabsize(kind, n)});
                b += (size_t)inst * r3_tabsize(kind, n);
                std::vector<int> lines, off;
                r3_phases(p->smoother, comp, dir, L.n1, L.n2, L.n3, lines, off);
                TabRef tr;
                tr.l = l;
                tr.comp = comp;
                tr.dir = dir;
                tr.lines = itab.size();
                itab.insert(itab.end(), lines.begin(), lines.end());
                tr.off = itab.size();
                itab.insert(itab.end(), off.begin(), off.end());
                tr.nphase = (int)off.size() - 1;
                refs.push_back(tr);
            }
        // FP32 storage of the level
        {
            float *fb = (float *)b;
            L.irc = fb; fb += L.n1 + 2;
            L.irv = fb; fb += L.n1 + 2;
            L.iqc = fb; fb += L.n1 + 2;
            L.iqv = fb; fb += L.n1 + 2;
            std::vector<float> rr(4 * (size_t)(L.n1 + 2));
            for (int i = 0; i <= L.n1 + 1; ++i) {
                const double rc = rv_host[i], rv = rv_host[L.n1 + 2 + i];
                rr[i] = (float)(1.0 / rc);
                rr[L.n1 + 2 + i] = (float)(1.0 / rv);
                rr[2 * (L.n1 + 2) + i] = (float)(1.0 / (rc * rc));
                rr[3 * (L.n1 + 2) + i] = (float)(1.0 / (rv * rv));
            }
            cudaMemcpy(L.irc, rr.data(), sizeof(float) * rr.size(), cudaMemcpyHostToDevice);
            L.ihr = (float)(1.0 / L.hr);
            L.ihhr = (float)(1.0 / L.hhr);
            L.ihhz = (float)(1.0 / L.hhz);
            L.ihhp = (float)(1.0 / L.hhp);
            for (int comp = 1; comp <= 3; ++comp)
                for (int dir = 0; dir < 3; ++dir) {
                    const int n = r3_len(comp, dir, L.n1, L.n2, L.n3);
                    const int inst = dir == 0 ? 1 : r3_imax(comp, L.n1);
                    L.fac32[comp][dir] = fb;
                    fb += (size_t)inst * r3_tabsize(r3_kind(comp, dir), n);
                }
            b = (double *)(((uintptr_t)fb + 15) & ~(uintptr_t)15);
        }
    }
    if ((size_t)(b - h->pool) > need || (size_t)(wb - h->work) > wneed) {
        gb_r3d_destroy(h);
        gb_set_error("gb_r3d_create: multigrid pool layout mismatch");
        return GB_ERR_CUDA;
    }
    e = cudaMalloc(&h->itab, sizeof(int) * itab.size());
    if (e != cudaSuccess) { gb_r3d_destroy(h); gb_set_error("gb_r3d_create: phase tables"); return GB_ERR_ALLOC; }
    cudaMemcpy(h->itab, itab.data(), sizeof(int) * itab.size(), cudaMemcpyHostToDevice);
    for (const TabRef &tr : refs) {
        R3Lev &L = d.lev[tr.l];
        L.lines[tr.comp][tr.dir] = h->itab + tr.lines;
        L.poff[tr.comp][tr.dir] = h->itab + tr.off;
        L.nphase[tr.comp][tr.dir] = tr.nphase;
    }
    // sin and cos of theta = 6.283185307/np k (rot3dmghor.f:373-378), host libm
    {
        std::vector<double> tab(2 * (size_t)(np + 1), 0.0);
        if (d.horizontal)
            for (int k = 0; k <= np; ++k) {
                const double theta = 6.283185307 / (double)np * (double)k;
                tab[k] = sin(theta);
                tab[np + 1 + k] = cos(theta);
            }
        e = cudaMalloc(&h->tables, sizeof(double) * tab.size());
        if (e != cudaSuccess) { gb_r3d_destroy(h); gb_set_error("gb_r3d_create: tables"); return GB_ERR_ALLOC; }
        cudaMemcpy(h->tables, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice);
        d.sinth = h->tables;
        d.costh = h->tables + np + 1;
    }
    // small state
    e = cudaMalloc(&h->small, 4096 + 2 * sizeof(double) * (size_t)(np + 2));
    if (e != cudaSuccess) { gb_r3d_destroy(h); gb_set_error("gb_r3d_create: state"); return GB_ERR_ALLOC; }
    cudaMemset(h->small, 0, 4096 + 2 * sizeof(double) * (size_t)(np + 2));
    char *sm = (char *)h->small;
    d.resmax = (unsigned long long *)(sm + 0);    // 8 slots
    d.nanflag = (int *)(sm + 64);                 // 8 slots
    d.abort = (int *)(sm + 128);
    d.steps_done = (int *)(sm + 192);
    d.solve_status = (int *)(sm + 256);           // 4 slots
    d.solve_sweeps = (int *)(sm + 320);           // 4 slots
    h->sync = (unsigned *)(sm + 512);             // 4 barriers, 128 bytes apart
    d.trans = (double *)(sm + 4096);
    d.trans2 = d.trans + (np + 2);
    for (int c = 0; c < 4; ++c) {
        d.gs[c].count = h->sync + R3_SYNC_STRIDE * c;
        d.gs[c].gen = h->sync + R3_SYNC_STRIDE * c + 1;
        d.gs[c].err = (int *)(h->sync + R3_SYNC_STRIDE * c + 2);
        d.gs[c].limit = GB_GRID_WAIT_LIMIT_DEFAULT;
        d.gs[c].tally = (unsigned long long *)(sm + 448) + c;   // 4 counters, one per component
    }
    // factor tables
    FacJob *djobs = nullptr;
    e = cudaMalloc(&djobs, sizeof(FacJob) * jobs.size());
    if (e != cudaSuccess) { gb_r3d_destroy(h); gb_set_error("gb_r3d_create: factor jobs"); return GB_ERR_ALLOC; }
    cudaMemcpy(djobs, jobs.data(), sizeof(FacJob) * jobs.size(), cudaMemcpyHostToDevice);
    k_r3d_factors<<<gb_ceil_div(jobs.size(), 64), 64>>>(d, djobs, (int)jobs.size());
    {
        // FP32 tables: the same job list, destinations in the FP32 pool
        std::vector<float *> dst(jobs.size());
        for (size_t q = 0; q < jobs.size(); ++q) {
            const FacJob &J = jobs[q];
            const R3Lev &L = d.lev[J.lev];
            dst[q] = L.fac32[J.comp][J.dir] + (J.tab - L.fac[J.comp][J.dir]);
        }
        float **ddst = nullptr;
        e = cudaMalloc(&ddst, sizeof(float *) * dst.size());
        if (e == cudaSuccess) {
            cudaMemcpy(ddst, dst.data(), sizeof(float *) * dst.size(), cudaMemcpyHostToDevice);
            k_r3d_factors32<<<gb_ceil_div(jobs.size(), 64), 64>>>(d, djobs, (int)jobs.size(), ddst);
            cudaDeviceSynchronize();
            cudaFree(ddst);
        }
    }
    e = cudaDeviceSynchronize();
    cudaFree(djobs);
    if (e != cudaSuccess) { gb_set_error("gb_r3d_create: factors: %s", cudaGetErrorString(e)); gb_r3d_destroy(h); return GB_ERR_CUDA; }
    // cooperative grid: every block resident
    int dev = 0, sms = 0, coop = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    int worst = 1 << 30;
    const void *kerns[6] = {(const void *)k_r3d_solve<1>, (const void *)k_r3d_solve<2>, (const void *)k_r3d_solve<3>,
                            (const void *)k_r3d_solve_mixed<1>, (const void *)k_r3d_solve_mixed<2>,
                            (const void *)k_r3d_solve_mixed<3>};
    for (int q = 0; q < 6; ++q) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kerns[q], R3_THREADS, 0);
        worst = std::min(worst, per_sm);
    }
    if (!coop || worst < 1) {
        gb_r3d_destroy(h);
        gb_set_error("gb_r3d_create: cooperative launch unavailable (coop=%d, blocks/SM=%d)", coop, worst);
        return GB_ERR_CUDA;
    }
    h->grid = sms * std::min(worst, 2);
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) { gb_r3d_destroy(h); gb_set_error("gb_r3d_create: streams"); return GB_ERR_CUDA; }
    *out = h;
    return GB_OK;
}

extern "C" void *gb_r3d_stream(gb_r3d *h) { return h ? (void *)h->stream : nullptr; }

extern "C" int gb_r3d_barrier_counts(gb_r3d *h, unsigned long long *counts, int *blocks, int reset)
{
    if (!h) { gb_set_error("gb_r3d_barrier_counts: null context"); return GB_ERR_INVALID; }
    GB_CUDA_TRY(cudaStreamSynchronize(h->side));
    GB_CUDA_TRY(cudaStreamSynchronize(h->stream));
    unsigned long long c[4] = {0, 0, 0, 0};
    GB_CUDA_TRY(cudaMemcpy(c, h->dev.gs[0].tally, sizeof(c), cudaMemcpyDeviceToHost));
    if (counts)
        for (int i = 0; i < 3; ++i) counts[i] = c[i + 1];
    if (blocks) *blocks = h->grid;
    if (reset) GB_CUDA_TRY(cudaMemset(h->dev.gs[0].tally, 0, sizeof(c)));
    return GB_OK;
}

extern "C" int gb_r3d_set_wait_limit(gb_r3d *h, long long polls)
{
    if (!h || polls < 0) {
        gb_set_error("gb_r3d_set_wait_limit: need a context and polls >= 0");
        return GB_ERR_INVALID;
    }
    for (int c = 0; c < 4; ++c) h->dev.gs[c].limit = polls;
    return GB_OK;
}

static int r3_io(gb_r3d *h, int field, double *host, int ld1, int ld2, bool to_dev)
{
    if (!h || !host || field < 0 || field >= GB_R_COUNT || ld1 < h->dev.ni || ld2 < h->dev.nj) {
        gb_set_error("gb_r3d_%s_field: invalid argument", to_dev ? "set" : "get");
        return GB_ERR_INVALID;
    }
    const R3Dev &d = h->dev;
    cudaMemcpy3DParms m;
    memset(&m, 0, sizeof(m));
    cudaPitchedPtr hp = make_cudaPitchedPtr(host, sizeof(double) * (size_t)ld1, (size_t)d.ni, (size_t)ld2);
    cudaPitchedPtr dp = make_cudaPitchedPtr(d.fld[field], sizeof(double) * (size_t)d.ni, (size_t)d.ni, (size_t)d.nj);
    m.srcPtr = to_dev ? hp : dp;
    m.dstPtr = to_dev ? dp : hp;
    m.extent = make_cudaExtent(sizeof(double) * (size_t)d.ni, (size_t)d.nj, (size_t)d.nk);
    m.kind = to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    GB_CUDA_TRY(cudaMemcpy3DAsync(&m, h->stream));
    GB_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return GB_OK;
}

extern "C" int gb_r3d_set_field(gb_r3d *h, int field, const double *host, int ld1, int ld2)
{
    return r3_io(h, field, (double *)host, ld1, ld2, true);
}

extern "C" int gb_r3d_get_field(gb_r3d *h, int field, double *host, int ld1, int ld2)
{
    return r3_io(h, field, host, ld1, ld2, false);
}

static const int R3_TPB = 256;

static void r3_launch_transport(gb_r3d *h, int what, int step, cudaStream_t s)
{
    const R3Dev &d = h->dev;
    const long long nr = d.nr, nz = d.nz, npp = d.np + 1;
    switch (what) {
    case 0: k_r3d_avort<<<gb_ceil_div(nr * (nz - 1) * npp, R3_TPB), R3_TPB, 0, s>>>(d); break;
    case 1: k_r3d_bvort<<<gb_ceil_div((nr - 1) * (nz - 1) * npp, R3_TPB), R3_TPB, 0, s>>>(d); break;
    case 2: k_r3d_cvort<<<gb_ceil_div((nr - 1) * nz * npp, R3_TPB), R3_TPB, 0, s>>>(d); break;
    case 3: k_r3d_temp<<<gb_ceil_div(nr * (nz + 2) * npp, R3_TPB), R3_TPB, 0, s>>>(d); break;
    case 4:
        k_r3d_heat_k<<<gb_ceil_div(d.np, 128), 128, 0, s>>>(d);
        k_r3d_heat_sum<<<1, 32, 0, s>>>(d, step);
        break;
    case 5: k_r3d_rhs<1><<<gb_ceil_div(nr * (nz - 1) * npp, R3_TPB), R3_TPB, 0, s>>>(d); break;
    case 6: k_r3d_rhs<2><<<gb_ceil_div(nr * nz * npp, R3_TPB), R3_TPB, 0, s>>>(d); break;
    case 7: k_r3d_rhs<3><<<gb_ceil_div((nr - 1) * nz * npp, R3_TPB), R3_TPB, 0, s>>>(d); break;
    case 8: k_r3d_update<<<gb_ceil_div((long long)d.ni * d.nj * d.nk, R3_TPB), R3_TPB, 0, s>>>(d, step); break;
    }
}

// One component's solve on `grid` blocks (at most h->grid, all resident).
// The w and v solves of a step run side by side on half the blocks each:
// their blocks together never exceed the resident capacity, and each waits
// only at its own barrier.
static int r3_launch_solve(gb_r3d *h, int comp, int step, cudaStream_t s, int grid)
{
    GB_CUDA_TRY(cudaMemsetAsync(h->sync + R3_SYNC_STRIDE * comp, 0, sizeof(unsigned) * 4, s));
    GB_CUDA_TRY(cudaMemsetAsync(h->dev.resmax + 2 * comp, 0, sizeof(unsigned long long) * 2, s));
    GB_CUDA_TRY(cudaMemsetAsync(h->dev.nanflag + 2 * comp, 0, sizeof(int) * 2, s));
    R3Dev D = h->dev;
    void *args[] = {&D, &step};
    const bool mixed = h->p.precision == GB_PRB_MIXED;
    const void *k = comp == 1   ? (mixed ? (const void *)k_r3d_solve_mixed<1> : (const void *)k_r3d_solve<1>)
                    : comp == 2 ? (mixed ? (const void *)k_r3d_solve_mixed<2> : (const void *)k_r3d_solve<2>)
                                : (mixed ? (const void *)k_r3d_solve_mixed<3> : (const void *)k_r3d_solve<3>);
    cudaError_t e = cudaLaunchCooperativeKernel(k, grid, R3_THREADS, args, 0, s);
    if (e != cudaSuccess) {
        gb_set_error("gb_r3d: cooperative solve launch (%d blocks): %s", grid, cudaGetErrorString(e));
        return GB_ERR_CUDA;
    }
    return GB_OK;
}

static int r3_sync(gb_r3d *h, const char *what)
{
    cudaError_t e = cudaStreamSynchronize(h->side);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) { gb_set_error("%s: %s", what, cudaGetErrorString(e)); return GB_ERR_CUDA; }
    unsigned sy[4 * R3_SYNC_STRIDE];
    GB_CUDA_TRY(cudaMemcpy(sy, h->sync, sizeof(sy), cudaMemcpyDeviceToHost));
    for (int c = 1; c <= 3; ++c)
        if (sy[R3_SYNC_STRIDE * c + 2]) {
            gb_set_error("%s: a grid barrier wait timed out (component %d)", what, c);
            return GB_TIMEOUT;
        }
    return GB_OK;
}

static void r3_clear_abort(gb_r3d *h) { cudaMemsetAsync(h->dev.abort, 0, sizeof(int), h->stream); }

#define R3_ROUTINE(name, what)                                  \
    extern "C" int gb_r3d_##name(gb_r3d *h)                     \
    {                                                           \
        if (!h) return GB_ERR_INVALID;                          \
        r3_clear_abort(h);                                      \
        r3_launch_transport(h, what, -1, h->stream);            \
        return r3_sync(h, "gb_r3d_" #name);                     \
    }
R3_ROUTINE(avorticity, 0)
R3_ROUTINE(bvorticity, 1)
R3_ROUTINE(cvorticity, 2)
R3_ROUTINE(temperature, 3)
R3_ROUTINE(rhsw, 5)
R3_ROUTINE(rhsv, 6)
R3_ROUTINE(rhsu, 7)
R3_ROUTINE(update, 8)
#undef R3_ROUTINE

extern "C" int gb_r3d_heat(gb_r3d *h, double *trans1)
{
    if (!h) return GB_ERR_INVALID;
    r3_clear_abort(h);
    r3_launch_transport(h, 4, -1, h->stream);
    int st = r3_sync(h, "gb_r3d_heat");
    if (st != GB_OK) return st;
    if (trans1) GB_CUDA_TRY(cudaMemcpy(trans1, h->dev.trans, sizeof(double), cudaMemcpyDeviceToHost));
    return GB_OK;
}

extern "C" int gb_r3d_heat2(gb_r3d *h, double *trans1, double *trans2)
{
    if (!h) return GB_ERR_INVALID;
    r3_clear_abort(h);
    r3_launch_transport(h, 4, -1, h->stream);
    int st = r3_sync(h, "gb_r3d_heat2");
    if (st != GB_OK) return st;
    if (trans1) GB_CUDA_TRY(cudaMemcpy(trans1, h->dev.trans, sizeof(double), cudaMemcpyDeviceToHost));
    if (trans2) GB_CUDA_TRY(cudaMemcpy(trans2, h->dev.trans2, sizeof(double), cudaMemcpyDeviceToHost));
    return GB_OK;
}

extern "C" int gb_r3d_nu2(gb_r3d *h, int nsteps, double *nu2)
{
    if (!h || nsteps < 0 || nsteps > h->hist_cap || (nsteps > 0 && !nu2)) {
        gb_set_error("gb_r3d_nu2: invalid argument");
        return GB_ERR_INVALID;
    }
    if (nsteps > 0)
        GB_CUDA_TRY(cudaMemcpy(nu2, h->hist_nu + h->hist_cap, sizeof(double) * (size_t)nsteps, cudaMemcpyDeviceToHost));
    return GB_OK;
}

extern "C" int gb_r3d_poisson(gb_r3d *h, int which, int *sweeps)
{
    if (!h || which < 1 || which > 3) { gb_set_error("gb_r3d_poisson: invalid argument"); return GB_ERR_INVALID; }
    r3_clear_abort(h);
    int st = r3_launch_solve(h, which, -1, h->stream, h->grid);
    if (st != GB_OK) return st;
    st = r3_sync(h, "gb_r3d_poisson");
    if (st != GB_OK) return st;
    int out[2] = {0, 0};
    GB_CUDA_TRY(cudaMemcpy(&out[0], h->dev.solve_status + which, sizeof(int), cudaMemcpyDeviceToHost));
    GB_CUDA_TRY(cudaMemcpy(&out[1], h->dev.solve_sweeps + which, sizeof(int), cudaMemcpyDeviceToHost));
    if (sweeps) *sweeps = out[1];
    return out[0];
}

extern "C" int gb_r3d_step(gb_r3d *h, int nsteps, double *nu, int *sweeps, int *steps_done)
{
    if (!h || nsteps < 0) { gb_set_error("gb_r3d_step: invalid argument"); return GB_ERR_INVALID; }
    if (steps_done) *steps_done = 0;
    if (nsteps == 0) return GB_OK;
    if (nsteps > h->hist_cap) {
        cudaFree(h->hist_nu);
        cudaFree(h->hist_sw);
        h->hist_nu = nullptr;
        h->hist_sw = nullptr;
        h->hist_cap = 0;
        GB_CUDA_TRY(cudaMalloc(&h->hist_nu, 2 * sizeof(double) * (size_t)nsteps));
        GB_CUDA_TRY(cudaMalloc(&h->hist_sw, sizeof(int) * 3 * (size_t)nsteps));
        h->hist_cap = nsteps;
    }
    h->dev.hist_nu = h->hist_nu;
    h->dev.hist_nu2 = h->hist_nu + h->hist_cap;
    h->dev.hist_sw = h->hist_sw;
    cudaStream_t s = h->stream;
    GB_CUDA_TRY(cudaMemsetAsync(h->hist_sw, 0, sizeof(int) * 3 * (size_t)nsteps, s));
    GB_CUDA_TRY(cudaMemsetAsync(h->hist_nu, 0, 2 * sizeof(double) * (size_t)h->hist_cap, s));
    GB_CUDA_TRY(cudaMemsetAsync(h->dev.steps_done, 0, sizeof(int), s));
    GB_CUDA_TRY(cudaMemsetAsync(h->dev.abort, 0, sizeof(int), s));
    for (int step = 0; step < nsteps; ++step) {
        r3_launch_transport(h, 0, step, s);
        r3_launch_transport(h, 1, step, s);
        r3_launch_transport(h, 2, step, s);
        r3_launch_transport(h, 3, step, s);
        r3_launch_transport(h, 4, step, s);
        r3_launch_transport(h, 5, step, s);
        // rhsv reads An and Cn only, and the w and v solves touch disjoint
        // fields: the v solve runs beside the w solve, on the side stream
        GB_CUDA_TRY(cudaEventRecord(h->ev_fork, s));
        GB_CUDA_TRY(cudaStreamWaitEvent(h->side, h->ev_fork, 0));
        const int half = std::max(1, h->grid / 2);
        int st = r3_launch_solve(h, 1, step, s, half);
        if (st == GB_OK) {
            r3_launch_transport(h, 6, step, h->side);
            st = r3_launch_solve(h, 2, step, h->side, h->grid - half);
        }
        if (st == GB_OK) {
            GB_CUDA_TRY(cudaEventRecord(h->ev_join, h->side));
            GB_CUDA_TRY(cudaStreamWaitEvent(s, h->ev_join, 0));
            r3_launch_transport(h, 7, step, s);
            st = r3_launch_solve(h, 3, step, s, h->grid);
        }
        if (st != GB_OK) return st;
        r3_launch_transport(h, 8, step, s);
    }
    int st = r3_sync(h, "gb_r3d_step");
    if (st != GB_OK) return st;
    int done = 0, ab = 0;
    GB_CUDA_TRY(cudaMemcpy(&done, h->dev.steps_done, sizeof(int), cudaMemcpyDeviceToHost));
    GB_CUDA_TRY(cudaMemcpy(&ab, h->dev.abort, sizeof(int), cudaMemcpyDeviceToHost));
    if (steps_done) *steps_done = done;
    if (nu && done > 0) GB_CUDA_TRY(cudaMemcpy(nu, h->hist_nu, sizeof(double) * (size_t)done, cudaMemcpyDeviceToHost));
    if (sweeps) {
        const int n = std::min(nsteps, done + 1);
        GB_CUDA_TRY(cudaMemcpy(sweeps, h->hist_sw, sizeof(int) * 3 * (size_t)n, cudaMemcpyDeviceToHost));
    }
    return ab ? ab : GB_OK;
}
