// Internal state of a device-resident 2D periodic Rayleigh-Benard instance.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "gbcommon.cuh"

#define PRB_MAXLEV 7

// One multigrid level of one equation (COMMON /step/, /ints/ of
// velvor2dperiodicrbconv.f:1810-1814, plus the packed v/f slots).
struct MgLevel {
    int n1, n3;
    double hr;           // radial spacing of the level
    double hhri, hhpi;   // 1/hr^2, 1/hp^2 of the level
    double hri;          // 1/hr
    const double *fac;   // factored line matrix (pdma for v, tdma for u)
    double *v, *f;       // packed (n1+1)*(n3+1) solution / right-hand side
    double *rvi, *rvq;   // annulus: 1/r and 1/r^2 of row i (n1+2 entries)
    // mixed precision: the FP32 correction cycle's storage
    float *v32, *f32;    // packed correction / right-hand side
    float *fac32;        // factors with the pivots stored as reciprocals
    float *rvi32, *rvq32;
};

// Device description of one Poisson solve (poisson2 or poisson3).
struct MgEq {
    int which;           // 2: v (cell centred, pentadiagonal), 3: u (face, tridiagonal)
    int nr, np, ld, nlev, mode, maxsweeps;
    int polar;           // the (r, phi) operator (annulus and Taylor-Couette)
    int nrelax;          // relaxations per relax call: 3 in the annulus, else 1
    int seam_keep;       // the annulus's corser keeps the coarse seam residual
    int xwall;           // the tank: side walls in x (velvor2dhorconvtank.f:1032-1303)
    int stop_on_max;     // the sweep limit fails the step (PRB's STOP) or only is reported
    int smem_fac;        // mixed solve: floats of shared memory before its line buffer (>= the level-1 factors)
    double r0;
    double tolcon, sor;
    MgLevel lev[PRB_MAXLEV];
    double *psic, *psif, *rc, *rf, *tempa;   // COMMON /arrays/ (per equation)
    float *psif32, *rc32;                    // mixed precision: FP32 correction and residual
    double *psi, *psip;                      // solution and previous level (in/out)
    const double *rhs;
    int *status;         // [0] status, [1] sweeps
    double *resmax;      // last level-1 residual max norm
    int *abort;          // set on failure: later kernels of a step skip their work
};

struct PrbDev {
    int nr, np, ld;
    int polar;           // GB_PRB_ANNULUS or GB_PRB_TAYCOU: the (r, phi) plane
    int oblique;         // GB_PRB_OBLIQUE
    int taycou;          // GB_PRB_TAYCOU: the moving outer wall
    int tank;            // GB_PRB_TANK or GB_PRB_DVD: side walls in x, np+2 columns per field
    int dvd;             // GB_PRB_DVD: the differentially heated cavity's differences
    const double *fac_xw1, *fac_xw2;   // the tank's tdma factors along x, n = np-1 and np
    double velo;         // its speed -(Ta**0.5) Ptl rmax / 2 (host libm pow)
    double rmax;
    double robert;       // Robert filter coefficient: 0.02 layer, 0.05 annulus, 0.01 Taylor-Couette
    double dt, Ra, Pr, dr, dp, dri, dpi;
    double r0, Re;
    double *f[GB_F_COUNT];
    const double *fac_r1, *fac_x, *fac_rT;
    double *heat;
    unsigned long long *clamps;
    int *abort, *step_index, *mg_status;
    double *mg_resmax;
    double *nu_hist;
    int *sweep_hist;
    int hist_cap;
    // time-loop diagnostics (PRB:404-459), null when off: running means of
    // T^2, T, u^2, v^2 (four arrays of diag_stride doubles, columns
    // k = 0..np of leading dimension ld used), the kt of the step in flight,
    // per-step CFL maxima (2 per history slot, bit patterns)
    double *diag;
    size_t diag_stride;
    int *diag_kt;
    unsigned long long *cfl_hist;
};

struct gb_prb {
    gb_prb_params p;
    int nlev;
    size_t fsz;
    double dr_set = 0.0, dp_set = 0.0;  // verbatim spacings of a Fortran caller, 0 = derived
    PrbDev dev;
    double *fields = nullptr;
    double *factors = nullptr;
    void *small = nullptr;
    void *hist = nullptr;
    int hist_cap = 0;
    // multigrid
    MgEq eq_host[2];          // [0] v (which 2), [1] u (which 3)
    MgEq *eq_dev = nullptr;   // device copy, 2 entries
    double *mg_pool = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph_exec = nullptr, graph_exec1 = nullptr;
    gb_prb_params graph_scalars;
    long long launches = 0, launches_per_step = 0;
    int ncol = 0;                 // columns per field: np+1, np+2 in the tank
    double *diag_buf = nullptr;   // 4 running means + kt + CFL history (hist_cap slots)
    int diag_cap = 0;
    int steps_done = 0;
    int mg_spread = 1;            // CTAs per zebra solve (gb_prb_set_solve_spread): 1 or 8
};

int prb_mg_levels(int nr, int variant);
int prb_mg_create(gb_prb *h);
void prb_mg_destroy(gb_prb *h);
int prb_launch_mg(gb_prb *h, int do_v, int do_u, cudaStream_t s);
void prb_mg_launch_eqs(const MgEq *d_eqs, int neq, int mixed, int spread, size_t smem, cudaStream_t s);
size_t prb_mg_smem(const gb_prb *h);
int prb_mg_cluster_ctas();
int prb_refresh_scalars(gb_prb *h);
// the tank's transport (tank.cu)
int tank_launch_cvorticity(gb_prb *h, int first, cudaStream_t s);
int tank_launch_temperature(gb_prb *h, int first, cudaStream_t s);
int tank_launch_rhs(gb_prb *h, int do_v, int do_u, cudaStream_t s);
int tank_launch_update(gb_prb *h, cudaStream_t s);
