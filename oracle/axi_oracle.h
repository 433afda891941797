/*
 * CPU oracle for the axisymmetric rotating-annulus step of rotann2.f ("AXI"):
 * vorticity, swirl velocity and temperature by Dufort-Frankel with the
 * Arakawa Jacobian, Thom wall vorticity, the wall heat flux, and the
 * streamfunction multigrid (alternating r-line / z-line Gauss-Seidel,
 * 9-point restriction, bilinear prolongation, plain V-cycle).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of tests/, smoke() and bench.py's
 * CPU legs; never linked into the product.  PARITY PINNED for the uniform
 * grid: it reproduces bit for bit rotann2.f run as its main program through
 * the translator tests/golden/f77.py (tests/test_reference_runs.py).  The
 * stretched mode composes rotann2.f's physics with grid.f's weights and
 * rcsc.f's multigrid, which are pinned separately; no reference program
 * runs that composition.
 * Double precision, the reference's left-to-right order, -ffp-contract=off.
 *
 * Arrays are the reference's (0:nr, 0:nz) arrays, column-major with leading
 * dimension ld = nr+1 (element (i,j) at i + ld*j).
 */
#ifndef AXI_ORACLE_H
#define AXI_ORACLE_H

#include "str_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

#define AXI_LEX   0   /* r-lines j = 1..n2-1, then z-lines i = 1..n1-1, in order (rotann2.f:698-725) */
#define AXI_ZEBRA 1   /* odd lines, then even lines, in each direction */

typedef struct {
    int nr, nz, ld;
    double dt, dr, dz, r0, rmax, zmax, Ra, Re, Ptl;
    double cf1, cf2, cf3, cf4;               /* COMMON /val/ (rotann2.f:66-69) */
    double *phi, *omegn, *omeg, *omegp, *veln, *vel, *velp;
    double *thetan, *theta, *thetap;
    /* multigrid (COMMON /backup/ /arrays/ /step/ /ints/) */
    int nlev, n1[8], n2[8];
    double hr[8], hz[8], hhr[8], hhz[8];
    double *rval;                            /* 0..nr */
    double *v[8], *f[8];
    double *psic, *psif, *rc, *rf, *tempa;
    double tolcon;                           /* 1e-6 (rotann2.f:689) */
    int nrel;                                /* 2 (rotann2.f:618-619) */
    int maxsweeps;                           /* nvs = 10000 (rotann2.f:617) */
    int mode;                                /* AXI_LEX or AXI_ZEBRA */
    int last_sweeps;
    double last_resmax;
    /* stretched grid (NULL: rotann2.f's uniform grid); see orc_axi_set_stretched */
    const orc_str_grid_t *sg;
    orc_str_mg_t *smg;
    double hw[5];                            /* stretched: inner-wall d/dr weights on r(0..4) */
} orc_axi_t;

/* The same physics on a non-uniform (r, z) grid: grid.f's level-1 positions
 * and finite-difference weights (orc_str_levels + orc_str_coefficients) and
 * rcsc.f's stretched multigrid for the streamfunction (orc_str_poisson; its
 * operator psi_rr + psi_r/r - psi/r^2 + psi_zz is rotann2.f's).  rotann2.f
 * has no such mode: the reference's only stretched-grid driver is rcsc.f,
 * whose transport this follows for the derivative weights.  At a point
 * (i, j) of the stretched transport:
 *   d/dr x    = cr1 x(i-1) + cr2 x(i) + cr3 x(i+1)            (rcsc.f dum2)
 *   d2/dr2 x  = the 4-point crr weights, orientation switching at nr/2
 *               (rcsc.f dum1a / dum3a off the centre), centre crr_c
 *   the same in z with cz, czz and nz/2;
 *   every central difference (x(j+1) - x(j-1)) / (2 dz) of rotann2.f's
 *   vorticity, velocity and temperature becomes d/dz x, every
 *   (x(i+1) + x(i-1)) / dr^2 the off-centre part of d2/dr2 x, every
 *   (x(i+1) - x(i-1)) / (2 r dr) the off-centre part of (d/dr x) / r;
 *   the Dufort-Frankel centre: sigma = crr_c + cr2 / r + czz_c replaces
 *   -2/dr^2 - 2/dz^2 (rcsc.f's cnr + cnz, doubled), so cf1 becomes
 *   1/(2 Ptl dt) - sigma/2 and cf2 1/(2 Ptl dt) + sigma/2 (cf3, cf4 with dt);
 *   the Arakawa sum is divided by 3 (r(i+1) - r(i-1)) (z(j+1) - z(j-1))
 *   (12 hr hz on the uniform grid: the Jacobian in index space over the
 *   local metric);
 *   the temperature's mirrored wall rows j = 0, nz: d/dz = 0,
 *   d2/dz2 x = 2 (x(i, 1) - x(i, 0)) / h^2 with h the wall spacing;
 *   Thom wall vorticity 2 psi(next) / h^2 with the wall spacing (rcsc.f
 *   update, :706-751); the heat flux with the five-point one-sided d/dr
 *   weights at the inner wall on r(0..4) (grid.f's fdif, grid.f:926-1032,
 *   fourth order as rotann2.f's heat stencil) and the trapezoid rule in z. */
int  orc_axi_set_stretched(orc_axi_t *s, const orc_str_grid_t *g, orc_str_mg_t *m);

int  orc_axi_init(orc_axi_t *s, int nr, int nz, double dt, double r0, double rmax, double zmax,
                  double Ra, double Re, double Ptl);
void orc_axi_free(orc_axi_t *s);
/* kind 0: the reference's start (rotann2.f:76-93): conduction profile
 * 1 - ln(r/rmax)/ln(r0/rmax) with +0.01 at (nr/4, nz/4); kind 1: the same
 * profile plus seeded uniform noise of amplitude amp (splitmix64, j-major
 * over rows i = 1..nr-1).  Both copy the previous time level (rotann2.f:131-136). */
void orc_axi_initial(orc_axi_t *s, int kind, unsigned long long seed, double amp);

void orc_axi_arakawa(const orc_axi_t *s, double *arak, const double *psi, const double *th);
void orc_axi_vorticity(orc_axi_t *s);
void orc_axi_velocity(orc_axi_t *s);
void orc_axi_temperature(orc_axi_t *s);
double orc_axi_heat(const orc_axi_t *s);
void orc_axi_update(orc_axi_t *s);
/* poisson(phi, omegn) (rotann2.f:598-666): returns 0 when converged (psi
 * updated), 1 when the sweep limit was reached (psi untouched). */
int  orc_axi_poisson(orc_axi_t *s, double *psi, const double *rhs, int *sweeps);
void orc_axi_relax(orc_axi_t *s, int nrel, int klev, int *nconv);
void orc_axi_corser(orc_axi_t *s, int klev);
void orc_axi_finer(orc_axi_t *s, int klev);

/* One step of the main loop (rotann2.f:147-152): vorticity, velocity,
 * temperature, poisson, update, heat.  *nu receives httrans
 * (rotann2.f:155), *converged the main loop's steady-state test
 * (rotann2.f:162-194, REAL*4 threshold 1e-6).  Returns the poisson status. */
int  orc_axi_step(orc_axi_t *s, double *nu, int *sweeps, int *converged);

#ifdef __cplusplus
}
#endif
#endif
