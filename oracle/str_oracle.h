/*
 * CPU oracle for the stretched-grid streamfunction operator of rcsc.f
 * ("STR") and the coefficient build of grid.f:
 *
 *   grid.f:723-857  wall-clustered spacings (geometric expansion factor
 *                   near both walls, uniform core), or uniform spacings;
 *   grid.f:859-924  levels: coarse spacings are sums of fine pairs,
 *                   positions their running sums, at most 6 levels;
 *   grid.f:926-1115 finite-difference weights by inverting the Taylor
 *                   matrix of the stencil points (Gaussian elimination with
 *                   partial pivoting, gausse);
 *   grid.f:178-226  per level: first-derivative weights on (i-1, i, i+1),
 *                   second-derivative weights on (i-1..i+2) for i <= n/2
 *                   and on (i-2..i+1) above;
 *   rcsc.f:1118-1444 the multigrid: psi_rr + psi_r / r - psi / r^2 + psi_zz
 *                   with those weights, pentadiagonal r-line and z-line
 *                   Gauss-Seidel (relax, tolcon 1e-6, nrel 2), nine-point
 *                   restriction clearing rows and columns 0 and n1 of the
 *                   coarse level in both directions, bilinear prolongation,
 *                   plain V-cycle from psi itself (no over-relaxation), no
 *                   STOP after nvs = 10000 sweeps.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of tests/ and bench.py's CPU legs;
 * never linked into the product.  PARITY PINNED to grid.f and rcsc.f run
 * through the translator tests/golden/f77.py.  Double precision, the
 * reference's order,
 * -ffp-contract=off.
 *
 * Arrays: psi and rhs are (0:n1, 0:n2) column-major with leading dimension
 * n1+1 (level 1).  Level l's tables: r[l][0..n1], cr[l][3*(i-1)+k] and
 * crr[l][4*(i-1)+k] for i = 1..n1-1, czz[l][4*(j-1)+k] for j = 1..n2-1.
 */
#ifndef STR_ORACLE_H
#define STR_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define STR_MAXLEV 8
#define STR_MAXN 4097

/* grid (grid.f:723-857).  gef > 0: first spacing d1, spacings growing by
 * gef until their sum passes dist (capped at n/2 points), mirrored at the
 * far wall, the rest uniform; gef <= 0: uniform.  Returns 0, or -1 where
 * the reference STOPs ("too many grid points in GEF region", "grid points
 * exceeded"). */
int orc_str_spacing_gef(int n, double lo, double hi, double dist, double gef, double d1, double *h);

/* level (grid.f:859-924) for level-1 spacings hr1[1..n1], hz1[1..n2]
 * (1-based, index 0 unused); fills n1[l], n2[l], hr[l][1..], hz[l][1..],
 * r[l][0..], z[l][0..] and returns nlev (halvings while both halve exactly
 * and are >= 4, capped at 6). */
typedef struct {
    int nlev;
    int n1[STR_MAXLEV], n2[STR_MAXLEV];
    double *hr[STR_MAXLEV], *hz[STR_MAXLEV], *r[STR_MAXLEV], *z[STR_MAXLEV];
    double *cr[STR_MAXLEV], *crr[STR_MAXLEV], *cz[STR_MAXLEV], *czz[STR_MAXLEV];
    double cr0[3], crn[3], cz0[3], czn[3];   /* one-sided wall weights of level 1 (grid.f:228-243) */
} orc_str_grid_t;

int  orc_str_levels(orc_str_grid_t *g, int n1, int n2, const double *hr1, const double *hz1, double r0,
                    double zmin, int maxlev);
void orc_str_grid_free(orc_str_grid_t *g);
/* fdif (grid.f:926-1032) with nans = 0: weights of the nx points
 * x[k-nref+1 .. k-nref+nx] (x 0-based here) for derivatives 0..nx-1;
 * w[d*nx + p] = weight of point p for derivative d.  Returns -1 on a
 * singular matrix (the reference STOPs). */
int  orc_str_fdif(int nx, int nref, int k, const double *x, double *w);
/* The coefficient tables of every level (grid.f:178-243). */
int  orc_str_coefficients(orc_str_grid_t *g);

/* Multigrid state (COMMON /backup/ /arrays/ /step/ /ints/ /coeff/). */
typedef struct {
    const orc_str_grid_t *g;
    int nlev, ld;
    double *v[STR_MAXLEV], *f[STR_MAXLEV];
    double *psif, *rc;
    double tolcon;     /* 1e-6 (rcsc.f:1216) */
    int nrel;          /* 2 (rcsc.f:1144-1145) */
    int maxsweeps;     /* nvs = 10000 (rcsc.f:1143) */
    int mode;          /* 0: the reference's line order; 1: four colours of lines (index mod 4 =
                          1, 2, 3, 0), each colour's lines independent */
    double last_resmax;
} orc_str_mg_t;

int  orc_str_mg_init(orc_str_mg_t *m, const orc_str_grid_t *g, int nlev);
void orc_str_mg_free(orc_str_mg_t *m);
/* poisson(psi, rhs, nlev, vel) (rcsc.f:1118-1195): returns 0 when converged
 * (psi updated), 1 after maxsweeps sweeps (psi untouched), 2 on a NaN
 * residual; *sweeps the sweep count. */
int  orc_str_poisson(orc_str_mg_t *m, double *psi, const double *rhs, int *sweeps);
void orc_str_relax(orc_str_mg_t *m, int nrel, int klev, int *nconv);
void orc_str_corser(orc_str_mg_t *m, int klev);
void orc_str_finer(orc_str_mg_t *m, int klev);

#ifdef __cplusplus
}
#endif
#endif
