/*
 * CPU oracle for the 3D rotating annulus of rot3dmg.f ("R3D"): the
 * Dufort-Frankel update of the three staggered vorticity components A, B, C
 * and of the temperature with hybrid upwinding, the wall vorticities and wall
 * temperatures of update, the inner-wall heat flux, the right-hand sides of
 * the three velocity Poisson equations, and the velocity multigrid
 * (r-, z- and phi-line Gauss-Seidel per sweep, 27-point full weighting,
 * trilinear prolongation, plain V-cycle with SOR 1.2).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of tests/, smoke() and bench.py's
 * CPU legs; never linked into the product.  PARITY PINNED to rot3dmg.f and
 * rot3dmghor.f run through the translator tests/golden/f77.py
 * (tests/test_reference_runs.py).
 * Double precision, the reference's left-to-right order, -ffp-contract=off;
 * the REAL*4 literal 0.2 of relax1/2/3 (rot3dmg.f:1626, 1634, 1664, 1672,
 * 1800, 1805, 2029, 2034, 2106, 2112) is the float it rounds to.
 *
 * Every field is the reference's (0:kr, 0:kz, 0:kp) array cut to
 * (0:nr+1, 0:nz+1, 0:np), column-major: element (i, j, k) at
 * i + (nr+2) * (j + (nz+2) * k).
 */
#ifndef R3D_ORACLE_H
#define R3D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Line orderings of relax1/2/3.  R3D_LEX is the reference's: r-lines with
 * k outer and j inner (rot3dmg.f:1572-1573), z-lines k outer and i inner
 * (:1609-1610), phi-lines j outer and i inner (:1649-1650).  R3D_ZEBRA is
 * the parallel ordering: in each direction, the lines whose two transverse
 * indices have an even sum, then those with an odd sum; within a colour,
 * first the lines on two one-sided boundary rows (the rows whose stencils
 * reach two lines over, e.g. i = 1 reading i + 2), then those on one such
 * row, then the rest.  A line reads only lines of the other colour and,
 * on a one-sided row, the line two over of its own colour on fewer
 * one-sided rows, which comes later: every line of a colour sees the
 * colour's lines as they were before the colour's pass, so the lines of a
 * colour can be solved all at once. */
#define R3D_LEX   0
#define R3D_ZEBRA 1

#define R3D_OK        0
#define R3D_MAXSWEEPS 1   /* the reference STOPs here (rot3dmg.f:1259) */
#define R3D_NAN       2
#define R3D_INVALID   5

#define R3D_MAXLEV 8

typedef struct {
    int nr, nz, np;
    int ni, nj, nk;                 /* nr+2, nz+2, np+1 */
    double dt, r0, rmax, zmax, Ra, Re, Gr, Ptl;
    double dr, dz, dp, pi;
    /* COMMON /sol1/ /sol2/ /sol3/ and the main program's rhs arrays */
    double *An, *A, *Ap, *Bn, *B, *Bp, *Cn, *C, *Cp;
    double *thn, *th, *thp;
    double *uel, *vel, *wel, *uelp, *velp, *welp;
    double *urh, *vrh, *wrh;
    /* multigrid (poissoninit, rot3dmg.f:1153-1213) */
    int nlev;
    int n1[R3D_MAXLEV], n2[R3D_MAXLEV], n3[R3D_MAXLEV];
    double hr[R3D_MAXLEV], hz[R3D_MAXLEV], hp[R3D_MAXLEV];
    double hhr[R3D_MAXLEV], hhz[R3D_MAXLEV], hhp[R3D_MAXLEV];
    double *v[R3D_MAXLEV], *f[R3D_MAXLEV], *res[R3D_MAXLEV];
    double tolcon;                  /* 1e-5 (rot3dmg.f:1562) */
    double sor;                     /* 1.2 (rot3dmg.f:1263) */
    int nrel;                       /* nrel1 = nrel2 = 2 (rot3dmg.f:1237-1238) */
    int maxsweeps;                  /* STOP beyond 500 sweeps (rot3dmg.f:1259) */
    int mode;                       /* R3D_LEX or R3D_ZEBRA */
    double last_resmax;
    int last_sweeps;
    /* rot3dmghor.f, the annulus with its axis horizontal (set by
     * orc_r3d_set_horizontal): gravity Gr Ptl across the axis as the only
     * body force in the three vorticity updates (:477-479, :604-606,
     * :747-749) with sin and cos of theta = 6.283185307/np k (libm, per
     * k = 0..np); the heat flux of both cylinders over the band
     * j = nz/2-3 .. nz/2+3 (:913-945); the inner cylinder hot (thn = 1 at
     * i = 0, 0 at i = nr+1, :1042-1043); a plain V-cycle without the
     * whole-cycle over-relaxation and without the psip copies (:1287-1315,
     * commented out there); tolcon 1e-6 (:1599, :1798, :2051); the start
     * T = ln r / ln r0 + ... with the point (nr/2, nz/2, np/2) halved
     * (:133-141); Nusselt numbers nz/6 r0 ln(r0/rmax) trans1 / (zmax 2 pi)
     * and the same with rmax and trans2 (:264-267). */
    int horizontal;
    double *sinth, *costh;
    double nu2;                     /* httrans2 of the last step */
} orc_r3d_t;

/* Sets sizes, constants (rot3dmg.f:92-96) and the multigrid levels; all
 * fields zero.  Returns R3D_INVALID when nr, nz < 4, or np is not a multiple
 * of 2^nlev with at least 4 phi intervals on the coarsest level. */
int  orc_r3d_init(orc_r3d_t *s, int nr, int nz, int np, double dt, double r0, double rmax, double zmax,
                  double Ra, double Re, double Gr, double Ptl);
void orc_r3d_free(orc_r3d_t *s);
/* The reference's start (rot3dmg.f:103-131): zero flow, temperature
 * 1 - ln r / ln r0 + amp (rmax - r)(r - r0) cos(nval phi), the point
 * (nr/4, nz/4, np/2) halved, and the previous time level copied
 * (rot3dmg.f:220-230). */
void orc_r3d_initial(orc_r3d_t *s, int nval, double amp);
/* Switches s to rot3dmghor.f (see the horizontal field); call after init. */
int  orc_r3d_set_horizontal(orc_r3d_t *s);

void orc_r3d_avorticity(orc_r3d_t *s);
void orc_r3d_bvorticity(orc_r3d_t *s);
void orc_r3d_cvorticity(orc_r3d_t *s);
void orc_r3d_temperature(orc_r3d_t *s);
double orc_r3d_heat(const orc_r3d_t *s);
/* heat(trans1, trans2) of rot3dmghor.f:913-945 (both cylinders). */
double orc_r3d_heat2(const orc_r3d_t *s, double *trans2);
void orc_r3d_update(orc_r3d_t *s);
void orc_r3d_rhsw(orc_r3d_t *s);
void orc_r3d_rhsv(orc_r3d_t *s);
void orc_r3d_rhsu(orc_r3d_t *s);

/* poisson1 (which = 1: w, wel/welp/wrh), poisson2 (2: v), poisson3 (3: u),
 * rot3dmg.f:1216-1540.  Returns R3D_OK with the velocity and its previous
 * level updated, or R3D_MAXSWEEPS / R3D_NAN. */
int  orc_r3d_poisson(orc_r3d_t *s, int which, int *sweeps);
/* relax1/2/3 on level klev (1-based) with nrel sweeps; nconv as the
 * reference sets it.  corser / finer move between klev and klev +/- 1. */
void orc_r3d_relax(orc_r3d_t *s, int which, int nrel, int klev, int *nconv);
void orc_r3d_corser(orc_r3d_t *s, int klev);
void orc_r3d_finer(orc_r3d_t *s, int klev);

/* One step of the main loop (rot3dmg.f:241-253); *nu receives httrans
 * (rot3dmg.f:255), sweeps[3] the sweep counts of the w, v and u solves.
 * Returns the first failing solve's status (the reference STOPs there). */
int  orc_r3d_step(orc_r3d_t *s, double *nu, int *sweeps);

#ifdef __cplusplus
}
#endif
#endif
