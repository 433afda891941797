/*
 * CPU oracle for the 2D periodic Rayleigh-Benard hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker used by tests/,
 * __graft_entry__.smoke() and the cpu_baseline / reference legs of bench.py.
 * Nothing in the product (codesthesis_dir_gb300/) links or calls it.
 *
 * It is a plain-C restatement of the Fortran 77 routines of
 * monashubuntudir_velvor2dperiodicrbconvdir/velvor2dperiodicrbconv.f
 * ("PRB" below), double precision throughout, evaluated in the
 * reference's left-to-right operation order, compiled with
 * -ffp-contract=off so that no multiply-add is fused.
 *
 * PARITY PINNED to the reference's own source.  The reference ships no
 * tests, golden vectors or stored outputs and the image has no Fortran
 * compiler, so the reference's drivers are run on the CPU by a translator
 * of their Fortran (tests/golden/f77.py: IEEE binary64 / binary32
 * arithmetic in source order); this restatement reproduces those runs bit
 * for bit (tests/test_reference_runs.py), the Taylor-Couette driver with
 * the relax2 of its newer sibling (velvor2dtaycouheat.f forms a line's
 * right-hand side only for k = 1 and its first solve STOPs).  Its own
 * invariants (dense-solve agreement of the banded solvers, manufactured
 * solutions, conduction Nusselt number 1, periodic-seam identities) are
 * checked too.
 *
 * Array convention: every field is the reference's (0:kr,1,0:kp) array,
 * stored column-major, element (i,k) at index i + ld*k, 0 <= i <= ld-1,
 * 0 <= k <= np.  ld is the declared leading dimension (kr+1 in the
 * reference, 291 for kr=290); the oracle's own state uses ld = nr+2.
 */
#ifndef PRB_ORACLE_H
#define PRB_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Smoother orderings of the multigrid line relaxation. */
#define ORC_LEX   0   /* k = 1..n3 in order: the reference schedule (PRB:2113-2191) */
#define ORC_ZEBRA 1   /* odd k lines, then even k lines: the GPU-parallel schedule */

/* Status codes, shared with the GPU library. */
#define ORC_OK        0
#define ORC_MAXSWEEPS 1   /* the reference STOPs here (PRB:1843) */
#define ORC_NAN       2
#define ORC_INVALID   5

/* Banded solvers, 1-based semantics of PRB:3046-3164 on 0-based arrays.
 * Inputs are destroyed exactly as in the reference. */
void orc_tdma(double *a, double *b, double *c, double *y, double *r, int n);
void orc_ptdma(double *a, double *b, double *c, double *y, double *r, int n);
void orc_pdma(double *a, double *b, double *c, double *d, double *e,
              double *r, double *x, int n);

/* Multigrid state (COMMON /backup/, /arrays/, /step/, /ints/ of PRB). */
typedef struct {
    int nr, np, ld, nlev;
    int n1[7], n3[7];
    double hr[7], hp[7], hhr[7], hhp[7];
    double *v[7], *f[7];                 /* packed per-level storage */
    double *psic, *psif, *rc, *rf, *tempa;
    double tolcon;                       /* 2e-6 in PRB:2086 */
    double sor;                          /* 1.2 in PRB:1850 */
    int maxsweeps;                       /* 500 in PRB:1843 */
    int mode;                            /* ORC_LEX or ORC_ZEBRA */
    int zero_scratch;                    /* 1: zero v,f of mgen doubles per call (PRB:1822-1825) */
    long mgen;                           /* size zeroed when zero_scratch */
    double *scratch_v, *scratch_f;       /* the mgen-sized buffers when zero_scratch */
    int last_sweeps;
    double last_resmax;
    /* variant ORC_PRB (velvor2dperiodicrbconv.f) or ORC_ANNULUS (the polar
     * (r,phi) plane of velvor2dnewsch3.4.f): polar coefficients, three
     * relaxations per call, no reset of the coarse seam of rc, level cap 5 */
    int variant;
    double r0;
    /* ORC_TANK (velvor2dhorconvtank.f:1163-1303): side walls in x.  relax2
     * runs and measures lines k = 1..n3-1 (the v walls k = 0, n3 are not
     * relaxed); relax3's last line k = n3 takes k = 0 (zero) as its k+1
     * neighbour and resets psif(0) to zero instead of copying the seam;
     * tolcon 5e-6; the final update writes v on k = 1..np-1 and zeroes
     * k = 0, np, u on k = 1..np and zeroes k = 0, np+1. */
    int xwall;
} orc_mg_t;

#define ORC_PRB     0
#define ORC_ANNULUS 1
#define ORC_OBLIQUE 2   /* the layer with gravity at 45 degrees (mpkoks.f:769-770, :974-975) */
/* the annulus with a moving outer cylinder, velvor2dtaycouheat.f: the
 * annulus's transport with Robert filter 0.01 (:605, :837), the outer wall
 * v = -(Ta**0.5) Ptl rmax / 2 (the start :177, update :1587), its wall
 * vorticity (8/3 v(nr+1) + v(nr-1)/3 - 3 v(nr))/dr + v(nr+1)/rmax (:1589-1590)
 * and its term in rhsv at i = nr (:1668-1670); the multigrid of PRB (one
 * relaxation per visit, the coarse seam reset, STOP after 500 sweeps, at
 * most 4 levels) with the polar operator and tolcon 1e-5 (:1234, :1345). */
#define ORC_TAYCOU  3
/* the horizontal-convection tank, velvor2dhorconvtank.f (tank_oracle.c):
 * the layer closed by side walls in x */
#define ORC_TANK    4
/* the differentially heated cavity benchmark, velvor2ddvdbenchmark.f: the
 * tank's side-walled scheme with the DVD differences (tank_oracle.c) */
#define ORC_DVD     5

int  orc_mg_init(orc_mg_t *mg, int nr, int np, double dr, double dp);
/* Same with the variant and inner radius of the annulus driver. */
int  orc_mg_init_variant(orc_mg_t *mg, int nr, int np, double dr, double dp, int variant, double r0);
void orc_mg_free(orc_mg_t *mg);
/* which = 2: poisson2/relax2 (cell-centred v, pentadiagonal r-lines)
 * which = 3: poisson3/relax3 (face u, tridiagonal r-lines)
 * psi, psip, rhs use leading dimension ld_io.  Returns a status code;
 * *sweeps receives the number of outer sweeps taken. */
int  orc_poisson(orc_mg_t *mg, int which, double *psi, double *psip,
                 const double *rhs, int ld_io, int *sweeps);

/* Individual multigrid building blocks (exposed for unit tests). */
void orc_relax(orc_mg_t *mg, int which, int nrel, int klev, int *nconv);
void orc_corser(orc_mg_t *mg, int klev);
void orc_finer(orc_mg_t *mg, int klev);

/* Physical state of PRB (COMMON /sol1/ /sol2/ /sol3/ /num/ /val/ /radius/). */
typedef struct {
    int nr, np, ld;
    double dt, dr, dp, Ra, Pr, r0, rmax, xx;
    double *An, *A, *Ap, *Bn, *B, *Bp, *Cn, *C, *Cp;
    double *thn, *th, *thp;
    double *uel, *vel, *wel, *uelp, *velp, *welp;
    double *urh, *vrh;
    long clamp_count;                    /* "WARNING! Temp damped" count */
    int variant;                         /* ORC_PRB, ORC_ANNULUS, ORC_OBLIQUE or ORC_TAYCOU */
    double Re;                           /* rotational Reynolds number (annulus) */
    double Ta;                           /* Taylor number (ORC_TAYCOU; COMMON /val/ Gr there) */
} orc_prb_t;

int  orc_prb_alloc(orc_prb_t *s, int nr, int np, int ld);
void orc_prb_free(orc_prb_t *s);

void orc_cvorticity1(orc_prb_t *s);
void orc_cvorticity(orc_prb_t *s);
void orc_temperature1(orc_prb_t *s);
void orc_temperature(orc_prb_t *s);
void orc_heat(const orc_prb_t *s, double *trans1, double *trans2);
void orc_update(orc_prb_t *s);
void orc_rhsv(orc_prb_t *s);
void orc_rhsu(orc_prb_t *s);

/* One time step of the PRB main loop (PRB:341-388 for kt=1, PRB:363-388
 * otherwise).  nu[0], nu[1] receive httrans, httrans2; sweeps[0], sweeps[1]
 * the outer sweep counts of the v and u solves.  Returns a status code. */
int  orc_prb_step(orc_prb_t *s, orc_mg_t *mgv, orc_mg_t *mgu, int kt,
                  double *nu, int *sweeps);

/* Diagnostics of the time loop.  Arrays are (ld, np+1) column-major like the
 * fields.
 *
 * orc_prb_diag_accum, PRB:404-416 (velvor2dnewsch3.4.f:404-416 alike): at step
 * kt >= 2 the running means over the block's steps 2..kt of T^2, T, u^2 and
 * v^2, m = (1/(kt-1)) m (kt-2) + (1/(kt-1)) x, rows 0..nr+1, k = 0..np.
 *
 * orc_prb_cfl, PRB:420-459: max |u dt / dr| over i = 1..nr and
 * max |v dt / (r dp)| over i = 1..nr-1 (r = 1 in PRB, r0 + (i - 1/2) dr in
 * the annulus, velvor2dnewsch3.4.f:437-445); NaN entries never win a
 * comparison.
 *
 * orc_prb_zmtm, PRB:474-493: per row i = 0..nr+1, the zonal means
 * (sum msqT - sum mT^2) / (np+1), (sum msqU / (np+1))**0.5 and
 * (sum msqV / (np+1))**0.5 (libm pow, as the compiled Fortran evaluates
 * **0.5d0), summed over k = 0..np in order; out[3 i + c]. */
void orc_prb_diag_accum(const orc_prb_t *s, int kt, double *msqT, double *mT, double *msqU, double *msqV);
void orc_prb_cfl(const orc_prb_t *s, double *cflu, double *cflv);
void orc_prb_zmtm(const orc_prb_t *s, const double *msqT, const double *mT, const double *msqU,
                  const double *msqV, double *out);

/* The tank (tank_oracle.c); the state's fields have np+2 columns. */
void orc_tank_cvorticity(orc_prb_t *s, int first);
void orc_tank_temperature(orc_prb_t *s, int first);
void orc_tank_heat(const orc_prb_t *s, double *trans1, double *trans2);
void orc_tank_update(orc_prb_t *s);
void orc_tank_rhsv(orc_prb_t *s);
void orc_tank_rhsu(orc_prb_t *s);
void orc_tank_initial(orc_prb_t *s);

/* Initial conditions.  kind 0: the reference's own deterministic profile
 * (PRB:137-186; for ORC_ANNULUS the conduction profile 1 - ln r / ln r0
 * with the sine ripple of velvor2dnewsch3.4.f:131-150).  kind 1: linear conduction plus seeded uniform noise of
 * amplitude amp drawn from splitmix64(seed), periodic duplicate k=np equal
 * to k=0.  Both set Ap..thp, uelp, velp as PRB:316-331 does. */
void orc_prb_initial(orc_prb_t *s, int kind, unsigned long long seed, double amp);

#ifdef __cplusplus
}
#endif
#endif
