/*
 * gb300_convection.h -- C ABI of the GB300 (sm_103a) implementation of the
 * time-step hot path of the rotating-annulus / Rayleigh-Benard convection
 * codes (martin-king/codesthesis_dir, Fortran 77).
 *
 * Library: codesthesis_dir_gb300/_build/libgb300conv.so
 *
 * Three layers, all plain C types (pointers, sizes, status codes):
 *
 *  1. gfortran-compatible drop-in symbols (lower case, trailing underscore,
 *     every argument by reference) for the subroutines of
 *     monashubuntudir_velvor2dperiodicrbconvdir/velvor2dperiodicrbconv.f
 *     (abbreviated PRB below).  They read and write the caller's COMMON
 *     blocks /sol1/ /sol2/ /sol3/ /num/ /val/ /radius/ exactly as the
 *     Fortran routines they replace, and run the work on the GPU.
 *
 *  2. A context API (gb_prb_*) that keeps every field resident on the
 *     device between calls and steps; the drop-in symbols are thin wrappers
 *     over one process-wide context.
 *
 *  3. The batched Poisson solver (gb_batch_*) and batched banded line
 *     solvers (gb_*_batch).
 *
 * Status codes: every entry point that can fail returns (or stores) one of
 * GB_OK ... GB_ERR_*; no entry point exits the process (the reference STOPs
 * after 500 multigrid sweeps, PRB:1843; here that is GB_MAXSWEEPS).
 * gb_last_error() gives a one-line description of the last failure on the
 * calling thread.
 */
#ifndef GB300_CONVECTION_H
#define GB300_CONVECTION_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define GB_OK            0
#define GB_MAXSWEEPS     1  /* multigrid hit its sweep limit (PRB:1843 STOPs there) */
#define GB_NAN           2  /* a NaN residual was seen */
#define GB_TIMEOUT       3  /* a bounded device-side wait gave up */
#define GB_ERR_ALLOC     4  /* device or host allocation failed */
#define GB_ERR_INVALID   5  /* invalid argument or grid size */
#define GB_ERR_CUDA      6  /* CUDA runtime error (see gb_last_error) */

const char *gb_last_error(void);
/* Library build string: version, target architecture, build flags. */
const char *gb_version(void);

/* ---------------------------------------------------------------- fields */
/* Field identifiers, in the order of the reference COMMON blocks
 * /sol1/ An,A,Ap,Bn,B,Bp,Cn,C,Cp  /sol2/ thn,th,thp
 * /sol3/ uel,vel,wel,uelp,velp,welp (PRB:69-71), plus the two Poisson
 * right-hand sides urh, vrh of the main program (PRB:60). */
enum gb_prb_field {
    GB_F_An = 0, GB_F_A, GB_F_Ap, GB_F_Bn, GB_F_B, GB_F_Bp, GB_F_Cn, GB_F_C, GB_F_Cp,
    GB_F_thn, GB_F_th, GB_F_thp,
    GB_F_uel, GB_F_vel, GB_F_wel, GB_F_uelp, GB_F_velp, GB_F_welp,
    GB_F_urh, GB_F_vrh,
    GB_F_COUNT
};

/* Smoother orderings of the multigrid line relaxation. */
#define GB_SMOOTHER_LEX   0  /* k = 1..n3 in order: the reference schedule (PRB:2113-2191) */
#define GB_SMOOTHER_ZEBRA 1  /* odd k lines, then even k lines (all lines of a colour in parallel) */

/* Parameters of one 2D periodic Rayleigh-Benard instance.  Defaults that
 * reproduce the reference: tolcon 2e-6 (PRB:2086), sor 1.2 (PRB:1850),
 * maxsweeps 500 (PRB:1843), xx 3 (PRB:132), smoother LEX. */
typedef struct gb_prb_params {
    int nr;          /* intervals in r (wall-normal), even, >= 4 */
    int np;          /* intervals in the periodic direction, even, >= 4 */
    double dt, r0, rmax, xx;
    double Ra, Pr;   /* Rayleigh and Prandtl numbers (COMMON /val/ Ra, Ptl) */
    double tolcon;   /* absolute max-norm residual tolerance of the level-1 relax */
    double sor;      /* over-relaxation factor of the whole-cycle change */
    int maxsweeps;   /* outer multigrid sweep limit */
    int smoother;    /* GB_SMOOTHER_LEX or GB_SMOOTHER_ZEBRA */
    int variant;     /* GB_PRB_LAYER, GB_PRB_ANNULUS or GB_PRB_OBLIQUE */
    double Re;       /* rotational Reynolds number (COMMON /val/ Re; annulus only) */
    int precision;   /* GB_PRB_FP64 (bit-exact) or GB_PRB_MIXED (FP32 cycles inside FP64 defect correction) */
    double Ta;       /* Taylor number (GB_PRB_TAYCOU; read into COMMON /val/ Gr there) */
} gb_prb_params;

/* Precision of the velocity multigrid solves.
 *   GB_PRB_FP64:  the reference algorithm in FP64, bit-identical to it.
 *   GB_PRB_MIXED: FP64 defect correction: each outer iteration forms the
 *                 FP64 residual r = rhs - A psi on the finest level, stops
 *                 when its max norm is below tolcon, and otherwise runs the
 *                 reference's multigrid sweep schedule in FP32 on A e = r
 *                 from e = 0 and updates psi += w e in FP64 (w = 1 on the
 *                 first iteration, then the reference's over-relaxation
 *                 1.2).  The sweep count reported is the number of FP32
 *                 cycles.  Transport, Nusselt integrals and boundary
 *                 conditions stay FP64. */
#define GB_PRB_FP64  0
#define GB_PRB_MIXED 1

/* Geometry and physics of an instance.
 *   GB_PRB_LAYER:   the periodic plane layer of velvor2dperiodicrbconv.f
 *                   (x period xx, dp = xx/np, Nu = trans*(rmax-r0)/xx).
 *   GB_PRB_ANNULUS: the (r, phi) plane of the rotating annulus,
 *                   iarchomedir_groke_storage_users_mpking_rotannconvvelvorplane_continueddir/
 *                   velvor2dnewsch3.4.f: dp = 2 pi/np, polar terms in the
 *                   transport (:710-993, :1140-1393), in rhsv/rhsu
 *                   (:1666-1730) and in relax2/relax3 (:2071-2596), Robert
 *                   filter 0.05, rotational buoyancy 2 Ra (-thr u - thh v/r)/Re/Ptl
 *                   (:779), up to 5 multigrid levels (:1778), three
 *                   relaxations per level visit (:2134, :2410), no reset of
 *                   the coarse seam residual in corser (:2696-2704), no STOP
 *                   after the sweep limit (:1853), Nu = -r0 ln(r0/rmax)
 *                   trans1/(2 pi) (:386-387).
 *   GB_PRB_OBLIQUE: the layer with gravity along the diagonal,
 *                   monashubuntudir_velvor2dperiodicrbconvdir/mpkoks.f: the
 *                   buoyancy term of both vorticity updates is
 *                   RHS2 = -Ra thr 0.707106781 (REAL*4 literal; :769-770,
 *                   :974-975) instead of -Ra thh; all else is the layer's.
 *   GB_PRB_TAYCOU:  the annulus with a moving outer cylinder,
 *                   monashubuntudir_velvor2dtaycouheatdir/velvor2dtaycouheat.f:
 *                   the annulus's geometry and transport with Robert filter
 *                   0.01 (:605, :837); the outer wall moves at
 *                   v = -(Ta**0.5) Ptl rmax / 2 (the start :177 and every
 *                   update :1587, libm pow), its wall vorticity is
 *                   (8/3 v(nr+1) + v(nr-1)/3 - 3 v(nr))/dr + v(nr+1)/rmax
 *                   (:1589-1590) and rhsv adds its term at i = nr
 *                   (:1668-1670); the multigrid is PRB's (one relaxation
 *                   per visit, coarse seam reset, STOP after 500 sweeps,
 *                   at most 4 levels) with the polar operator and tolcon
 *                   1e-5 (:1234, :1345); Nu as the annulus's.
 *   GB_PRB_TANK:    the horizontal-convection tank,
 *                   monashubuntudir_velvor2dhorconvtankdir/velvor2dhorconvtank.f:
 *                   the layer closed by side walls at x = 0 and x = xx; C
 *                   and v on the faces k = 0..np, T and u on the cells
 *                   k = 1..np with ghost columns 0 and np+1, so every field
 *                   has np+2 columns (set/get_field move np+2 columns);
 *                   plain Thomas x-lines; the top wall T = k/np, an
 *                   insulated bottom and insulated side walls (:812-845);
 *                   heat over k = np/2..np-1; Nu = 2 trans, the first step
 *                   storing 2 trans2 in httrans and zero in httrans2
 *                   (:197-198); the multigrid with side walls (v lines
 *                   k = 1..np-1, u lines k = 1..np against the zero wall)
 *                   and tolcon 5e-6.  FP64 only.
 *   GB_PRB_DVD:     the differentially heated cavity benchmark,
 *                   monashubuntudir_velvor2ddvdbenchmarkdir/velvor2ddvdbenchmark.f:
 *                   the tank's scheme (np+2 columns, same multigrid) with
 *                   xx = 1, T = 0 and 1 on the bottom and top rows and
 *                   insulated side walls (:822-830), side-wall vorticities
 *                   -u(1)/dp and u(np)/dp (:819-820), buoyancy -Ra thr
 *                   (:437, :560), its own wall rows of the T derivatives
 *                   (:382-383, :601, :696), the T Robert filter on
 *                   i = 1..nr, heat over k = 2..np-1 and Nu = trans (with
 *                   the tank's first-step quirk).  FP64 only. */
#define GB_PRB_LAYER   0
#define GB_PRB_ANNULUS 1
#define GB_PRB_OBLIQUE 2
#define GB_PRB_TAYCOU  3
#define GB_PRB_TANK    4
#define GB_PRB_DVD     5

/* Fills *p with the reference defaults for an nr x np grid
 * (dt 1e-7, r0 0.5, rmax 1, xx 3, Ra 1e7, Pr 0.71: the PRB input deck). */
void gb_prb_default_params(gb_prb_params *p, int nr, int np);
/* The annulus defaults (velvor2dnewsch3.4.f with its input.s: dt 2e-8,
 * r0 0.5, rmax 1, Ra 8e8, Re 1.06148e5, Pr 0.71; tolcon 1e-5 (:2093),
 * sweep limit 10000 (:1829)). */
void gb_prb_default_params_annulus(gb_prb_params *p, int nr, int np);
/* The Taylor-Couette defaults (velvor2dtaycouheat.f with its input.s: dt
 * 2e-8, r0 0.5, rmax 1, Ra 6e8, Re 91927, Ta 0, Pr 0.71; tolcon 1e-5, sweep
 * limit 500). */
void gb_prb_default_params_taycou(gb_prb_params *p, int nr, int np);
/* The tank defaults (velvor2dhorconvtank.f with its input.s: dt 5e-8,
 * r0 0.5, rmax 1.5, xx 3.1, Ra 8.63e7, Pr 10; tolcon 5e-6, sweep limit 500). */
void gb_prb_default_params_tank(gb_prb_params *p, int nr, int np);
/* The cavity defaults (velvor2ddvdbenchmark.f with its input.s: dt 2e-6,
 * r0 0, rmax 1, xx 1, Ra 1e6, Pr 0.71; tolcon 5e-6, sweep limit 500). */
void gb_prb_default_params_dvd(gb_prb_params *p, int nr, int np);

typedef struct gb_prb gb_prb;

/* Creates a device-resident instance on the current CUDA device; every
 * field starts at zero.  Replaces poissoninit (PRB:1724) plus the COMMON
 * storage of the fields.  nlev_out (may be NULL) receives the multigrid
 * level count, computed as poissoninit does (halvings of nr, capped at 4;
 * at 5 for the annulus). */
int gb_prb_create(const gb_prb_params *p, gb_prb **out, int *nlev_out);
int gb_prb_destroy(gb_prb *h);

/* Host <-> device copies of one field.  host is a column-major
 * (0:ld-1, 0:np) array with leading dimension ld >= nr+2 (ld = kr+1 = 291
 * for the reference's COMMON arrays); rows 0..nr+1 and columns 0..np move. */
int gb_prb_set_field(gb_prb *h, int field, const double *host, int ld);
int gb_prb_get_field(gb_prb *h, int field, double *host, int ld);
/* Device pointer and leading dimension of a field (for zero-copy callers). */
int gb_prb_field_device_ptr(gb_prb *h, int field, double **dev, int *ld);

/* One routine each, on the device-resident fields (replacing PRB:584-1721):
 *   first != 0: Cvorticity1 / temperature1 (forward first step),
 *   first == 0: Cvorticity / temperature (leapfrog + Robert filter). */
int gb_prb_cvorticity(gb_prb *h, int first);        /* PRB:584-778, PRB:786-1048 */
int gb_prb_temperature(gb_prb *h, int first);       /* PRB:1056-1212, PRB:1220-1443 */
int gb_prb_heat(gb_prb *h, double *trans1, double *trans2); /* PRB:1452-1500 */
int gb_prb_rhsv(gb_prb *h);                         /* PRB:1629-1676 */
int gb_prb_rhsu(gb_prb *h);                         /* PRB:1679-1721 */
/* which = 2: poisson2 on vel/velp/vrh (PRB:1796-1927);
 * which = 3: poisson3 on uel/uelp/urh (PRB:1930-2059).
 * Returns GB_OK, GB_MAXSWEEPS or GB_NAN; *sweeps gets the sweep count. */
int gb_prb_poisson(gb_prb *h, int which, int *sweeps);
/* CTAs that share one two-colour solve of this instance (FP64 or mixed):
 * 1 (the default: one CTA per equation) or 8 (the lines of a colour, the
 * residuals and the transfers of each level are spread over a cluster of 8
 * CTAs that meet at the hardware cluster barrier and reduce through
 * distributed shared memory).  Both give the same bits; the reference's
 * line order always uses one CTA.  The solve of a line is a dependent
 * chain that a cluster does not shorten: on the 129 x 65 layer the cluster
 * takes 0.95-1.02x the time of one CTA.  No counterpart in the reference
 * (its solves are serial). */
int gb_prb_set_solve_spread(gb_prb *h, int ctas);
/* update (PRB:1557-1626); *clamps (may be NULL) gets the number of
 * temperatures clamped, each of which the reference reports with
 * 'WARNING! Temp damped'. */
int gb_prb_update(gb_prb *h, long long *clamps);

/* nsteps steps of the main loop (PRB:341-388 for kt == 1, PRB:363-388
 * after), kt0 the index of the first.  nu (2*nsteps, may be NULL) receives
 * httrans, httrans2 per step (Nu = trans*(rmax-r0)/xx, PRB:386-388);
 * sweeps (2*nsteps, may be NULL) the v and u sweep counts.  The steps run
 * from a CUDA graph; the v and u solves run concurrently (the reference's
 * OpenMP sections, PRB:370-380). */
int gb_prb_step(gb_prb *h, int kt0, int nsteps, double *nu, int *sweeps);
/* The CUDA stream (cudaStream_t) every call on h runs on, for callers that
 * order their own work or time the steps with events on it. */
void *gb_prb_stream(gb_prb *h);
/* Asynchronous stepping for callers that keep many instances in flight
 * (the served loop): run_begin sizes the per-step history for up to
 * nsteps_total steps and resets the counters; run_enqueue queues nsteps
 * graph-replayed steps (kt0: index of the first, 1 = the forward step) on
 * the instance's stream and returns at once; run_query returns 1 when the
 * queued steps are done, 0 while they run (a negative status on an error);
 * run_end waits and copies the history of the first nsteps steps (as
 * gb_prb_step does) and the number of steps completed.  gb_prb_step is
 * run_begin + run_enqueue + run_end. */
int gb_prb_run_begin(gb_prb *h, int nsteps_total);
int gb_prb_run_enqueue(gb_prb *h, int kt0, int nsteps);
int gb_prb_run_query(gb_prb *h);
int gb_prb_run_end(gb_prb *h, int nsteps, double *nu, int *sweeps, int *steps_done);

/* Time-loop diagnostics on the device (PRB:404-493; velvor2dnewsch3.4.f:
 * 404-493 for the annulus), fused into the step's update kernel so the step
 * reads nothing back (a kernel of their own after the tank's and the
 * cavity's update: velvor2dhorconvtank.f:424-513, velvor2ddvdbenchmark.f:
 * 434-518, the same means and scans over columns k = 0..np).  Enabled, every graph-replayed step with kt >= 2
 * updates the running means of T^2, T, u^2 and v^2 over the block's steps
 * 2..kt (m = (1/(kt-1)) m (kt-2) + (1/(kt-1)) x; the reference keeps them
 * in weln, welp, Bp and vrms, PRB:408-416), and records the step's CFL
 * maxima max |u dt/dr| over rows 1..nr and max |v dt/(r dp)| over rows
 * 1..nr-1, r = 1 in the layer and r0 + (i - 1/2) dr in the annulus
 * (PRB:420-459).  A run that starts again at kt0 = 2 (a "more iterations"
 * block) starts the means again, as the reference's factor (kt-2) does.
 *
 * diag_enable: on != 0 allocates and zeroes the running means (again, when
 * already on); 0 frees them.  Graphs are rebuilt on the next run.
 * diag_zonal: out[3 i + c], i = 0..nr+1: the rows of zmtmtempvar.dat
 * (PRB:474-493): zonal-mean time variance of T, zonal rms of u, of v (sqrt;
 * the reference's **0.5d0 goes through libm pow and agrees to an ulp).
 * diag_mean: running mean q (0: T^2, 1: T, 2: u^2, 3: v^2) into host
 * (ld, np+1) column-major.
 * diag_cfl: cfl[2 s + 0..1], the u and v CFL maxima of step s of the last
 * run (0, 0 for a kt = 1 step and for steps that did not run). */
int gb_prb_diag_enable(gb_prb *h, int on);
int gb_prb_diag_zonal(gb_prb *h, double *out);
int gb_prb_diag_mean(gb_prb *h, int q, double *host, int ld);
int gb_prb_diag_cfl(gb_prb *h, int nsteps, double *cfl);

/* ------------------------------------------- gfortran-compatible drop-in */
/* These read/write the caller's COMMON blocks (declared by the Fortran main
 * program; the library carries weak references of the reference's sizes,
 * kr = 290, kp = 1610).  Other PARAMETER bounds: call gb_prb_bind_bounds
 * (or set GB300_PRB_KR / GB300_PRB_KP) before poissoninit_. */
void gb_prb_bind_bounds(int kr, int kp);
/* The smoother used by the drop-in symbols (default LEX, the reference's). */
void gb_prb_bind_smoother(int smoother);
/* Tolerance and sweep limit of the drop-in solves (default 2e-6, 500:
 * PRB:2086, PRB:1843; for the annulus 1e-5, 10000). */
void gb_prb_bind_tolerance(double tolcon, int maxsweeps);
/* Which driver the drop-in symbols serve: GB_PRB_LAYER (default) or
 * GB_PRB_ANNULUS (also selected by GB300_PRB_VARIANT=annulus).  The annulus
 * routines read r0 from COMMON /radius/ r0,rmax (weak reference radius_, or
 * gb_prb_bind_radius) and Re from /val/. */
void gb_prb_bind_variant(int variant);
void gb_prb_bind_radius(double *radius);
/* Explicit COMMON storage for callers that are not a Fortran main program:
 * sol1 = 9 arrays An..Cp, sol2 = thn,th,thp, sol3 = uel..welp, each
 * (kr+1)*(kp+1) doubles; num = {double dt,dr,dz,dp; int nr,nz,np};
 * val = {Ra, Re, Ptl, Gr}.  Pass NULLs to return to the weak symbols. */
void gb_prb_bind_common(double *sol1, double *sol2, double *sol3, void *num, double *val);

/* The 2D drivers' Fortran names; a translation unit that defines the 3D
 * annulus's drop-ins (include/gb300_r3d_fortran.h, same names with other
 * arguments) defines GB300_NO_PRB_DROPIN before including this header. */
#ifndef GB300_NO_PRB_DROPIN
void poissoninit_(int *nr, int *nz, int *np, double *dr, double *dz, double *dp,
                  int *nlev);                                   /* PRB:1724 */
void poisson2_(double *psi, double *psip, double *rhs, int *nr, int *nz, int *np,
               double *dr, double *dz, double *dp, int *nlev);  /* PRB:1796 */
void poisson3_(double *psi, double *psip, double *rhs, int *nr, int *nz, int *np,
               double *dr, double *dz, double *dp, int *nlev);  /* PRB:1930 */
void cvorticity1_(void);                                        /* PRB:584 */
void cvorticity_(void);                                         /* PRB:786 */
void temperature1_(void);                                       /* PRB:1056 */
void temperature_(void);                                        /* PRB:1220 */
void heat_(double *trans1, double *trans2);                     /* PRB:1452 */
void update_(void);                                             /* PRB:1557 */
void rhsv_(double *vrh);                                        /* PRB:1629 */
void rhsu_(double *urh);                                        /* PRB:1679 */
#endif
/* Status and sweep count of the last drop-in call on this process. */
int gb_prb_last_status(void);
int gb_prb_last_sweeps(void);

/* ------------------------------------- axisymmetric annulus (rotann2.f) */
/* The (r, z) meridional-plane rotating annulus of rotann2.f ("AXI"):
 * vorticity omega, streamfunction phi, swirl velocity v and temperature
 * theta on a vertex grid (0:nr, 0:nz), Dufort-Frankel transport with the
 * Arakawa Jacobian (:268-459), Thom wall vorticity (:497-539), inner-wall
 * heat flux (:468-487), and the streamfunction multigrid (:543-854:
 * alternating r-line / z-line Gauss-Seidel, nine-point restriction,
 * bilinear prolongation, plain V-cycle with nrel = 2, tolcon 1e-6, no STOP
 * after nvs = 10000 sweeps).  Fields are column-major (0:ld-1, 0:nz) with
 * ld >= nr+1 (the reference's ld is nrmax+1 = 129). */
enum gb_axi_field {
    GB_A_phi = 0, GB_A_omegn, GB_A_omeg, GB_A_omegp, GB_A_veln, GB_A_vel, GB_A_velp,
    GB_A_thetan, GB_A_theta, GB_A_thetap, GB_A_COUNT
};

typedef struct gb_axi_params {
    int nr, nz;          /* intervals in r and z (both even) */
    double dt, r0, rmax, zmax;
    double Ra, Re, Pr;   /* COMMON /val/ Ra, Re, Ptl */
    double tolcon;       /* max-norm residual tolerance (1e-6, rotann2.f:689) */
    int maxsweeps;       /* nvs (10000, rotann2.f:617) */
    int nrel;            /* relaxations per level visit (2, rotann2.f:618-619) */
    int smoother;        /* GB_SMOOTHER_LEX (the reference's order) or GB_SMOOTHER_ZEBRA */
    int precision;       /* GB_PRB_FP64 or GB_PRB_MIXED (FP32 V-cycles in FP64 defect correction) */
} gb_axi_params;

typedef struct gb_axi gb_axi;

/* Defaults of rotann2.f for an nr x nz grid (tolcon, nvs, nrel; LEX, FP64). */
void gb_axi_default_params(gb_axi_params *p, int nr, int nz);
/* Replaces poissoninit (rotann2.f:543) plus the COMMON storage; nlev_out
 * (may be NULL) receives the level count (halvings while nr and nz stay
 * even, capped at 6). */
int gb_axi_create(const gb_axi_params *p, gb_axi **out, int *nlev_out);
/* As gb_axi_create with the grid spacings given: a Fortran driver's own dr,
 * dz from COMMON /num/ (rotann2.f:22), used verbatim. */
int gb_axi_create_spacing(const gb_axi_params *p, double dr, double dz, gb_axi **out, int *nlev_out);
int gb_axi_destroy(gb_axi *h);
int gb_axi_set_field(gb_axi *h, int field, const double *host, int ld);
int gb_axi_get_field(gb_axi *h, int field, double *host, int ld);
int gb_axi_vorticity(gb_axi *h);                     /* rotann2.f:268-316 */
int gb_axi_velocity(gb_axi *h);                      /* rotann2.f:324-370 */
int gb_axi_temperature(gb_axi *h);                   /* rotann2.f:379-424 */
/* poisson(phi, omegn) (rotann2.f:598-666): GB_OK, or GB_MAXSWEEPS with phi
 * untouched (the reference returns silently there). */
int gb_axi_poisson(gb_axi *h, int *sweeps);
int gb_axi_update(gb_axi *h);                        /* rotann2.f:497-539 */
int gb_axi_heat(gb_axi *h, double *trans);           /* rotann2.f:468-487 */
/* nsteps steps of the main loop (rotann2.f:147-194), one CUDA graph per
 * step.  nu (nsteps, may be NULL) receives httrans = -r0 ln(r0/rmax) trans /
 * (zmax rmax) per step, sweeps (nsteps) the multigrid sweep counts.  The
 * reference stops when max |omega - omega_p|, |v - v_p| and |T - T_p| are
 * all below the REAL*4 1e-6 (:191); the steps stop there too, and
 * *steps_done (may be NULL) receives the number of steps taken. */
int gb_axi_step(gb_axi *h, int nsteps, double *nu, int *sweeps, int *steps_done);
void *gb_axi_stream(gb_axi *h);
/* Asynchronous stepping, as gb_prb_run_* (nu and sweeps: one per step). */
int gb_axi_run_begin(gb_axi *h, int nsteps_total);
int gb_axi_run_enqueue(gb_axi *h, int nsteps);
int gb_axi_run_query(gb_axi *h);
int gb_axi_run_end(gb_axi *h, int nsteps, double *nu, int *sweeps, int *steps_done);

/* ------------------------------------------------------ instance gangs */
/* Many device-resident instances of different grid sizes stepped together
 * (the served parameter sweep's continuous batching).  No counterpart in the
 * reference: its runs are separate processes chained by job scripts
 * (monashubuntudir_velvor2dhorconvtankdir/sleeprun.s:1-8).  Every phase of
 * a step (each transport routine, the heat flux, the right-hand sides, the
 * update, the bookkeeping) is one launch over the blocks of all members; the
 * multigrid solves of all members are one launch of one block per equation.
 * Each member runs exactly its own routines, so its fields, Nusselt history
 * and sweep counts are bit-identical to stepping it alone.
 *
 * Members: instances after gb_*_run_begin(h, total); nsteps_total[q] is
 * member q's total step count of the run: the gang stops a member whose
 * step index reaches it (its abort flag becomes 4, which gb_*_run_end
 * reports as success), so members of different lengths share the gang's
 * launches.  All members have the same precision.  A PRB gang runs leapfrog
 * steps only: enqueue each member's first step (kt = 1) on its own stream
 * first (gb_prb_run_enqueue); layer and annulus variants without
 * diagnostics.  An AXI gang takes uniform-grid annulus instances and all
 * of their steps.  Create waits for the members' own streams; enqueue queues
 * nsteps steps of every member (one CUDA graph launch per step) on `stream`
 * (NULL: the gang's own stream); query reports 1 when the gang's stream is
 * idle, 0 while it works, -status on error; collect each member with
 * gb_*_run_end once the gang is idle.  Destroy the gang (not the members)
 * when the membership changes. */
typedef struct gb_prb_gang gb_prb_gang;
int gb_prb_gang_create(gb_prb *const *members, const int *nsteps_total, int n, gb_prb_gang **out);
int gb_prb_gang_enqueue(gb_prb_gang *g, int nsteps, void *stream);
int gb_prb_gang_query(gb_prb_gang *g);
void *gb_prb_gang_stream(gb_prb_gang *g);
long long gb_prb_gang_launches_per_step(const gb_prb_gang *g);
/* CTAs per equation of a PRB gang's batched multigrid: 1 (the default) or
 * 8 (a cluster per equation, as gb_prb_set_solve_spread); the same bits
 * either way.  Takes effect at the next enqueue. */
int gb_prb_gang_set_solve_spread(gb_prb_gang *g, int ctas);
int gb_prb_gang_destroy(gb_prb_gang *g);
typedef struct gb_axi_gang gb_axi_gang;
int gb_axi_gang_create(gb_axi *const *members, const int *nsteps_total, int n, gb_axi_gang **out);
int gb_axi_gang_enqueue(gb_axi_gang *g, int nsteps, void *stream);
int gb_axi_gang_query(gb_axi_gang *g);
void *gb_axi_gang_stream(gb_axi_gang *g);
int gb_axi_gang_destroy(gb_axi_gang *g);

/* ---------------------------------------- 3D rotating annulus (rot3dmg.f) */
/* The 3D rotating annulus of rot3dmg.f ("R3D"): vorticity components A, B,
 * C and temperature by Dufort-Frankel with hybrid upwinding (:341-873), the
 * inner-wall heat flux (:882-909), wall vorticities and temperatures
 * (:964-1023), the right-hand sides (:1026-1150) and multigrid solves
 * (:1153-2344) of the three velocity components: r-, z- and phi-line
 * Gauss-Seidel per sweep, 27-point full weighting, trilinear prolongation,
 * plain V-cycle with nrel = 2, SOR 1.2, tolcon 1e-5, STOP beyond 500
 * sweeps.  Every field is a column-major (0:ld1-1, 0:ld2-1, 0:np) array,
 * ld1 >= nr+2 and ld2 >= nz+2 (the reference's are kr+1 = 34 and kz+1 =
 * 34, rot3dmg.f:23); element (i, j, k) at i + ld1*(j + ld2*k). */
enum gb_r3d_field {
    GB_R_An = 0, GB_R_A, GB_R_Ap, GB_R_Bn, GB_R_B, GB_R_Bp, GB_R_Cn, GB_R_C, GB_R_Cp,
    GB_R_thn, GB_R_th, GB_R_thp, GB_R_uel, GB_R_vel, GB_R_wel, GB_R_uelp, GB_R_velp, GB_R_welp,
    GB_R_urh, GB_R_vrh, GB_R_wrh, GB_R_COUNT
};

typedef struct gb_r3d_params {
    int nr, nz, np;           /* intervals in r, z and phi */
    double dt, r0, rmax, zmax;
    double Ra, Re, Gr, Pr;    /* COMMON /val/ Ra, Re, Ptl, Gr (rot3dmg.f:38) */
    double tolcon;            /* max-norm residual tolerance (1e-5, rot3dmg.f:1562) */
    double sor;               /* over-relaxation between sweeps (1.2, rot3dmg.f:1263) */
    int maxsweeps;            /* the reference STOPs beyond 500 sweeps (rot3dmg.f:1259) */
    int nrel;                 /* relaxations per level visit (2, rot3dmg.f:1237-1238) */
    int smoother;             /* GB_SMOOTHER_LEX: the reference's line order, run as wavefronts of
                                 independent lines; GB_SMOOTHER_ZEBRA: two colours of lines, the
                                 lines on one-sided boundary rows first within a colour (each
                                 colour one phase of the device solve) */
    int precision;            /* GB_PRB_FP64 or GB_PRB_MIXED (FP32 V-cycles in FP64 defect correction) */
    int variant;              /* GB_R3D_VERTICAL (rot3dmg.f) or GB_R3D_HORIZONTAL (rot3dmghor.f) */
} gb_r3d_params;

/* Which 3D annulus.
 *   GB_R3D_VERTICAL:   rot3dmg.f, the rotating annulus with a vertical axis.
 *   GB_R3D_HORIZONTAL: rot3dmghor.f, the annulus with its axis horizontal:
 *     the only body force in the vorticity updates is gravity across the
 *     axis, RHS2 = sin(theta) Gr Ptl thz (A, :477-479), cos(theta) Gr Ptl thz
 *     (B, :604-606), -(1/r) Gr Ptl cos(theta) thh - Gr Ptl sin(theta) thr
 *     (C, :747-749), theta = 6.283185307/np k with libm's sin and cos; the
 *     inner cylinder is hot (T = 1 at i = 0, 0 at i = nr+1, :1042-1043);
 *     heat gives both cylinders' fluxes over the band j = nz/2-3 .. nz/2+3
 *     (:913-945; nz >= 6); the V-cycles run without the whole-cycle
 *     over-relaxation and without the psip copies (:1287-1315; sor is
 *     ignored); the reference's tolerance is 1e-6 (:1599, :1798, :2051; set
 *     tolcon); Nusselt numbers nz/6 r0 ln(r0/rmax) trans1 / (zmax 2 pi) and
 *     nz/6 rmax ln(r0/rmax) trans2 / (zmax 2 pi) (:264-267). */
#define GB_R3D_VERTICAL   0
#define GB_R3D_HORIZONTAL 1

typedef struct gb_r3d gb_r3d;

/* Defaults of rot3dmg.f for an nr x nz x np grid (LEX, FP64). */
void gb_r3d_default_params(gb_r3d_params *p, int nr, int nz, int np);
/* Replaces poissoninit (rot3dmg.f:1153-1213) plus the COMMON storage;
 * nlev_out (may be NULL) receives the level count (halvings while nr and
 * nz halve exactly and both are >= 4, capped at 4).  np must be a multiple
 * of 2^nlev with at least 4 phi intervals on the coarsest level. */
int gb_r3d_create(const gb_r3d_params *p, gb_r3d **out, int *nlev_out);
/* As gb_r3d_create with the grid spacings given: a Fortran driver's own
 * dr, dz, dp from COMMON /num/ (rot3dmg.f:93-95), so that no spacing is
 * recomputed from r0, rmax, zmax (the routines never see zmax). */
int gb_r3d_create_spacing(const gb_r3d_params *p, double dr, double dz, double dp, gb_r3d **out, int *nlev_out);
int gb_r3d_destroy(gb_r3d *h);
int gb_r3d_set_field(gb_r3d *h, int field, const double *host, int ld1, int ld2);
int gb_r3d_get_field(gb_r3d *h, int field, double *host, int ld1, int ld2);
int gb_r3d_avorticity(gb_r3d *h);     /* rot3dmg.f:341-469 */
int gb_r3d_bvorticity(gb_r3d *h);     /* rot3dmg.f:477-593 */
int gb_r3d_cvorticity(gb_r3d *h);     /* rot3dmg.f:601-728 */
int gb_r3d_temperature(gb_r3d *h);    /* rot3dmg.f:736-873 */
int gb_r3d_heat(gb_r3d *h, double *trans1);   /* rot3dmg.f:882-909 */
/* heat(trans1, trans2) of rot3dmghor.f:913-945 (GB_R3D_HORIZONTAL; the
 * vertical annulus gives trans2 = 0). */
int gb_r3d_heat2(gb_r3d *h, double *trans1, double *trans2);
int gb_r3d_rhsw(gb_r3d *h);           /* rot3dmg.f:1026-1063 */
int gb_r3d_rhsv(gb_r3d *h);           /* rot3dmg.f:1066-1108 */
int gb_r3d_rhsu(gb_r3d *h);           /* rot3dmg.f:1111-1150 */
/* poisson1 (which = 1: wel, welp, wrh), poisson2 (2: vel), poisson3 (3: uel),
 * rot3dmg.f:1216-1540: GB_OK, GB_MAXSWEEPS (the reference STOPs), GB_NAN or
 * GB_TIMEOUT; *sweeps (may be NULL) receives the sweep count. */
int gb_r3d_poisson(gb_r3d *h, int which, int *sweeps);
int gb_r3d_update(gb_r3d *h);         /* rot3dmg.f:964-1023 */
/* nsteps steps of the main loop (rot3dmg.f:241-253).  nu (nsteps, may be
 * NULL) receives httrans = -r0 ln(r0/rmax) trans1 / (zmax 2 pi) per step
 * (:255), sweeps (3*nsteps, may be NULL) the w, v and u sweep counts.  A
 * failing solve ends the run (the reference STOPs); *steps_done (may be
 * NULL) receives the steps completed and the return value the status. */
int gb_r3d_step(gb_r3d *h, int nsteps, double *nu, int *sweeps, int *steps_done);
/* httrans2 of each step of the last gb_r3d_step run (GB_R3D_HORIZONTAL's
 * outer-cylinder Nusselt number, rot3dmghor.f:266-267; zero for the
 * vertical annulus); nu is the step run's httrans1 there. */
int gb_r3d_nu2(gb_r3d *h, int nsteps, double *nu2);
void *gb_r3d_stream(gb_r3d *h);
/* Polls a grid-wide barrier wait of the cooperative multigrid launches may
 * take before the solve gives up with GB_TIMEOUT (default 2^24, about
 * 1-2 s); 0 gives up at the first wait that is not already released.  The
 * reference has no counterpart (its solves run on host threads); the
 * context stays usable after a timeout, its fields hold whatever the
 * interrupted step left. */
int gb_r3d_set_wait_limit(gb_r3d *h, long long polls);
/* Grid barriers passed by the w, v and u solves (counts[0..2]) since the
 * context was created or last reset (reset != 0 clears them after reading),
 * and the number of blocks the solves launch with (*blocks, may be NULL; the
 * w and v solves of a step run side by side on half of them each).  With
 * gb_measure_grid_barrier this gives the barrier term of a step's latency.
 * No counterpart in the reference (its solves have no barriers). */
int gb_r3d_barrier_counts(gb_r3d *h, unsigned long long *counts, int *blocks, int reset);

/* ------------------------- stretched-grid streamfunction solve (rcsc.f) */
/* The multigrid of rcsc.f:1118-1444 on a non-uniform (r, z) grid: operator
 * psi_rr + psi_r / r - psi / r^2 + psi_zz with the per-level finite-
 * difference weights of grid.f (rcsc.f reads them from grid.f's file,
 * :82-97), pentadiagonal r-line and z-line Gauss-Seidel (tolcon 1e-6,
 * nrel 2), nine-point restriction that clears rows and columns 0 and n1 of
 * the coarse level in both directions, bilinear prolongation, plain V-cycle
 * from psi itself with no over-relaxation, no STOP after nvs = 10000
 * sweeps.  Level l (0-based here) is (n1 >> l) x (n2 >> l). */
typedef struct gb_str_level {
    int n1, n2;
    const double *r;     /* r(0..n1) of the level */
    const double *cr;    /* first-derivative weights of rows i = 1..n1-1 on (i-1, i, i+1): [3*(i-1) + k] */
    const double *crr;   /* second-derivative weights on (i-1..i+2) for i <= n1/2, else (i-2..i+1): [4*(i-1) + k] */
    const double *czz;   /* the same in z for rows j = 1..n2-1: [4*(j-1) + k] */
} gb_str_level;

typedef struct gb_str gb_str;

/* smoother: GB_SMOOTHER_LEX (the reference's line order, one thread) or
 * GB_SMOOTHER_ZEBRA (four colours of lines, index mod 4 = 1, 2, 3, 0; a line
 * reads the lines one and two away, so no line reads one of its colour). */
int gb_str_create(int nlev, const gb_str_level *levels, double tolcon, int maxsweeps, int nrel, int smoother,
                  gb_str **out);
/* poisson(psi, rhs) on host arrays (0:ld-1, 0:n2), ld >= n1+1: GB_OK (psi
 * updated), GB_MAXSWEEPS (psi untouched: the reference returns silently) or
 * GB_NAN; *sweeps (may be NULL) the sweep count. */
int gb_str_poisson(gb_str *h, double *psi, const double *rhs, int ld, int *sweeps);
int gb_str_destroy(gb_str *h);

/* ------------------------- axisymmetric annulus on a stretched grid */
/* rotann2.f's annulus (the gb_axi_* entry points above, same fields and
 * time loop) on a non-uniform (r, z) grid.  rotann2.f itself is uniform;
 * the reference's stretched-grid method is rcsc.f's (weights from grid.f),
 * and this mode takes from it: every derivative of rotann2.f's vorticity,
 * velocity and temperature with grid.f's level-1 weights (first
 * derivatives on (i-1, i, i+1), second derivatives on four points switching
 * orientation at n/2, rcsc.f's dum* functions), the Dufort-Frankel centre
 * crr_c + cr_2/r + czz_c in place of -2/dr^2 - 2/dz^2 (rcsc.f's cnr, cnz),
 * the Arakawa sum over the local metric 3 (r(i+1) - r(i-1)) (z(j+1) -
 * z(j-1)), the temperature's mirrored top and bottom rows with their wall
 * spacing, Thom wall vorticity with the wall spacings (rcsc.f update,
 * :706-751), the heat flux with five-point one-sided d/dr weights at the
 * inner wall (hw, from grid.f's fdif on r(0..4)) and the trapezoid rule in
 * z, and rcsc.f's stretched multigrid (gb_str above, whose operator is
 * rotann2.f's) for the streamfunction, in FP64 or mixed precision (FP32
 * V-cycles inside FP64 defect correction).  On a uniform grid the transport
 * equals rotann2.f's to rounding. */
typedef struct gb_axi_grid {
    int nlev;                       /* multigrid levels */
    const gb_str_level *levels;     /* grid.f's levels (level 1 first: r, cr, crr, czz) */
    const double *z;                /* level-1 z(0..nz) */
    const double *cz;               /* level-1 d/dz weights of rows j = 1..nz-1 on (j-1, j, j+1): [3*(j-1) + k] */
    const double *hw;               /* 5 weights of d/dr at r(0) on r(0..4) */
} gb_axi_grid;
int gb_axi_create_stretched(const gb_axi_params *p, const gb_axi_grid *g, gb_axi **out, int *nlev_out);

/* ------------------------------------------------ batched banded solvers */
/* nlines independent systems with the same n; line l's element j sits at
 * base + l*line_stride + j*elem_stride in each array.  Device pointers.
 * The matrices may differ per line.  Inputs are preserved (unlike the
 * reference, whose solvers overwrite them).
 *   tdma:  PRB:3046-3064 (a sub, b diag, c super)
 *   ptdma: PRB:3066-3116 (periodic: a(1) couples to x(n), c(n) to x(1))
 *   pdma:  PRB:3118-3164 (a 2nd sub, b sub, c diag, d super, e 2nd super) */
int gb_tdma_batch(const double *a, const double *b, const double *c, const double *r,
                  double *y, int n, int nlines, long long line_stride, long long elem_stride,
                  void *stream);
int gb_ptdma_batch(const double *a, const double *b, const double *c, const double *r,
                   double *y, int n, int nlines, long long line_stride, long long elem_stride,
                   void *stream);
int gb_pdma_batch(const double *a, const double *b, const double *c, const double *d,
                  const double *e, const double *r, double *x, int n, int nlines,
                  long long line_stride, long long elem_stride, void *stream);

/* The same pentadiagonal batch without any allocation, for callers that
 * cannot allocate device memory when they call: a Fortran driver whose
 * storage is all static (COMMON blocks sized by PARAMETER at compile time)
 * and which has no way to handle an allocation failure in the middle of a
 * time step, or a program that has handed the device to its own memory
 * pool or budget (a server admitting work against a fixed device-memory
 * budget) and must not let the CUDA runtime grow its own pool.  No
 * counterpart in the reference (its pdma works on arrays the caller owns).
 * Limit: 5*n*nlines <= GB_PDMA_NOALLOC_MAX_DOUBLES (4 MiB of scratch that
 * every GPU loading the library holds until exit); larger requests return
 * GB_ERR_INVALID without launching.  The first call on each device looks up
 * the scratch array's device address; the address is kept for the life of
 * the process, so a cudaDeviceReset after that first call is not
 * supported.  Each call waits
 * for its stream before it returns (its status covers the kernel), so the
 * calls of one host thread never overlap one another; all calls share the
 * scratch, so calls from different host threads that overlap on the GPU
 * race.  Results are identical to gb_pdma_batch. */
#define GB_PDMA_NOALLOC_MAX_DOUBLES 524288u
int gb_pdma_batch_noalloc(const double *a, const double *b, const double *c, const double *d,
                          const double *e, const double *r, double *x, int n, int nlines,
                          long long line_stride, long long elem_stride, void *stream);

/* ------------------------------------------------- batched Poisson solve */
/* Many independent Dirichlet problems nabla^2 psi = f on n x n vertex grids
 * (n = 2^m + 1, 3 <= n <= 8193) of the unit square, psi = 0 on the boundary;
 * V(nu1,nu2) red-black Gauss-Seidel cycles with full-weighting restriction
 * and bilinear prolongation (the transfer operators of rotann2.f:755-854)
 * until ||f - A psi||_2 <= rtol ||f||_2.  Problem p occupies n[p]^2
 * doubles, row-major, starting at offset sum_{q<p} n[q]^2. */
#define GB_BATCH_FP64  0   /* plain FP64 V-cycles */
#define GB_BATCH_MIXED 1   /* FP32 inner V-cycles inside defect correction; the
                              outer residual in float-pair arithmetic (~48-bit
                              significands: f and psi held as FP32 hi + lo
                              pairs during the solve), psi returned in FP64 */
#define GB_BATCH_MIXED_F64OUTER 2  /* FP32 inner V-cycles inside FP64 defect
                              correction: the outer residual r = f - A psi, its
                              norm and the update psi += e in FP64 on the
                              caller's arrays; r rounded to FP32 is the inner
                              cycles' right-hand side */

typedef struct gb_batch gb_batch;

int gb_batch_create(int nprob, const int *n, int precision, int nu1, int nu2, double rtol,
                    int max_cycles, gb_batch **out);

/* The tunables of a batched solve.  gb_batch_create uses local_n 65, fuse 2
 * (1 for GB_BATCH_FP64), inner 1 and the graph execution mode.  local_n,
 * fuse and exec change only the speed (every combination gives the same
 * bits); nu1, nu2 and inner change the iteration itself. */
typedef struct {
    int nu1, nu2;     /* red-black sweeps before / after the coarse correction */
    int inner;        /* FP32 V-cycles per defect-correction step (1 for GB_BATCH_FP64) */
    int local_n;      /* levels with n <= local_n are solved by one block per problem in
                         shared memory: 33, 65 or 129 (at most 65 for GB_BATCH_FP64) */
    int fuse;         /* red-black sweeps fused into one tile pass: 1 or 2 (halo 2*fuse,
                         two more where the pass also restricts) */
    int exec;         /* GB_BATCH_EXEC_GRAPH or GB_BATCH_EXEC_PERSISTENT */
    double ms;        /* autotuner output: measured milliseconds per solve */
} gb_batch_tuning;

/* Creates a handle with the given tunables (t->ms is ignored). */
int gb_batch_create_tuned(int nprob, const int *n, int precision, double rtol, int max_cycles,
                          const gb_batch_tuning *t, gb_batch **out);

/* Autotuner (no counterpart in the reference, whose multigrid has no
 * tunables beyond PARAMETERs).  Times every candidate configuration of a
 * size mix on the current device with CUDA events on a stream of its own:
 * one untimed solve, then `reps` timed solves of d_f (device, packed, the
 * caller's right-hand side: convergence depends on it) into d_psi (device
 * scratch of the same size), and keeps the fastest time to solution.
 * Candidates: inner 2..5 (mixed; 1 for GB_BATCH_FP64) x local_n 33, 65, 129
 * x fuse 1, 2 x graph / persistent execution, at the given nu1, nu2; with
 * tune_nu != 0 also nu in (1,1), (1,2), (2,1), (2,2), (3,3).  A candidate
 * whose solve does not return GB_OK is skipped.  The winner goes to *best;
 * table (table_cap entries, may be NULL) receives every candidate timed and
 * *table_len (may be NULL) their number.  cache_path (may be NULL: then the
 * environment variable GB300_BATCH_TUNE_CACHE, else no file) names a text
 * file of earlier winners keyed by device name, SM count, precision, nu,
 * rtol, max_cycles and the multiset of sizes; a hit returns the cached
 * winner without timing (*from_cache = 1, may be NULL) and a miss appends
 * the new winner.  Also answers repeated calls within a process from memory. */
int gb_batch_autotune(int nprob, const int *n, int precision, int nu1, int nu2, int tune_nu, double rtol,
                      int max_cycles, const double *d_f, double *d_psi, int reps, const char *cache_path,
                      gb_batch_tuning *best, gb_batch_tuning *table, int table_cap, int *table_len,
                      int *from_cache);
int gb_batch_destroy(gb_batch *b);
/* Mixed solves only: V-cycles per outer (defect-correction) iteration,
 * 1..16 (default 1).  With k > 1 the outer residual, its norm and the
 * update of psi run once per k inner cycles, and convergence is tested
 * every k cycles. */
int gb_batch_set_inner_cycles(gb_batch *b, int inner);
/* How a solve is executed.  GRAPH (the default): one kernel per level
 * operation, one CUDA graph per outer iteration.  PERSISTENT (devices with
 * cooperative launch): one launch runs every level of every cycle of every
 * problem until all have converged, with bounded grid-wide barriers between
 * the level operations (a barrier that waits too long ends the solve with
 * GB_TIMEOUT).  Both run the same operations and give identical results. */
#define GB_BATCH_EXEC_GRAPH      0
#define GB_BATCH_EXEC_PERSISTENT 1
int gb_batch_set_exec(gb_batch *b, int mode);
/* Total doubles of the packed f / psi arrays. */
long long gb_batch_total_points(const gb_batch *b);
/* Polls a grid-wide barrier wait of the persistent execution mode may take
 * before the solve gives up with GB_TIMEOUT (default 2^24, about 1-2 s);
 * 0 gives up at the first wait that is not already released.  The handle
 * stays usable after a timeout. */
int gb_batch_set_wait_limit(gb_batch *b, long long polls);
/* Device-resident solve: d_f, d_psi device pointers (packed).  cycles and
 * relres (host, nprob each, may be NULL) receive per-problem V-cycle counts
 * and final relative residuals.  Returns GB_OK, GB_MAXSWEEPS, GB_NAN (a
 * problem's residual norm is a NaN or infinite: that problem stops at once)
 * or, in persistent mode, GB_TIMEOUT.  A mixed
 * solve keeps psi as float pairs in d_psi's own memory while it runs; d_psi
 * holds FP64 values again when the call returns (it synchronises stream). */
int gb_batch_solve_device(gb_batch *b, const double *d_f, double *d_psi, int *cycles,
                          double *relres, void *stream);
/* Host-buffer solve (copies in and out inside the call).  The first call
 * allocates a device staging buffer of 2 x total doubles that the handle
 * keeps until gb_batch_destroy. */
int gb_batch_solve_host(gb_batch *b, const double *h_f, double *h_psi, int *cycles,
                        double *relres);
/* Pipelined host-buffer solves for a stream of calls: call k's h_f is
 * uploaded on its own stream while call k-1 solves, and call k-1's solution
 * is downloaded on another while call k solves.  A submit queues call k's
 * upload, then runs the solve of the call submitted before it and returns
 * that solve's status (GB_OK when there was none); gb_batch_drain runs the
 * last submitted solve, waits for every download and returns its status.
 * Call k's cycles and relres are written when call k+1's submit (or the
 * drain) returns, its h_psi when the drain returns or call k+2's submit
 * has; h_f must stay unchanged until call k+1's submit returns.  Host
 * buffers should be page-locked for the copies to overlap.  The first
 * submit allocates 4 x total doubles that the handle keeps. */
int gb_batch_submit_host(gb_batch *b, const double *h_f, double *h_psi, int *cycles, double *relres);
int gb_batch_drain(gb_batch *b);
/* Number of kernel launches the last solve issued. */
long long gb_batch_last_launches(const gb_batch *b);
/* Times every launch of the finest-level smoothing kernel with CUDA events
 * on the solve's stream during later solves (enable = 0 stops). */
int gb_batch_profile(gb_batch *b, int enable);
/* Accumulated time (ms), launch count and algorithmic bytes of the
 * finest-level down operation (sweeps + residual + restriction; in
 * persistent mode: of the whole-solve launches); reset != 0 clears all
 * profile counters. */
int gb_batch_profile_read(gb_batch *b, double *ms, long long *launches, double *alg_bytes, int reset);
/* The same per operation kind (graph mode): 0 smoothing, 1 smoothing +
 * residual + restriction, 2 prolongation + smoothing, 4 outer passes after
 * a solve's first, 7 the first outer pass of each solve (it reads f alone);
 * finest level only, except the outer passes. */
#define GB_BATCH_OP_SMOOTH      0
#define GB_BATCH_OP_DOWN        1
#define GB_BATCH_OP_UP          2
#define GB_BATCH_OP_OUTER       4
#define GB_BATCH_OP_OUTER_FIRST 7
int gb_batch_profile_read_kind(gb_batch *b, int kind, double *ms, long long *launches, double *alg_bytes);

/* ------------------------------------------------------ device probes */
/* Issue rates of FP64 and FP32 fused multiply-adds on the current device
 * (instructions per second, every SM busy); the FP64 figure is the peak the
 * FP64-bound kernels are measured against. */
int gb_measure_issue_rates(double *fp64_fma_per_s, double *fp32_fma_per_s);
/* Time of one bounded grid barrier (microseconds) in a cooperative launch of
 * `blocks` x `threads` that does nothing else, averaged over `nbarriers`
 * barriers after one warm-up launch: the per-phase cost a persistent solve of
 * that launch shape pays on top of its work.  GB_ERR_INVALID when the blocks
 * cannot all be resident.  No counterpart in the reference (a latency probe
 * of this library's own barrier). */
int gb_measure_grid_barrier(int blocks, int threads, int nbarriers, double *us_per_barrier);
/* Compares the line solvers' division by a stored reciprocal (a product and
 * two fused multiply-adds that round to the IEEE quotient) with the hardware
 * FP64 division on n_random seeded operand pairs over the normal range
 * (random significands, near-exact quotients, small integers, signed zero
 * dividends); *mismatches gets the count of differing bit patterns.  No
 * counterpart in the reference (a check of this library's arithmetic). */
int gb_check_division(long long n_random, unsigned long long seed, long long *mismatches);
/* Compares the batched solver's integer-pipe float <-> double conversions
 * with the hardware conversions on the current device: every float bit
 * pattern through float -> double, and n_random seeded double bit patterns
 * (whole exponent range, the float range and its edges, rounding ties and
 * their neighbours) through double -> float.  The counts of differing
 * results go to *mismatches_f2d and *mismatches_d2f (two NaNs agree). */
int gb_check_conversions(long long n_random, unsigned long long seed, long long *mismatches_f2d,
                         long long *mismatches_d2f);

#ifdef __cplusplus
}
#endif
#endif /* GB300_CONVECTION_H */
