/*
 * gfortran-compatible drop-in entry points for the subroutines of rot3dmg.f
 * (the 3D rotating annulus), in their own shared library libgb300r3d.so:
 * they share names with the 2D drivers' subroutines (cvorticity_,
 * temperature_, heat_, update_, rhsv_, rhsu_, poissoninit_, poisson2_,
 * poisson3_), whose drop-ins live in libgb300conv.so.  A rot3dmg.f main
 * program links -lgb300r3d (which itself depends on libgb300conv.so)
 * instead of compiling the subroutines; everything is passed by reference.
 *
 * The argument-less routines read and write the caller's COMMON blocks
 * (rot3dmg.f:33-42) /sol1/ An,A,Ap,Bn,B,Bp,Cn,C,Cp, /sol2/ thn,th,thp,
 * /sol3/ uel,vel,wel,uelp,velp,welp, /num/ dt,dr,dz,dp,nr,nz,np, /val/
 * Ra,Re,Ptl,Gr and /radius/ r0,rmax, found through weak references to
 * gfortran's sol1_ ... radius_ or bound with gb_r3d_bind_common.  Arrays are
 * (0:kr,0:kz,0:kp) with the reference's PARAMETER bounds kr = kz = 33,
 * kp = 160 (rot3dmg.f:23) unless gb_r3d_bind_bounds or GB300_R3D_KR /
 * GB300_R3D_KZ / GB300_R3D_KP say otherwise.  Each call copies the fields the
 * Fortran routine reads to one process-wide device instance, runs the
 * routine's kernels and copies back the fields it writes; the untouched
 * parts of every array round-trip unchanged.
 */
#ifndef GB300_R3D_FORTRAN_H
#define GB300_R3D_FORTRAN_H

#ifdef __cplusplus
extern "C" {
#endif

/* poissoninit(nr,nz,np,dr,dz,dp,nlev), rot3dmg.f:1153-1213: nlev by the
 * reference rule; creates the device instance. */
void poissoninit_(int *nr, int *nz, int *np, double *dr, double *dz, double *dp, int *nlev);
/* poisson1/2/3(psi,psip,rhs,nr,nz,np,dr,dz,dp,nlev), rot3dmg.f:1216-1540
 * (w, v and u).  Beyond 500 sweeps the reference STOPs: here psi and psip
 * are left as they were and gb_r3d_last_status() returns 1. */
void poisson1_(double *psi, double *psip, double *rhs, int *nr, int *nz, int *np, double *dr, double *dz,
               double *dp, int *nlev);
void poisson2_(double *psi, double *psip, double *rhs, int *nr, int *nz, int *np, double *dr, double *dz,
               double *dp, int *nlev);
void poisson3_(double *psi, double *psip, double *rhs, int *nr, int *nz, int *np, double *dr, double *dz,
               double *dp, int *nlev);
void avorticity_(void);               /* rot3dmg.f:341-469 */
void bvorticity_(void);               /* rot3dmg.f:477-593 */
void cvorticity_(void);               /* rot3dmg.f:601-728 */
void temperature_(void);              /* rot3dmg.f:736-873 */
/* rot3dmg.f:882-909 heat(trans1); with the horizontal variant bound,
 * rot3dmghor.f:913-945 heat(trans1, trans2) (only then is trans2 read). */
void heat_(double *trans1, double *trans2);
void update_(void);                   /* rot3dmg.f:964-1023 */
void rhsw_(double *wrh);              /* rot3dmg.f:1026-1063 */
void rhsv_(double *vrh);              /* rot3dmg.f:1066-1108 */
void rhsu_(double *urh);              /* rot3dmg.f:1111-1150 */

/* Configuration, callable from C before poissoninit_. */
void gb_r3d_bind_bounds(int kr, int kz, int kp);
/* num points to { double dt, dr, dz, dp; int nr, nz, np; } (COMMON /num/),
 * val to { Ra, Re, Ptl, Gr }, radius to { r0, rmax }. */
void gb_r3d_bind_common(double *sol1, double *sol2, double *sol3, void *num, double *val, double *radius);
/* GB_SMOOTHER_LEX (default, the reference's line order) or GB_SMOOTHER_ZEBRA. */
void gb_r3d_bind_smoother(int smoother);
/* GB_PRB_FP64 (default) or GB_PRB_MIXED. */
void gb_r3d_bind_precision(int precision);
/* GB_R3D_VERTICAL (default, rot3dmg.f) or GB_R3D_HORIZONTAL (rot3dmghor.f,
 * same subroutine names; also GB300_R3D_VARIANT=horizontal): its tolerance
 * defaults to 1e-6. */
void gb_r3d_bind_variant(int variant);
/* tolcon (1e-5) and the sweep limit (500) of the solves. */
void gb_r3d_bind_tolerance(double tolcon, int maxsweeps);
/* Status of the last call (GB_OK, GB_MAXSWEEPS, GB_NAN, GB_TIMEOUT, GB_ERR_*)
 * and the sweep count of the last solve. */
int gb_r3d_last_status(void);
int gb_r3d_last_sweeps(void);

#ifdef __cplusplus
}
#endif
#endif /* GB300_R3D_FORTRAN_H */
