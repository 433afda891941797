/*
 * gb300_axi_fortran.h -- gfortran-compatible drop-in entry points for the
 * subroutines of rotann2.f (the axisymmetric rotating annulus): poissoninit_,
 * vorticity_, velocity_, temperature_, poisson_, update_, heat_.
 *
 * Library: codesthesis_dir_gb300/_build/libgb300axi.so (its own library:
 * the names clash with the 2D and 3D drivers' drop-ins).  A rotann2.f main
 * program links against it in place of its own subroutines.
 *
 * COMMON blocks (rotann2.f:19-23) are the caller's: gfortran's sol1_, sol2_,
 * num_, val_, radius_ (weak references), or bound explicitly with
 * gb_axi_bind_common.  Arrays are (0:nrmax, 0:nzmax) with nrmax = nzmax =
 * 128 (rotann2.f:9) unless gb_axi_bind_bounds or GB300_AXI_NRMAX /
 * GB300_AXI_NZMAX say otherwise.  Each call copies the fields to the
 * device, runs the routine there, and copies them back; parts of the arrays
 * outside (0:nr, 0:nz) are never touched.  Nothing exits the process: the
 * status of the last call is gb_axi_last_status().
 */
#ifndef GB300_AXI_FORTRAN_H
#define GB300_AXI_FORTRAN_H

#ifdef __cplusplus
extern "C" {
#endif

void poissoninit_(int *nr, int *nz, double *dr, double *dz);   /* rotann2.f:543 */
void vorticity_(void);                                          /* rotann2.f:268-316 */
void velocity_(void);                                           /* rotann2.f:324-370 */
void temperature_(void);                                        /* rotann2.f:379-424 */
/* poisson(psi, rhs): the streamfunction multigrid (rotann2.f:598-892),
 * called as poisson(phi, omegn) by the main program (:149). */
void poisson_(double *psi, double *rhs);
void update_(void);                                             /* rotann2.f:497-539 */
void heat_(double *trans);                                      /* rotann2.f:468-487 */

/* Configuration, callable from C before poissoninit_. */
void gb_axi_bind_bounds(int nrmax, int nzmax);
/* sol1 = phi,omegn,omeg,omegp,veln,vel,velp and sol2 = thetan,theta,thetap,
 * each (nrmax+1)*(nzmax+1) doubles; num points to { double dr, dz; int nr,
 * nz; double dt; } (COMMON /num/), val to { cf1, cf2, cf3, cf4, Ra, Re, Ptl },
 * radius to { r0 }.  Pass NULLs to return to the weak symbols. */
void gb_axi_bind_common(double *sol1, double *sol2, void *num, double *val, double *radius);
/* GB_SMOOTHER_LEX (default, the reference's line order) or GB_SMOOTHER_ZEBRA. */
void gb_axi_bind_smoother(int smoother);
/* GB_PRB_FP64 (default) or GB_PRB_MIXED. */
void gb_axi_bind_precision(int precision);
/* tolcon (1e-6, rotann2.f:689) and the sweep limit (nvs = 10000, :617). */
void gb_axi_bind_tolerance(double tolcon, int maxsweeps);
/* Status of the last call (GB_OK, GB_MAXSWEEPS, GB_NAN, GB_TIMEOUT, GB_ERR_*)
 * and the sweep count of the last poisson_. */
int gb_axi_last_status(void);
int gb_axi_last_sweeps(void);

#ifdef __cplusplus
}
#endif
#endif /* GB300_AXI_FORTRAN_H */
