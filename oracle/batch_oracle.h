/*
 * CPU oracle for the batched Dirichlet Poisson solve (many independent
 * problems of uneven size, V(nu1,nu2) red-black Gauss-Seidel cycles).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of tests/, smoke() and the CPU legs
 * of bench.py.  No reference driver solves this workload; its FP64 grid
 * transfers equal rotann2.f's corser and finer run through the translator
 * tests/golden/f77.py (tests/test_reference_runs.py), while the smoother
 * and residual below have no reference counterpart;
 * the grid transfer operators restate the vertex-centred multigrid of
 * rotann2.f (corser rotann2.f:755-801, finer rotann2.f:803-854) with the
 * radial terms dropped, and the smoother is point red-black Gauss-Seidel.
 *
 * Problem p is an n x n vertex grid (n = 2^m + 1 >= 3) on the unit square,
 * h = 1/(n-1), psi = 0 on the boundary, discretising
 *     (psi_E + psi_W + psi_N + psi_S - 4 psi) / h^2 = f.
 * Arrays are row-major (x fastest), problem p starting at offset[p].
 *
 * Arithmetic is written with explicit fma()/fmaf() exactly where the GPU
 * kernels use __fma_rn/__fmaf_rn, and nowhere else (-ffp-contract=off), so
 * the two agree bit for bit except for the order of the norm reductions.
 */
#ifndef BATCH_ORACLE_H
#define BATCH_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_BATCH_FP64  0
#define ORC_BATCH_MIXED 1   /* FP32 inner V-cycles, float-pair outer residual */
#define ORC_BATCH_MIXED_F64OUTER 2   /* FP32 inner V-cycles, FP64 outer residual, norm and update */

/* Solve every problem.  psi is overwritten (initial guess zero).  cycles[p]
 * receives the V-cycles taken, relres[p] the final ||f - A psi||_2/||f||_2.
 * inner: FP32 V-cycles per defect-correction step (mixed only).
 * Returns 0; 1 if any problem hit max_cycles; 2 if any problem's residual
 * norm was not finite (that problem stops at once).  Uses OpenMP threads
 * over problems when built with -fopenmp. */
int orc_batch_solve(int nprob, const int *n, const long long *offset,
                    const double *f, double *psi, int nu1, int nu2,
                    double rtol, int max_cycles, int precision, int inner,
                    int *cycles, double *relres);

/* Building blocks on one grid, exposed for unit tests. */
void orc_rb_sweep64(int n, double *psi, const double *f);
void orc_residual64(int n, const double *psi, const double *f, double *r);
void orc_restrict64(int n, const double *r, double *fc);
void orc_prolong_add64(int n, const double *ec, double *psi);
double orc_resnorm64(int n, const double *psi, const double *f);

#ifdef __cplusplus
}
#endif
#endif
