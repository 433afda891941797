/*
 * CPU oracle for the batched Dirichlet Poisson solve.  TEST INFRASTRUCTURE
 * ONLY (see batch_oracle.h).  No reference program solves this workload.
 *
 * Transfer operators follow rotann2.f: full-weighting restriction summed in
 * the order of corser (rotann2.f:773-785) and bilinear prolongation with the
 * corner sum of finer (rotann2.f:821-850), followed by the correction add
 * (rotann2.f:852-858).  The smoother is point red-black Gauss-Seidel.
 *
 * Every multiply by h^2, 1/h^2, 0.25 or 0.0625 is by a power of two, so the
 * fma() calls below round exactly as the unfused expressions would; they
 * are written to mirror the GPU kernels one operation for one operation.
 */
#include "batch_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define DEFINE_GRID_OPS(T, SFX, FMA)                                               \
    static void rb_half_##SFX(int n, T *psi, const T *f, T h2, int color)           \
    {                                                                               \
        for (int j = 1; j <= n - 2; ++j) {                                          \
            int i0 = (((1 + j) & 1) == color) ? 1 : 2;                              \
            for (int i = i0; i <= n - 2; i += 2) {                                  \
                size_t c = (size_t)j * n + i;                                       \
                T s = (psi[c - 1] + psi[c + 1]) + (psi[c - n] + psi[c + n]);        \
                psi[c] = FMA(-h2, f[c], s) * (T)0.25;                               \
            }                                                                       \
        }                                                                           \
    }                                                                               \
    static void residual_##SFX(int n, const T *psi, const T *f, T *r, T ih2)        \
    {                                                                               \
        for (int j = 1; j <= n - 2; ++j)                                            \
            for (int i = 1; i <= n - 2; ++i) {                                      \
                size_t c = (size_t)j * n + i;                                       \
                T s = (psi[c - 1] + psi[c + 1]) + (psi[c - n] + psi[c + n]);        \
                T lap = FMA((T)-4.0, psi[c], s);                                    \
                r[c] = FMA(-ih2, lap, f[c]);                                        \
            }                                                                       \
    }                                                                               \
    static void restrict_##SFX(int n, const T *r, T *fc)                            \
    {                                                                               \
        int nc = (n - 1) / 2 + 1;                                                   \
        for (int j = 1; j <= nc - 2; ++j)                                           \
            for (int i = 1; i <= nc - 2; ++i) {                                     \
                size_t c = (size_t)(2 * j) * n + (size_t)(2 * i);                   \
                T t = r[c];                                                         \
                t = t * (T)2.0 + r[c + 1] + r[c - 1];                               \
                t = t + r[c + n] + r[c - n];                                        \
                t = t * (T)2.0 + r[c + 1 + n] + r[c - 1 - n];                       \
                t = t + r[c + 1 - n] + r[c - 1 + n];                                \
                fc[(size_t)j * nc + i] = t * (T)0.0625;                             \
            }                                                                       \
    }                                                                               \
    static void prolong_add_##SFX(int n, const T *ec, T *psi)                       \
    {                                                                               \
        int nc = (n - 1) / 2 + 1;                                                   \
        for (int j = 1; j <= n - 2; ++j)                                            \
            for (int i = 1; i <= n - 2; ++i) {                                      \
                int i1 = i / 2, j1 = j / 2;                                         \
                const T *e = ec + (size_t)j1 * nc + i1;                             \
                T v;                                                                \
                if ((i & 1) == 0) {                                                 \
                    if ((j & 1) == 0) v = e[0];                                     \
                    else v = (e[0] + e[nc]) * (T)0.5;                               \
                } else {                                                            \
                    if ((j & 1) == 0) v = (e[0] + e[1]) * (T)0.5;                   \
                    else {                                                          \
                        T t = e[0] + e[nc + 1];                                     \
                        t = t + e[nc] + e[1];                                       \
                        v = t * (T)0.25;                                            \
                    }                                                               \
                }                                                                   \
                psi[(size_t)j * n + i] = psi[(size_t)j * n + i] + v;                \
            }                                                                       \
    }                                                                               \
    static void vcycle_##SFX(int nlev, const int *nl, T **psi, T **f, T **r,        \
                             int nu1, int nu2, int l)                               \
    {                                                                               \
        int n = nl[l];                                                              \
        T h = (T)1.0 / (T)(n - 1);                                                  \
        T h2 = h * h;                                                               \
        if (l == nlev - 1) {                                                        \
            rb_half_##SFX(n, psi[l], f[l], h2, 0);                                  \
            return;                                                                 \
        }                                                                           \
        for (int s = 0; s < nu1; ++s) {                                             \
            rb_half_##SFX(n, psi[l], f[l], h2, 0);                                  \
            rb_half_##SFX(n, psi[l], f[l], h2, 1);                                  \
        }                                                                           \
        residual_##SFX(n, psi[l], f[l], r[l], (T)1.0 / h2);                         \
        restrict_##SFX(n, r[l], f[l + 1]);                                          \
        memset(psi[l + 1], 0, sizeof(T) * (size_t)nl[l + 1] * nl[l + 1]);           \
        vcycle_##SFX(nlev, nl, psi, f, r, nu1, nu2, l + 1);                         \
        prolong_add_##SFX(n, psi[l + 1], psi[l]);                                   \
        for (int s = 0; s < nu2; ++s) {                                             \
            rb_half_##SFX(n, psi[l], f[l], h2, 0);                                  \
            rb_half_##SFX(n, psi[l], f[l], h2, 1);                                  \
        }                                                                           \
    }

DEFINE_GRID_OPS(double, 64, fma)
DEFINE_GRID_OPS(float, 32, fmaf)

void orc_rb_sweep64(int n, double *psi, const double *f)
{
    double h = 1.0 / (double)(n - 1);
    rb_half_64(n, psi, f, h * h, 0);
    rb_half_64(n, psi, f, h * h, 1);
}

void orc_residual64(int n, const double *psi, const double *f, double *r)
{
    double h = 1.0 / (double)(n - 1);
    memset(r, 0, sizeof(double) * (size_t)n * n);
    residual_64(n, psi, f, r, 1.0 / (h * h));
}

void orc_restrict64(int n, const double *r, double *fc)
{
    int nc = (n - 1) / 2 + 1;
    memset(fc, 0, sizeof(double) * (size_t)nc * nc);
    restrict_64(n, r, fc);
}

void orc_prolong_add64(int n, const double *ec, double *psi) { prolong_add_64(n, ec, psi); }

static double sumsq_interior(int n, const double *a)
{
    double s = 0.0;
    for (int j = 1; j <= n - 2; ++j)
        for (int i = 1; i <= n - 2; ++i) {
            double x = a[(size_t)j * n + i];
            s = fma(x, x, s);
        }
    return s;
}

double orc_resnorm64(int n, const double *psi, const double *f)
{
    double *r = (double *)calloc((size_t)n * n, sizeof(double));
    orc_residual64(n, psi, f, r);
    double s = sumsq_interior(n, r);
    free(r);
    return sqrt(s);
}

static int levels_of(int n, int *nl)
{
    int L = 0;
    while (1) {
        nl[L++] = n;
        if (n <= 3) break;
        n = (n - 1) / 2 + 1;
    }
    return L;
}

/* Float pairs (hi, lo) for the mixed solve's outer residual, the same
 * operations in the same order as the device: two_sum (Knuth, TAOCP vol. 2,
 * 4.2.2), the accurate pair sum of Dekker (1971) as the QD library's ieee_add
 * arranges it, and scalings by powers of two (exact). */
typedef struct {
    float hi, lo;
} fpair;

static void two_sum(float a, float b, float *s, float *e)
{
    *s = a + b;
    const float bb = *s - a;
    *e = (a - (*s - bb)) + (b - bb);
}

static void fast_two_sum(float a, float b, float *s, float *e)
{
    *s = a + b;
    *e = b - (*s - a);
}

static fpair fp_add(fpair a, fpair b)
{
    float s, e, t, f;
    two_sum(a.hi, b.hi, &s, &e);
    two_sum(a.lo, b.lo, &t, &f);
    e = e + t;
    fast_two_sum(s, e, &s, &e);
    e = e + f;
    fast_two_sum(s, e, &s, &e);
    fpair r = {s, e};
    return r;
}

static fpair fp_add_f(fpair a, float b)
{
    float s, e;
    two_sum(a.hi, b, &s, &e);
    e = e + a.lo;
    fast_two_sum(s, e, &s, &e);
    fpair r = {s, e};
    return r;
}

static fpair fp_scale(fpair a, float p)
{
    fpair r = {a.hi * p, a.lo * p};
    return r;
}

static int solve_one(int n, const double *f, double *psi, int nu1, int nu2, double rtol,
                     int max_cycles, int precision, int inner, int *cycles_out, double *relres_out)
{
    int nl[32];
    int L = levels_of(n, nl);
    size_t tot = 0;
    for (int l = 0; l < L; ++l) tot += (size_t)nl[l] * nl[l];
    const size_t nn = (size_t)n * n;
    memset(psi, 0, sizeof(double) * nn);
    double fn = sqrt(sumsq_interior(n, f));
    double *r64 = (double *)calloc(nn, sizeof(double));
    int cycles = 0, status = 0;
    double rn = fn;
    if (precision == ORC_BATCH_FP64) {
        double *pool = (double *)calloc(tot * 3, sizeof(double));
        double *P[32], *F[32], *R[32];
        size_t off = 0;
        for (int l = 0; l < L; ++l) {
            P[l] = pool + off; F[l] = pool + tot + off; R[l] = pool + 2 * tot + off;
            off += (size_t)nl[l] * nl[l];
        }
        P[0] = psi;
        memcpy(F[0], f, sizeof(double) * nn);
        for (;;) {
            if (cycles > 0) rn = orc_resnorm64(n, psi, f);
            if (!isfinite(rn)) { status = 2; break; }
            if (rn <= rtol * fn) break;
            if (cycles >= max_cycles) { status = 1; break; }
            vcycle_64(L, nl, P, F, R, nu1, nu2, 0);
            ++cycles;
        }
        free(pool);
    } else if (precision == ORC_BATCH_MIXED_F64OUTER) {
        /* FP64 defect correction around FP32 inner V-cycles: the outer
         * residual in FP64 (the plain solve's operations), rounded to FP32 as
         * the inner right-hand side; psi += e in FP64, e widened exactly */
        float *pool = (float *)calloc(tot * 3, sizeof(float));
        float *P[32], *F[32], *R[32];
        size_t off = 0;
        for (int l = 0; l < L; ++l) {
            P[l] = pool + off; F[l] = pool + tot + off; R[l] = pool + 2 * tot + off;
            off += (size_t)nl[l] * nl[l];
        }
        const double h = 1.0 / (double)(n - 1);
        const double ih2 = 1.0 / (h * h);
        for (;;) {
            double s = 0.0;
            for (int j = 1; j <= n - 2; ++j)
                for (int i = 1; i <= n - 2; ++i) {
                    const size_t c = (size_t)j * n + i;
                    const double sum = (psi[c - 1] + psi[c + 1]) + (psi[c - n] + psi[c + n]);
                    const double lap = fma(-4.0, psi[c], sum);
                    const double r = fma(-ih2, lap, f[c]);
                    F[0][c] = (float)r;
                    s = fma(r, r, s);
                }
            rn = sqrt(s);
            if (!isfinite(rn)) { status = 2; break; }
            if (rn <= rtol * fn) break;
            if (cycles >= max_cycles) { status = 1; break; }
            memset(P[0], 0, sizeof(float) * nn);
            for (int k = 0; k < inner; ++k) vcycle_32(L, nl, P, F, R, nu1, nu2, 0);
            for (int j = 1; j <= n - 2; ++j)
                for (int i = 1; i <= n - 2; ++i) {
                    const size_t c = (size_t)j * n + i;
                    psi[c] = psi[c] + (double)P[0][c];
                }
            cycles += inner;
        }
        free(pool);
    } else {
        float *pool = (float *)calloc(tot * 3, sizeof(float));
        float *P[32], *F[32], *R[32];
        size_t off = 0;
        for (int l = 0; l < L; ++l) {
            P[l] = pool + off; F[l] = pool + tot + off; R[l] = pool + 2 * tot + off;
            off += (size_t)nl[l] * nl[l];
        }
        /* f and psi as float pairs; 1/h^2 = 4^m is exact in FP32 (n = 2^m + 1) */
        fpair *fq = (fpair *)malloc(nn * sizeof(fpair));
        fpair *pq = (fpair *)calloc(nn, sizeof(fpair));
        float *r32 = (float *)calloc(nn, sizeof(float));
        for (size_t c = 0; c < nn; ++c) {
            fq[c].hi = (float)f[c];
            fq[c].lo = (float)(f[c] - (double)fq[c].hi);
        }
        const float hs = 1.0f / (float)(n - 1);
        const float ih2 = 1.0f / (hs * hs);
        int first = 1;
        for (;;) {
            /* outer residual r = f - A psi in pair arithmetic; its high part
             * is the FP32 right-hand side and, widened, the norm's term */
            double s = 0.0;
            for (int j = 1; j <= n - 2; ++j)
                for (int i = 1; i <= n - 2; ++i) {
                    const size_t c = (size_t)j * n + i;
                    const fpair sum = fp_add(fp_add(pq[c - 1], pq[c + 1]), fp_add(pq[c - n], pq[c + n]));
                    const fpair lap = fp_add(sum, fp_scale(pq[c], -4.0f));
                    const fpair r = fp_add(fq[c], fp_scale(lap, -ih2));
                    r32[c] = r.hi;
                    const double x = (double)r.hi;
                    s = fma(x, x, s);
                }
            rn = sqrt(s);
            if (first) fn = rn;   /* psi = 0: the norm of f's high parts */
            first = 0;
            if (!isfinite(rn)) { status = 2; break; }
            if (rn <= rtol * fn) break;
            if (cycles >= max_cycles) { status = 1; break; }
            /* inner FP32 V-cycles on A e = r, e0 = 0 */
            memcpy(F[0], r32, sizeof(float) * nn);
            memset(P[0], 0, sizeof(float) * nn);
            for (int k = 0; k < inner; ++k) vcycle_32(L, nl, P, F, R, nu1, nu2, 0);
            for (int j = 1; j <= n - 2; ++j)
                for (int i = 1; i <= n - 2; ++i) {
                    size_t c = (size_t)j * n + i;
                    pq[c] = fp_add_f(pq[c], P[0][c]);
                }
            cycles += inner;
        }
        for (size_t c = 0; c < nn; ++c) psi[c] = (double)pq[c].hi + (double)pq[c].lo;
        free(fq);
        free(pq);
        free(r32);
        free(pool);
    }
    free(r64);
    *cycles_out = cycles;
    *relres_out = (fn > 0.0) ? rn / fn : 0.0;
    return status;
}

int orc_batch_solve(int nprob, const int *n, const long long *offset, const double *f,
                    double *psi, int nu1, int nu2, double rtol, int max_cycles,
                    int precision, int inner, int *cycles, double *relres)
{
    if (inner < 1) inner = 1;
    int status = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(max : status)
    for (int p = 0; p < nprob; ++p) {
        const int st = solve_one(n[p], f + offset[p], psi + offset[p], nu1, nu2, rtol, max_cycles,
                            precision, inner, &cycles[p], &relres[p]);
        if (st > status) status = st;
    }
    return status;
}
