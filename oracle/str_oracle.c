/*
 * CPU oracle: restatement of grid.f's coefficient build and rcsc.f's
 * stretched-grid streamfunction multigrid ("STR").  TEST INFRASTRUCTURE
 * ONLY (the checker; never linked into the product).  PARITY PINNED: its
 * spacings, levels and weight tables equal grid.f's own main program, and
 * its multigrid equals rcsc.f's poisson on those tables, bit for bit, both
 * run through the translator tests/golden/f77.py
 * (tests/test_reference_runs.py); also checked by its own invariants (exact
 * weights on polynomials, second-order convergence on stretched grids,
 * agreement of the two line orders).
 *
 * Every expression keeps the reference's left-to-right order; x**2 is x*x.
 * Build with -ffp-contract=off (see Makefile).
 */
#include "str_oracle.h"
#include "prb_oracle.h"   /* orc_pdma: rcsc.f:1572-1619 is the same elimination */

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* grid.f                                                                   */
/* ------------------------------------------------------------------------ */

/* grid.f:737-790 (r; z is the same code at :792-842).  h is 1-based. */
int orc_str_spacing_gef(int n, double lo, double hi, double dist, double gef, double d1, double *h)
{
    if (gef <= 0.0) {
        for (int i = 1; i <= n; ++i) h[i] = (hi - lo) / (double)n;
        return 0;
    }
    h[1] = d1;
    double t = h[1];
    int imax = -1;
    for (int i = 2; i <= n / 2; ++i) {
        h[i] = h[i - 1] * gef;
        t = t + h[i];
        if (t > dist) {
            imax = i;
            t = t - h[i];
            break;
        }
    }
    if (imax < 0) return -1;           /* too many grid points in GEF region */
    if (2 * imax - 2 > n) return -1;   /* grid points exceeded */
    const double over = hi - lo - 2.0 * t;
    for (int i = imax; i <= n - imax + 1; ++i) h[i] = over / (double)(n - 2 * imax + 2);
    for (int i = n - imax + 1; i <= n; ++i) h[i] = h[n - i + 1];
    return 0;
}

/* level, grid.f:859-924 (without the interactive change of nlev). */
int orc_str_levels(orc_str_grid_t *g, int n1, int n2, const double *hr1, const double *hz1, double r0,
                   double zmin, int maxlev)
{
    memset(g, 0, sizeof(*g));
    int nlev = 0, itest = n1, itest2 = n1, jtest = n2, jtest2 = n2;
    for (int i = 2; i <= 8; ++i) {
        itest /= 2;
        jtest /= 2;
        if (itest * 2 - itest2 == 0 && jtest * 2 - jtest2 == 0) {
            if (itest2 >= 4 && jtest2 >= 4) nlev++;
            itest2 = itest;
            jtest2 = jtest;
        } else {
            break;
        }
    }
    if (nlev > 6) nlev = 6;
    if (maxlev > 0 && nlev > maxlev) nlev = maxlev;
    if (nlev < 1) return 0;
    g->nlev = nlev;
    for (int l = 1; l <= nlev; ++l) {
        const int a = n1 * 2 / (1 << l), b = n2 * 2 / (1 << l);
        g->n1[l] = a;
        g->n2[l] = b;
        g->hr[l] = (double *)calloc((size_t)a + 1, sizeof(double));
        g->hz[l] = (double *)calloc((size_t)b + 1, sizeof(double));
        g->r[l] = (double *)calloc((size_t)a + 1, sizeof(double));
        g->z[l] = (double *)calloc((size_t)b + 1, sizeof(double));
        g->cr[l] = (double *)calloc(3 * (size_t)a + 3, sizeof(double));
        g->crr[l] = (double *)calloc(4 * (size_t)a + 4, sizeof(double));
        g->cz[l] = (double *)calloc(3 * (size_t)b + 3, sizeof(double));
        g->czz[l] = (double *)calloc(4 * (size_t)b + 4, sizeof(double));
        g->r[l][0] = r0;
        for (int i = 1; i <= a; ++i) {
            g->hr[l][i] = l == 1 ? hr1[i] : g->hr[l - 1][2 * i] + g->hr[l - 1][2 * i - 1];
            g->r[l][i] = g->r[l][i - 1] + g->hr[l][i];
        }
        g->z[l][0] = zmin;
        for (int j = 1; j <= b; ++j) {
            g->hz[l][j] = l == 1 ? hz1[j] : g->hz[l - 1][2 * j] + g->hz[l - 1][2 * j - 1];
            g->z[l][j] = g->z[l][j - 1] + g->hz[l][j];
        }
    }
    return nlev;
}

void orc_str_grid_free(orc_str_grid_t *g)
{
    for (int l = 0; l < STR_MAXLEV; ++l) {
        free(g->hr[l]);
        free(g->hz[l]);
        free(g->r[l]);
        free(g->z[l]);
        free(g->cr[l]);
        free(g->crr[l]);
        free(g->cz[l]);
        free(g->czz[l]);
    }
    memset(g, 0, sizeof(*g));
}

/* gausse, grid.f:1034-1115.  a(j,i) is row i, column j of the system;
 * b(k,i) is right-hand side k of row i (n+2 of them); x(k,i) the solution. */
#define GA(j, i) a[(size_t)((j) - 1) + (size_t)n * (size_t)((i) - 1)]
#define GB(k, i) b[(size_t)((k) - 1) + (size_t)(n + 2) * (size_t)((i) - 1)]
#define GX(k, i) x[(size_t)((k) - 1) + (size_t)(n + 2) * (size_t)((i) - 1)]
static int gausse(double *a, double *b, double *x, int n)
{
    if (n == 1) {
        GX(1, 1) = GB(1, 1) / GA(1, 1);
        GX(2, 1) = GB(2, 1) / GA(1, 1);
        GX(3, 1) = GB(3, 1) / GA(1, 1);
        return 0;
    }
    for (int k = 1; k <= n - 1; ++k) {
        int kpvt = k;
        const int kp1 = k + 1;
        for (int i = kp1; i <= n; ++i)
            if (fabs(GA(k, kpvt)) < fabs(GA(k, i))) kpvt = i;
        if (fabs(GA(k, kpvt)) == 0.0) return -1;
        if (kpvt != k) {
            for (int j = k; j <= n; ++j) {
                const double save = GA(j, k);
                GA(j, k) = GA(j, kpvt);
                GA(j, kpvt) = save;
            }
            for (int j = 1; j <= n + 2; ++j) {
                const double save = GB(j, k);
                GB(j, k) = GB(j, kpvt);
                GB(j, kpvt) = save;
            }
        }
        for (int i = k + 1; i <= n; ++i) {
            const double q = -GA(k, i) / GA(k, k);
            GA(k, i) = 0.0;
            for (int j = k + 1; j <= n; ++j) GA(j, i) = GA(j, i) + q * GA(j, k);
            for (int j = 1; j <= n + 2; ++j) GB(j, i) = GB(j, i) + q * GB(j, k);
        }
    }
    for (int j = 1; j <= n + 2; ++j) GX(j, n) = GB(j, n) / GA(n, n);
    for (int i = n - 1; i >= 1; --i)
        for (int k = 1; k <= n + 2; ++k) {
            double s = 0.0;
            for (int j = i + 1; j <= n; ++j) s = s + GA(j, i) * GX(k, j);
            GX(k, i) = (GB(k, i) - s) / GA(i, i);
        }
    return 0;
}
#undef GA
#undef GB
#undef GX

/* fdif, grid.f:926-1032 (nans = 0). */
int orc_str_fdif(int nx, int nref, int k, const double *xr, double *w)
{
    const int n = nx;
    double x[64], a[64 * 64], b[66 * 64], ainv[66 * 64];
    if (nx < 1 || nx > 32) return -1;
    for (int i = 1; i <= nx; ++i) x[i] = xr[k - nref + i];
#define A(i, j) a[(size_t)((i) - 1) + (size_t)n * (size_t)((j) - 1)]
#define B(i, j) b[(size_t)((i) - 1) + (size_t)(n + 2) * (size_t)((j) - 1)]
#define AI(i, j) ainv[(size_t)((i) - 1) + (size_t)(n + 2) * (size_t)((j) - 1)]
    for (int j = 1; j <= nx; ++j) {
        double temp = 1.0;
        const double h = x[j] - x[nref];
        A(1, j) = 1.0;
        AI(1, j) = 0.0;
        B(1, j) = 0.0;
        for (int i = 2; i <= nx + 2; ++i) {
            if (j == nref) temp = 0.0;
            else temp = temp * h / (double)(i - 1);
            if (i <= nx) A(i, j) = temp;
            AI(i, j) = 0.0;
            if (i <= nx) B(i, j) = 0.0;
            else B(i, j) = -temp;
        }
    }
    for (int j = 1; j <= nx; ++j) {
        AI(j, j) = 1.0;
        B(j, j) = 1.0;
    }
    if (gausse(a, b, ainv, n) != 0) return -1;
    for (int d = 0; d < nx; ++d)
        for (int p = 0; p < nx; ++p) w[d * nx + p] = AI(p + 1, d + 1);
#undef A
#undef B
#undef AI
    return 0;
}

/* grid.f:178-243 */
int orc_str_coefficients(orc_str_grid_t *g)
{
    double w[16];
    for (int l = 1; l <= g->nlev; ++l) {
        const int n1 = g->n1[l], n2 = g->n2[l];
        for (int i = 1; i <= n1 - 1; ++i) {
            if (orc_str_fdif(3, 2, i, g->r[l], w)) return -1;
            for (int q = 0; q < 3; ++q) g->cr[l][3 * (i - 1) + q] = w[1 * 3 + q];
            if (orc_str_fdif(4, i <= n1 / 2 ? 2 : 3, i, g->r[l], w)) return -1;
            for (int q = 0; q < 4; ++q) g->crr[l][4 * (i - 1) + q] = w[2 * 4 + q];
        }
        for (int j = 1; j <= n2 - 1; ++j) {
            if (orc_str_fdif(3, 2, j, g->z[l], w)) return -1;
            for (int q = 0; q < 3; ++q) g->cz[l][3 * (j - 1) + q] = w[1 * 3 + q];
            if (orc_str_fdif(4, j <= n2 / 2 ? 2 : 3, j, g->z[l], w)) return -1;
            for (int q = 0; q < 4; ++q) g->czz[l][4 * (j - 1) + q] = w[2 * 4 + q];
        }
    }
    const int n1 = g->n1[1], n2 = g->n2[1];
    if (orc_str_fdif(3, 1, 0, g->r[1], w)) return -1;
    for (int q = 0; q < 3; ++q) g->cr0[q] = w[3 + q];
    if (orc_str_fdif(3, 3, n1, g->r[1], w)) return -1;
    for (int q = 0; q < 3; ++q) g->crn[q] = w[3 + q];
    if (orc_str_fdif(3, 1, 0, g->z[1], w)) return -1;
    for (int q = 0; q < 3; ++q) g->cz0[q] = w[3 + q];
    if (orc_str_fdif(3, 3, n2, g->z[1], w)) return -1;
    for (int q = 0; q < 3; ++q) g->czn[q] = w[3 + q];
    return 0;
}

/* ------------------------------------------------------------------------ */
/* rcsc.f multigrid                                                          */
/* ------------------------------------------------------------------------ */

#define PX(i, j) m->psif[(size_t)(i) + (size_t)ld * (size_t)(j)]

int orc_str_mg_init(orc_str_mg_t *m, const orc_str_grid_t *g, int nlev)
{
    memset(m, 0, sizeof(*m));
    m->g = g;
    m->nlev = nlev > 0 && nlev < g->nlev ? nlev : g->nlev;
    const int n1 = g->n1[1], n2 = g->n2[1];
    const int nmax = (n1 > n2 ? n1 : n2) + 1;
    m->ld = nmax;
    const size_t big = (size_t)nmax * (size_t)nmax;
    m->psif = (double *)calloc(big, sizeof(double));
    m->rc = (double *)calloc(big, sizeof(double));
    for (int l = 1; l <= m->nlev; ++l) {
        const size_t sz = (size_t)(g->n1[l] + 1) * (size_t)(g->n2[l] + 1);
        m->v[l] = (double *)calloc(sz, sizeof(double));
        m->f[l] = (double *)calloc(sz, sizeof(double));
    }
    m->tolcon = 1e-6;
    m->nrel = 2;
    m->maxsweeps = 10000;
    m->mode = 0;
    return m->psif && m->rc ? 0 : -1;
}

void orc_str_mg_free(orc_str_mg_t *m)
{
    free(m->psif);
    free(m->rc);
    for (int l = 0; l < STR_MAXLEV; ++l) {
        free(m->v[l]);
        free(m->f[l]);
    }
    memset(m, 0, sizeof(*m));
}

static void unpack(orc_str_mg_t *m, const double *src, double *dst, int l)
{
    const int n1 = m->g->n1[l], n2 = m->g->n2[l], ld = m->ld;
    for (int j = 0; j <= n2; ++j)
        for (int i = 0; i <= n1; ++i) dst[(size_t)i + (size_t)ld * j] = src[(size_t)i + (size_t)(n1 + 1) * j];
}

static void pack(orc_str_mg_t *m, const double *src, double *dst, int l)
{
    const int n1 = m->g->n1[l], n2 = m->g->n2[l], ld = m->ld;
    for (int j = 0; j <= n2; ++j)
        for (int i = 0; i <= n1; ++i) dst[(size_t)i + (size_t)(n1 + 1) * j] = src[(size_t)i + (size_t)ld * j];
}

/* r-line j (rcsc.f:1225-1261) */
static void rline(orc_str_mg_t *m, int klev, const double *rf, int j, double *w)
{
    const orc_str_grid_t *g = m->g;
    const int ld = m->ld, n1 = g->n1[klev], n2 = g->n2[klev];
    const double *r = g->r[klev], *cr = g->cr[klev], *crr = g->crr[klev], *czz = g->czz[klev];
    const int n = n1 - 1;
    double *pa = w, *pb = w + n, *pc = w + 2 * n, *pd = w + 3 * n, *pe = w + 4 * n, *pr = w + 5 * n, *ps = w + 6 * n;
#define CR(i, k) cr[3 * ((i) - 1) + (k) - 1]
#define CRR(i, k) crr[4 * ((i) - 1) + (k) - 1]
#define CZZ(j, k) czz[4 * ((j) - 1) + (k) - 1]
    for (int i = 1; i <= n1 - 1; ++i) {
        const int q = i - 1;
        if (i <= n1 / 2) {
            pa[q] = 0.0;
            pb[q] = CRR(i, 1) + CR(i, 1) / r[i];
            pc[q] = CRR(i, 2) + CR(i, 2) / r[i] - 1.0 / (r[i] * r[i]);
            pd[q] = CRR(i, 3) + CR(i, 3) / r[i];
            pe[q] = CRR(i, 4);
        } else {
            pa[q] = CRR(i, 1);
            pb[q] = CRR(i, 2) + CR(i, 1) / r[i];
            pc[q] = CRR(i, 3) + CR(i, 2) / r[i] - 1.0 / (r[i] * r[i]);
            pd[q] = CRR(i, 4) + CR(i, 3) / r[i];
            pe[q] = 0.0;
        }
        if (j <= n2 / 2) {
            pc[q] = pc[q] + CZZ(j, 2);
            pr[q] = -(CZZ(j, 1) * PX(i, j - 1) + CZZ(j, 3) * PX(i, j + 1) + CZZ(j, 4) * PX(i, j + 2)) +
                    rf[(size_t)i + (size_t)ld * j];
        } else {
            pc[q] = pc[q] + CZZ(j, 3);
            pr[q] = -(CZZ(j, 1) * PX(i, j - 2) + CZZ(j, 2) * PX(i, j - 1) + CZZ(j, 4) * PX(i, j + 1)) +
                    rf[(size_t)i + (size_t)ld * j];
        }
    }
    orc_pdma(pa, pb, pc, pd, pe, pr, ps, n);
    for (int i = 1; i <= n1 - 1; ++i) PX(i, j) = ps[i - 1];
}

/* z-line i (rcsc.f:1263-1298) */
static void zline(orc_str_mg_t *m, int klev, const double *rf, int i, double *w)
{
    const orc_str_grid_t *g = m->g;
    const int ld = m->ld, n1 = g->n1[klev], n2 = g->n2[klev];
    const double *r = g->r[klev], *cr = g->cr[klev], *crr = g->crr[klev], *czz = g->czz[klev];
    const int n = n2 - 1;
    double *pa = w, *pb = w + n, *pc = w + 2 * n, *pd = w + 3 * n, *pe = w + 4 * n, *pr = w + 5 * n, *ps = w + 6 * n;
    for (int j = 1; j <= n2 - 1; ++j) {
        const int q = j - 1;
        if (j <= n2 / 2) {
            pa[q] = 0.0;
            pb[q] = CZZ(j, 1);
            pc[q] = CZZ(j, 2) - 1.0 / (r[i] * r[i]);
            pd[q] = CZZ(j, 3);
            pe[q] = CZZ(j, 4);
        } else {
            pa[q] = CZZ(j, 1);
            pb[q] = CZZ(j, 2);
            pc[q] = CZZ(j, 3) - 1.0 / (r[i] * r[i]);
            pd[q] = CZZ(j, 4);
            pe[q] = 0.0;
        }
        if (i <= n1 / 2) {
            pc[q] = pc[q] + CRR(i, 2) + CR(i, 2) / r[i];
            pr[q] = -(CRR(i, 1) * PX(i - 1, j) + CRR(i, 3) * PX(i + 1, j) + CRR(i, 4) * PX(i + 2, j) +
                      (CR(i, 1) * PX(i - 1, j) + CR(i, 3) * PX(i + 1, j)) / r[i]) +
                    rf[(size_t)i + (size_t)ld * j];
        } else {
            pc[q] = pc[q] + CRR(i, 3) + CR(i, 2) / r[i];
            pr[q] = -(CRR(i, 1) * PX(i - 2, j) + CRR(i, 2) * PX(i - 1, j) + CRR(i, 4) * PX(i + 1, j) +
                      (CR(i, 1) * PX(i - 1, j) + CR(i, 3) * PX(i + 1, j)) / r[i]) +
                    rf[(size_t)i + (size_t)ld * j];
        }
    }
    orc_pdma(pa, pb, pc, pd, pe, pr, ps, n);
    for (int j = 1; j <= n2 - 1; ++j) PX(i, j) = ps[j - 1];
}

/* relax, rcsc.f:1197-1341 */
void orc_str_relax(orc_str_mg_t *m, int nrel, int klev, int *nconv)
{
    const orc_str_grid_t *g = m->g;
    const int ld = m->ld, n1 = g->n1[klev], n2 = g->n2[klev];
    const double *r = g->r[klev], *cr = g->cr[klev], *crr = g->crr[klev], *czz = g->czz[klev];
    *nconv = 0;
    double *rf = (double *)calloc((size_t)ld * (size_t)ld, sizeof(double));
    unpack(m, m->f[klev], rf, klev);
    unpack(m, m->v[klev], m->psif, klev);
    const int nmax = (n1 > n2 ? n1 : n2) + 2;
    double *w = (double *)malloc(sizeof(double) * 7 * (size_t)nmax);
    double resmax = 0.0;
    int anynan = 0;
    for (int irel = 1; irel <= nrel; ++irel) {
        if (m->mode == 0) {
            for (int j = 1; j <= n2 - 1; ++j) rline(m, klev, rf, j, w);
            for (int i = 1; i <= n1 - 1; ++i) zline(m, klev, rf, i, w);
        } else {
            /* four colours (index mod 4 = 1, 2, 3, 0): a line reads the lines
             * one and two away, never one of its own colour */
            for (int c = 1; c <= 4; ++c)
                for (int j = 1; j <= n2 - 1; ++j)
                    if ((j & 3) == (c & 3)) rline(m, klev, rf, j, w);
            for (int c = 1; c <= 4; ++c)
                for (int i = 1; i <= n1 - 1; ++i)
                    if ((i & 3) == (c & 3)) zline(m, klev, rf, i, w);
        }
        resmax = 0.0;
        anynan = 0;
        for (int i = 1; i <= n1 - 1; ++i)
            for (int j = 1; j <= n2 - 1; ++j) {
                double temp;
                if (i <= n1 / 2)
                    temp = CRR(i, 1) * PX(i - 1, j) + CRR(i, 2) * PX(i, j) + CRR(i, 3) * PX(i + 1, j) +
                           CRR(i, 4) * PX(i + 2, j) +
                           (CR(i, 1) * PX(i - 1, j) + CR(i, 2) * PX(i, j) + CR(i, 3) * PX(i + 1, j)) / r[i] -
                           PX(i, j) / (r[i] * r[i]);
                else
                    temp = CRR(i, 1) * PX(i - 2, j) + CRR(i, 2) * PX(i - 1, j) + CRR(i, 3) * PX(i, j) +
                           CRR(i, 4) * PX(i + 1, j) +
                           (CR(i, 1) * PX(i - 1, j) + CR(i, 2) * PX(i, j) + CR(i, 3) * PX(i + 1, j)) / r[i] -
                           PX(i, j) / (r[i] * r[i]);
                if (j <= n2 / 2)
                    temp = temp + CZZ(j, 1) * PX(i, j - 1) + CZZ(j, 2) * PX(i, j) + CZZ(j, 3) * PX(i, j + 1) +
                           CZZ(j, 4) * PX(i, j + 2);
                else
                    temp = temp + CZZ(j, 1) * PX(i, j - 2) + CZZ(j, 2) * PX(i, j - 1) + CZZ(j, 3) * PX(i, j) +
                           CZZ(j, 4) * PX(i, j + 1);
                temp = rf[(size_t)i + (size_t)ld * j] - temp;
                m->rc[(size_t)i + (size_t)ld * j] = temp;
                temp = fabs(temp);
                if (temp != temp) anynan = 1;
                if (temp > resmax) resmax = temp;
            }
    }
#undef CR
#undef CRR
#undef CZZ
    free(w);
    free(rf);
    pack(m, m->psif, m->v[klev], klev);
    if (klev == 1) m->last_resmax = anynan ? NAN : resmax;
    if (klev == 1 && resmax < m->tolcon) *nconv = 1;
}

/* corser, rcsc.f:1343-1390: nine-point restriction; rows and columns 0 and
 * n1 of the coarse level cleared in both directions (n1 for both, as in
 * rotann2.f). */
void orc_str_corser(orc_str_mg_t *m, int klev)
{
    const orc_str_grid_t *g = m->g;
    const int ld = m->ld, n1 = g->n1[klev], n2 = g->n2[klev];
    const int n1c = g->n1[klev + 1], n2c = g->n2[klev + 1];
    const size_t big = (size_t)ld * (size_t)ld;
    double *rf = (double *)malloc(sizeof(double) * big), *psic = (double *)calloc(big, sizeof(double));
    double *rc = m->rc;
    (void)n1;
    (void)n2;
    memcpy(rf, rc, sizeof(double) * big);
#define RF(i, j) rf[(size_t)(i) + (size_t)ld * (size_t)(j)]
    for (int i = 1; i <= n1c - 1; ++i)
        for (int j = 1; j <= n2c - 1; ++j) {
            const int ii = i + i, jj = j + j;
            double temp = RF(ii, jj);
            temp = temp * 2.0 + RF(ii + 1, jj) + RF(ii - 1, jj);
            temp = temp + RF(ii, jj + 1) + RF(ii, jj - 1);
            temp = temp * 2.0 + RF(ii + 1, jj + 1) + RF(ii - 1, jj - 1);
            temp = temp + RF(ii + 1, jj - 1) + RF(ii - 1, jj + 1);
            temp = temp / 16.0;
            rc[(size_t)i + (size_t)ld * j] = temp;
        }
#undef RF
    for (int i = 0; i <= n1c; ++i) {
        rc[(size_t)i] = 0.0;
        rc[(size_t)i + (size_t)ld * n1c] = 0.0;
    }
    for (int j = 0; j <= n1c; ++j) {
        rc[(size_t)ld * j] = 0.0;
        rc[(size_t)n1c + (size_t)ld * j] = 0.0;
    }
    pack(m, rc, m->f[klev + 1], klev + 1);
    pack(m, psic, m->v[klev + 1], klev + 1);
    free(rf);
    free(psic);
}

/* finer, rcsc.f:1392-1444 */
void orc_str_finer(orc_str_mg_t *m, int klev)
{
    const orc_str_grid_t *g = m->g;
    const int ld = m->ld, n1c = g->n1[klev];
    const int n1f = g->n1[klev - 1], n2f = g->n2[klev - 1];
    const double *pc = m->v[klev];
    const double *vf = m->v[klev - 1];
#define PC(i, j) pc[(size_t)(i) + (size_t)(n1c + 1) * (size_t)(j)]
    for (int i = 0; i <= n1f; ++i)
        for (int j = 0; j <= n2f; ++j) {
            const int i1 = i / 2, j1 = j / 2;
            double p;
            if (i1 * 2 == i) {
                if (j1 * 2 == j) p = PC(i1, j1);
                else p = (PC(i1, j1) + PC(i1, j1 + 1)) * 0.5;
            } else {
                if (j1 * 2 == j) {
                    p = (PC(i1, j1) + PC(i1 + 1, j1)) * 0.5;
                } else {
                    double temp = PC(i1, j1) + PC(i1 + 1, j1 + 1);
                    temp = temp + PC(i1, j1 + 1) + PC(i1 + 1, j1);
                    p = temp * 0.25;
                }
            }
            PX(i, j) = p + vf[(size_t)i + (size_t)(n1f + 1) * (size_t)j];
        }
#undef PC
    const size_t szc = (size_t)(n1c + 1) * (size_t)(g->n2[klev] + 1);
    memset(m->v[klev], 0, szc * sizeof(double));
    pack(m, m->psif, m->v[klev - 1], klev - 1);
}

/* poisson, rcsc.f:1118-1195 */
int orc_str_poisson(orc_str_mg_t *m, double *psi, const double *rhs, int *sweeps)
{
    const orc_str_grid_t *g = m->g;
    const int n1 = g->n1[1], n2 = g->n2[1], nlev = m->nlev, l1 = n1 + 1;
    for (int j = 0; j <= n2; ++j)
        for (int i = 0; i <= n1; ++i) {
            m->f[1][(size_t)i + (size_t)l1 * j] = rhs[(size_t)i + (size_t)l1 * j];
            m->v[1][(size_t)i + (size_t)l1 * j] = psi[(size_t)i + (size_t)l1 * j];
        }
    memset(m->rc, 0, sizeof(double) * (size_t)m->ld * (size_t)m->ld);
    int nconv = 0;
    for (int sweep = 1; sweep <= m->maxsweeps; ++sweep) {
        if (sweep == 1 || nlev == 1) orc_str_relax(m, m->nrel, 1, &nconv);
        if (nlev > 1) {
            for (int l = 1; l <= nlev - 1; ++l) {
                orc_str_corser(m, l);
                orc_str_relax(m, m->nrel, l + 1, &nconv);
            }
            for (int l = nlev; l >= 2; --l) {
                orc_str_finer(m, l);
                orc_str_relax(m, m->nrel, l - 1, &nconv);
            }
        }
        if (m->last_resmax != m->last_resmax) {
            if (sweeps) *sweeps = sweep;
            return 2;
        }
        if (nconv == 1) {
            const int ld = m->ld;
            for (int j = 0; j <= n2; ++j)
                for (int i = 0; i <= n1; ++i) psi[(size_t)i + (size_t)l1 * j] = PX(i, j);
            if (sweeps) *sweeps = sweep;
            return 0;
        }
    }
    if (sweeps) *sweeps = m->maxsweeps;
    return 1;
}
