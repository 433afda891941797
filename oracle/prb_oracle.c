/*
 * CPU oracle: restatement of the 2D periodic Rayleigh-Benard hot path of
 * monashubuntudir_velvor2dperiodicrbconvdir/velvor2dperiodicrbconv.f (PRB).
 *
 * TEST INFRASTRUCTURE ONLY -- the checker for tests/, smoke() and the CPU
 * legs of bench.py; never linked into the product.  PARITY PINNED to the
 * reference's own source: with no Fortran compiler in the image, the
 * reference's drivers are run on the CPU by a translator of their Fortran
 * (tests/golden/f77.py), and this file reproduces those runs bit for bit —
 * every field, Nusselt number and sweep count of the layer, its oblique
 * and annulus variants and the Taylor-Couette driver
 * (tests/test_reference_runs.py).  The one departure: velvor2dtaycouheat.f
 * forms a relax2 line's right-hand side only for k = 1 (:2132-2164), so its
 * first solve STOPs; this file forms every line's, as
 * velvor2dtaycouheat_new.f:2181-2182 does.
 *
 * Every expression keeps the reference's left-to-right evaluation order.
 * Fortran REAL*4 literals that the reference mixes into REAL*8 arithmetic
 * (2./3., 1./6., 0.01) are reproduced as the float values they round to.
 * Build with -O2 -ffp-contract=off (see Makefile).
 */
#include "prb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define IX(i, k) ((size_t)(i) + (size_t)ld * (size_t)(k))

/* ------------------------------------------------------------------------ */
/* Banded solvers                                                            */
/* ------------------------------------------------------------------------ */

/* Thomas algorithm, PRB:3046-3064. */
void orc_tdma(double *a, double *b, double *c, double *y, double *r, int n)
{
    for (int j = 1; j < n; ++j) {
        double fact = a[j] / b[j - 1];
        b[j] = b[j] - fact * c[j - 1];
        r[j] = r[j] - fact * r[j - 1];
    }
    y[n - 1] = r[n - 1] / b[n - 1];
    for (int j = n - 2; j >= 0; --j)
        y[j] = (r[j] - c[j] * y[j + 1]) / b[j];
}

/* Periodic Thomas algorithm with the fill-in column n, PRB:3066-3116.
 * Row 1 couples to unknown n through a(1); row n to unknown 1 through c(n). */
void orc_ptdma(double *a, double *b, double *c, double *y, double *r, int n)
{
    const int N = n - 1;
    double fact;
    for (int j = 1; j <= n - 3; ++j) {
        fact = a[j] / b[j - 1];
        b[j] = b[j] - fact * c[j - 1];
        a[j] = -fact * a[j - 1];
        r[j] = r[j] - fact * r[j - 1];
        fact = c[N] / b[j - 1];
        c[N] = -fact * c[j - 1];
        b[N] = b[N] - fact * a[j - 1];
        r[N] = r[N] - fact * r[j - 1];
    }
    fact = a[n - 2] / b[n - 3];
    b[n - 2] = b[n - 2] - fact * c[n - 3];
    c[n - 2] = c[n - 2] - fact * a[n - 3];
    r[n - 2] = r[n - 2] - fact * r[n - 3];
    fact = c[N] / b[n - 3];
    a[N] = a[N] - fact * c[n - 3];
    b[N] = b[N] - fact * a[n - 3];
    r[N] = r[N] - fact * r[n - 3];
    fact = a[N] / b[n - 2];
    b[N] = b[N] - fact * c[n - 2];
    r[N] = r[N] - fact * r[n - 2];
    y[N] = r[N] / b[N];
    y[n - 2] = (r[n - 2] - c[n - 2] * y[N]) / b[n - 2];
    for (int j = n - 3; j >= 0; --j)
        y[j] = (r[j] - c[j] * y[j + 1] - a[j] * y[N]) / b[j];
}

/* Pentadiagonal elimination with row normalisation, PRB:3118-3164.
 * a: second sub-diagonal, b: sub, c: diagonal, d: super, e: second super. */
void orc_pdma(double *a, double *b, double *c, double *d, double *e,
              double *r, double *x, int n)
{
    for (int k = 0; k <= n - 2; ++k) {
        d[k] = d[k] / c[k];
        e[k] = e[k] / c[k];
        r[k] = r[k] / c[k];
        c[k] = 1.0;
        c[k + 1] = c[k + 1] - b[k + 1] * d[k];
        if (k != n - 2) d[k + 1] = d[k + 1] - b[k + 1] * e[k];
        r[k + 1] = r[k + 1] - b[k + 1] * r[k];
        b[k + 1] = 0.0;
        if (k != n - 2) {
            b[k + 2] = b[k + 2] - a[k + 2] * d[k];
            c[k + 2] = c[k + 2] - a[k + 2] * e[k];
            r[k + 2] = r[k + 2] - a[k + 2] * r[k];
        }
    }
    x[n - 1] = r[n - 1] / c[n - 1];
    x[n - 2] = r[n - 2] - d[n - 2] * x[n - 1];
    for (int j = n - 3; j >= 0; --j)
        x[j] = r[j] - d[j] * x[j + 1] - e[j] * x[j + 2];
}

/* ------------------------------------------------------------------------ */
/* Multigrid (PRB:1724-2859)                                                 */
/* ------------------------------------------------------------------------ */

/* Level count and sizes, poissoninit PRB:1724-1793.  The level count is the
 * number of halvings of nr while the halved value is even and >= 4, capped
 * at 4; np only follows (n3 = np*2/2^l, integer division). */
int orc_mg_init(orc_mg_t *mg, int nr, int np, double dr, double dp)
{
    return orc_mg_init_variant(mg, nr, np, dr, dp, ORC_PRB, 0.0);
}

/* The annulus driver's poissoninit (velvor2dnewsch3.4.f:1736-1806) differs
 * only in the cap of 5 levels (:1778); its relax2/relax3 set tolcon = 10e-6
 * (:2093, :2389) and its poisson2/poisson3 run up to nvs = 10000 sweeps and
 * then return without a STOP (:1829, :1960). */
int orc_mg_init_variant(orc_mg_t *mg, int nr, int np, double dr, double dp, int variant, double r0)
{
    memset(mg, 0, sizeof(*mg));
    int nlev = 0, itest = nr, itest2 = nr;
    for (int i = 2; i <= 8; ++i) {
        itest = itest / 2;
        if (itest * 2 - itest2 == 0) {
            if (itest2 >= 4) nlev = nlev + 1;
            itest2 = itest;
        } else {
            break;
        }
    }
    if (variant == ORC_ANNULUS) {
        if (nlev > 5) nlev = 5;
    } else if (nlev >= 5) {
        nlev = 4;
    }
    if (nlev < 1 || np < 4) return ORC_INVALID;
    mg->nr = nr;
    mg->np = np;
    mg->ld = nr + 2;
    mg->nlev = nlev;
    for (int l = 1; l <= nlev; ++l) {
        mg->n1[l] = nr * 2 / (1 << l);
        mg->n3[l] = np * 2 / (1 << l);
        mg->hr[l] = dr * (double)(1 << l) * 0.5;
        mg->hp[l] = dp * (double)(1 << l) * 0.5;
        mg->hhr[l] = mg->hr[l] * mg->hr[l];
        mg->hhp[l] = mg->hp[l] * mg->hp[l];
        size_t sz = (size_t)(mg->n1[l] + 1) * (size_t)(mg->n3[l] + 1);
        mg->v[l] = (double *)calloc(sz, sizeof(double));
        mg->f[l] = (double *)calloc(sz, sizeof(double));
    }
    size_t full = (size_t)mg->ld * (size_t)(np + 1);
    mg->psic = (double *)calloc(full, sizeof(double));
    mg->psif = (double *)calloc(full, sizeof(double));
    mg->rc = (double *)calloc(full, sizeof(double));
    mg->rf = (double *)calloc(full, sizeof(double));
    mg->tempa = (double *)calloc(full, sizeof(double));
    mg->tolcon = 2.0e-6;
    mg->sor = 1.2;
    mg->maxsweeps = 500;
    mg->mode = ORC_LEX;
    mg->zero_scratch = 0;
    mg->mgen = 650000;
    mg->variant = variant;
    mg->r0 = r0;
    if (variant == ORC_ANNULUS) {
        mg->tolcon = 10.0e-6;
        mg->maxsweeps = 10000;
        mg->mgen = 2000000;
    }
    if (variant == ORC_TAYCOU) mg->tolcon = 1.0e-5;   /* velvor2dtaycouheat.f:1234, :1345 */
    if (variant == ORC_TANK || variant == ORC_DVD) {   /* velvor2dhorconvtank.f:1163, :1264 */
        mg->tolcon = 5.0e-6;
        mg->xwall = 1;
    }
    return ORC_OK;
}

void orc_mg_free(orc_mg_t *mg)
{
    for (int l = 1; l <= mg->nlev; ++l) {
        free(mg->v[l]);
        free(mg->f[l]);
    }
    free(mg->psic); free(mg->psif); free(mg->rc); free(mg->rf); free(mg->tempa);
    free(mg->scratch_v); free(mg->scratch_f);
    memset(mg, 0, sizeof(*mg));
}

/* trans1 / trans2, PRB:2805-2846: pack a level region into its 1D slot and back. */
static void trans1(const orc_mg_t *mg, const double *a2, double *a1, int l)
{
    const int ld = mg->ld, n1 = mg->n1[l], n3 = mg->n3[l];
    for (int k = 0; k <= n3; ++k)
        for (int i = 0; i <= n1; ++i)
            a1[(size_t)k * (n1 + 1) + i] = a2[IX(i, k)];
}

static void trans2(const orc_mg_t *mg, const double *a1, double *a2, int l)
{
    const int ld = mg->ld, n1 = mg->n1[l], n3 = mg->n3[l];
    for (int k = 0; k <= n3; ++k)
        for (int i = 0; i <= n1; ++i)
            a2[IX(i, k)] = a1[(size_t)k * (n1 + 1) + i];
}

/* Line k of the cell-centred (v) relaxation, PRB:2113-2191 (annulus:
 * velvor2dnewsch3.4.f:2140-2182).  rvq[i] = 1/r^2 of row i (1 in PRB). */
static void relax2_line(orc_mg_t *mg, int klev, int k, const double *ca,
                        const double *cb, const double *cc, const double *cd,
                        const double *ce, const double *rvq, double hhpi, double *wa,
                        double *wb, double *wc, double *wd, double *we, double *wr, double *ws)
{
    const int ld = mg->ld, n1 = mg->n1[klev], n3 = mg->n3[klev];
    double *psif = mg->psif;
    const double *rf = mg->rf;
    int ka = k + 1, km = k - 1;
    if (k == n3) ka = 1;
    for (int i = 1; i <= n1; ++i) {
        wa[i - 1] = ca[i];
        wb[i - 1] = cb[i];
        wc[i - 1] = cc[i];
        wd[i - 1] = cd[i];
        we[i - 1] = ce[i];
        wr[i - 1] = -(psif[IX(i, ka)] + psif[IX(i, km)]) * hhpi * rvq[i] + rf[IX(i, k)];
    }
    orc_pdma(wa, wb, wc, wd, we, wr, ws, n1);
    for (int i = 1; i <= n1; ++i) {
        psif[IX(i, k)] = ws[i - 1];
        if (k == n3) psif[IX(i, 0)] = psif[IX(i, k)];
    }
}

/* Line k of the face (u) relaxation, PRB:2414-2460 (annulus:
 * velvor2dnewsch3.4.f:2415-2452). */
static void relax3_line(orc_mg_t *mg, int klev, int k, const double *ca,
                        const double *cb, const double *cc, const double *rvq, double hhpi,
                        double *wa, double *wb, double *wc, double *wr, double *ws)
{
    const int ld = mg->ld, n1 = mg->n1[klev], n3 = mg->n3[klev];
    double *psif = mg->psif;
    const double *rf = mg->rf;
    int ka = k + 1, km = k - 1;
    if (k == n3) ka = mg->xwall ? 0 : 1;
    for (int i = 1; i <= n1 - 1; ++i) {
        wa[i - 1] = ca[i];
        wb[i - 1] = cb[i];
        wc[i - 1] = cc[i];
        wr[i - 1] = -(psif[IX(i, ka)] + psif[IX(i, km)]) * hhpi * rvq[i] + rf[IX(i, k)];
    }
    orc_tdma(wa, wb, wc, ws, wr, n1 - 1);
    for (int i = 1; i <= n1 - 1; ++i) {
        psif[IX(i, k)] = ws[i - 1];
        if (k == n3) psif[IX(i, 0)] = mg->xwall ? 0.0 : psif[IX(i, k)];
    }
}

/* relax2 (PRB:2063-2371) for which == 2, relax3 (PRB:2374-2600) for which == 3.
 * nconv is set when klev == 1 and the max-norm residual is below tolcon.
 * A NaN residual sets mg->last_resmax to NaN (the reference's max ignores it).
 *
 * ORC_ANNULUS follows relax2/relax3 of velvor2dnewsch3.4.f:2071-2596: the
 * polar operator d2/dr2 + (1/r) d/dr + (1/r^2) d2/dphi2 with the extra 1/r^2
 * diagonal term of the staggered velocity components, radii r = r0 +
 * (i-1/2) hr (v) and r = i hr + r0 (u) of the level, and three relaxations
 * per call whatever nrel says (:2134, :2410). */
void orc_relax(orc_mg_t *mg, int which, int nrel, int klev, int *nconv)
{
    const int ld = mg->ld, n1 = mg->n1[klev], n3 = mg->n3[klev];
    const int polar = (mg->variant == ORC_ANNULUS || mg->variant == ORC_TAYCOU);
    double *psif = mg->psif, *rc = mg->rc, *rf = mg->rf;
    *nconv = 0;
    trans2(mg, mg->f[klev], rf, klev);
    const double hhri = 1.0 / mg->hhr[klev];
    const double hri = 1.0 / mg->hr[klev];
    const double hhpi = 1.0 / mg->hhp[klev];
    if (mg->variant == ORC_ANNULUS) nrel = 3;

    const int nmax = n1 + 2;
    double *buf = (double *)malloc(sizeof(double) * (size_t)nmax * 14);
    double *ca = buf, *cb = ca + nmax, *cc = cb + nmax, *cd = cc + nmax, *ce = cd + nmax;
    double *wa = ce + nmax, *wb = wa + nmax, *wc = wb + nmax, *wd = wc + nmax;
    double *we = wd + nmax, *wr = we + nmax, *ws = wr + nmax;
    double *rvi = ws + nmax, *rvq = rvi + nmax;

    for (int i = 0; i < nmax; ++i) { rvi[i] = 1.0; rvq[i] = 1.0; }
    if (which == 2) {
        /* coefficients, PRB:2128-2156 (computed at k == 1, reused for every
         * line); annulus velvor2dnewsch3.4.f:2104-2131 */
        for (int i = 1; i <= n1; ++i) {
            if (polar) {
                const double rval = mg->r0 + ((double)i - 0.5) * mg->hr[klev];
                rvi[i] = 1.0 / rval;
                rvq[i] = rvi[i] * rvi[i];
                if (i == 1) {
                    ca[i] = 0.0;
                    cb[i] = 0.0;
                    cc[i] = -2.0 * hhri - 2.0 * hhpi * rvq[i] + rvq[i];
                    cd[i] = 5.0 / 3.0 * hhri + 4.0 / 3.0 * hri * rvi[i];
                    ce[i] = -0.2 * hhri;
                } else if (i == n1) {
                    ca[i] = -0.2 * hhri;
                    cb[i] = 5.0 / 3.0 * hhri - 4.0 / 3.0 * hri * rvi[i];
                    cc[i] = -2.0 * hhri - 2.0 * hhpi * rvq[i] + rvq[i];
                    cd[i] = 0.0;
                    ce[i] = 0.0;
                } else {
                    ca[i] = 0.0;
                    cb[i] = hhri - 1.5 * hri * rvi[i];
                    cc[i] = -(2.0 * hhri + 2.0 * hhpi * rvq[i]) + rvq[i];
                    cd[i] = hhri + 1.5 * hri * rvi[i];
                    ce[i] = 0.0;
                }
            } else if (i == 1) {
                ca[i] = 0.0;
                cb[i] = 0.0;
                cc[i] = -2.0 * hhri - 2.0 * hhpi * rvq[i];
                cd[i] = 5.0 / 3.0 * hhri;
                ce[i] = -0.2 * hhri;
            } else if (i == n1) {
                ca[i] = -0.2 * hhri;
                cb[i] = 5.0 / 3.0 * hhri;
                cc[i] = -2.0 * hhri - 2.0 * hhpi * rvq[i];
                cd[i] = 0.0;
                ce[i] = 0.0;
            } else {
                ca[i] = 0.0;
                cb[i] = hhri;
                cc[i] = -(2.0 * hhri + 2.0 * hhpi * rvq[i]);
                cd[i] = hhri;
                ce[i] = 0.0;
            }
        }
    } else {
        /* PRB:2421-2436; annulus velvor2dnewsch3.4.f:2401-2408 */
        for (int i = 1; i <= n1 - 1; ++i) {
            if (polar) {
                const double rval = (double)i * mg->hr[klev] + mg->r0;
                rvi[i] = 1.0 / rval;
                rvq[i] = rvi[i] * rvi[i];
                ca[i] = hhri - 1.5 * hri * rvi[i];
                cb[i] = -(2.0 * hhri - rvq[i] + 2.0 * hhpi * rvq[i]);
                cc[i] = hhri + 1.5 * hri * rvi[i];
            } else {
                ca[i] = hhri;
                cb[i] = -(2.0 * hhri + 2.0 * hhpi * rvq[i]);
                cc[i] = hhri;
            }
        }
    }

    double resmax = 0.0;
    int anynan = 0;
    const int klast = (mg->xwall && which == 2) ? n3 - 1 : n3;   /* the tank's v walls k = 0, n3 */
    for (int irel = 1; irel <= nrel; ++irel) {
        if (mg->mode == ORC_LEX) {
            for (int k = 1; k <= klast; ++k) {
                if (which == 2) relax2_line(mg, klev, k, ca, cb, cc, cd, ce, rvq, hhpi, wa, wb, wc, wd, we, wr, ws);
                else relax3_line(mg, klev, k, ca, cb, cc, rvq, hhpi, wa, wb, wc, wr, ws);
            }
        } else {
            for (int parity = 1; parity >= 0; --parity) {
                for (int k = 1; k <= klast; ++k) {
                    if ((k & 1) != parity) continue;
                    if (which == 2) relax2_line(mg, klev, k, ca, cb, cc, cd, ce, rvq, hhpi, wa, wb, wc, wd, we, wr, ws);
                    else relax3_line(mg, klev, k, ca, cb, cc, rvq, hhpi, wa, wb, wc, wr, ws);
                }
            }
        }
        /* residual and its max norm, PRB:2306-2357 / PRB:2553-2587
         * (annulus velvor2dnewsch3.4.f:2300-2346 / :2546-2579) */
        resmax = 0.0;
        for (int k = 1; k <= klast; ++k) {
            int ka = k + 1, km = k - 1;
            if (k == n3) ka = mg->xwall ? 0 : 1;
            if (which == 2) {
                for (int i = 1; i <= n1; ++i) {
                    double temp;
                    if (polar) {
                        temp = (psif[IX(i, ka)] - 2.0 * psif[IX(i, k)] + psif[IX(i, km)]) * hhpi * rvq[i] +
                               psif[IX(i, k)] * rvq[i];
                        if (i == 1)
                            temp = temp + (-2.0 * psif[IX(i, k)] + 5.0 / 3.0 * psif[IX(i + 1, k)] -
                                           0.2 * psif[IX(i + 2, k)]) * hhri +
                                   4.0 / 3.0 * psif[IX(i + 1, k)] * hri * rvi[i];
                        else if (i == n1)
                            temp = temp + (-2.0 * psif[IX(i, k)] + 5.0 / 3.0 * psif[IX(i - 1, k)] -
                                           0.2 * psif[IX(i - 2, k)]) * hhri -
                                   4.0 / 3.0 * psif[IX(i - 1, k)] * hri * rvi[i];
                        else
                            temp = temp + (psif[IX(i - 1, k)] - 2.0 * psif[IX(i, k)] + psif[IX(i + 1, k)]) * hhri +
                                   1.5 * (psif[IX(i + 1, k)] - psif[IX(i - 1, k)]) * hri * rvi[i];
                    } else {
                        temp = (psif[IX(i, ka)] - 2.0 * psif[IX(i, k)] + psif[IX(i, km)]) * hhpi * rvq[i];
                        if (i == 1)
                            temp = temp + (-2.0 * psif[IX(i, k)] + 5.0 / 3.0 * psif[IX(i + 1, k)] -
                                           0.2 * psif[IX(i + 2, k)]) * hhri;
                        else if (i == n1)
                            temp = temp + (-2.0 * psif[IX(i, k)] + 5.0 / 3.0 * psif[IX(i - 1, k)] -
                                           0.2 * psif[IX(i - 2, k)]) * hhri;
                        else
                            temp = temp + (psif[IX(i - 1, k)] - 2.0 * psif[IX(i, k)] + psif[IX(i + 1, k)]) * hhri;
                    }
                    temp = rf[IX(i, k)] - temp;
                    rc[IX(i, k)] = temp;
                    temp = fabs(temp);
                    if (temp != temp) anynan = 1;
                    if (temp > resmax) resmax = temp;
                }
            } else {
                for (int i = 1; i <= n1 - 1; ++i) {
                    double temp;
                    if (polar)
                        temp = (psif[IX(i + 1, k)] + psif[IX(i - 1, k)]) * hhri +
                               1.5 * (psif[IX(i + 1, k)] - psif[IX(i - 1, k)]) * hri * rvi[i] +
                               psif[IX(i, k)] * rvq[i] +
                               (psif[IX(i, ka)] + psif[IX(i, km)]) * hhpi * rvq[i] -
                               psif[IX(i, k)] * (2.0 * hhri + 2.0 * hhpi * rvq[i]);
                    else
                        temp = (psif[IX(i + 1, k)] + psif[IX(i - 1, k)]) * hhri +
                               (psif[IX(i, ka)] + psif[IX(i, km)]) * hhpi * rvq[i] -
                               psif[IX(i, k)] * (2.0 * hhri + 2.0 * hhpi * rvq[i]);
                    temp = rf[IX(i, k)] - temp;
                    rc[IX(i, k)] = temp;
                    temp = fabs(temp);
                    if (temp != temp) anynan = 1;
                    if (temp > resmax) resmax = temp;
                }
            }
        }
    }
    free(buf);
    trans1(mg, psif, mg->v[klev], klev);
    if (klev == 1) mg->last_resmax = anynan ? NAN : resmax;
    if (klev == 1 && resmax < mg->tolcon) *nconv = 1;
}

/* Restriction to level klev+1, corser PRB:2603-2718: full weighting written
 * as the 27-point formula with the j neighbours collapsed, summed left to
 * right; faces and the periodic seam of rc, psic and psif zeroed. */
void orc_corser(orc_mg_t *mg, int klev)
{
    const int ld = mg->ld;
    const int n1 = mg->n1[klev], n3 = mg->n3[klev];
    const int n1c = mg->n1[klev + 1], n3c = mg->n3[klev + 1];
    double *rc = mg->rc, *rf = mg->rf, *psic = mg->psic, *psif = mg->psif;
    for (int k = 0; k <= n3; ++k)
        for (int i = 0; i <= n1; ++i) rf[IX(i, k)] = rc[IX(i, k)];
    for (int k = 1; k <= n3c - 1; ++k) {
        for (int i = 1; i <= n1c - 1; ++i) {
            const int ii = i + i, kk = k + k;
            const int iip = ii + 1, iim = ii - 1, kkp = kk + 1, kkm = kk - 1;
            psic[IX(i, k)] = 0.0;
            psif[IX(i, k)] = 0.0;
            double t = rf[IX(ii, kk)];
            t = t + t;
            t = t + rf[IX(iip, kk)];
            t = t + rf[IX(iim, kk)];
            t = t + rf[IX(ii, kk)];
            t = t + rf[IX(ii, kk)];
            t = t + rf[IX(ii, kkp)];
            t = t + rf[IX(ii, kkm)];
            t = t + t;
            t = t + rf[IX(iip, kk)];
            t = t + rf[IX(iip, kk)];
            t = t + rf[IX(iim, kk)];
            t = t + rf[IX(iim, kk)];
            t = t + rf[IX(iip, kkp)];
            t = t + rf[IX(iip, kkm)];
            t = t + rf[IX(iim, kkp)];
            t = t + rf[IX(iim, kkm)];
            t = t + rf[IX(ii, kkp)];
            t = t + rf[IX(ii, kkm)];
            t = t + rf[IX(ii, kkp)];
            t = t + rf[IX(ii, kkm)];
            t = t + t;
            t = t + rf[IX(iip, kkp)];
            t = t + rf[IX(iip, kkm)];
            t = t + rf[IX(iip, kkp)];
            t = t + rf[IX(iip, kkm)];
            t = t + rf[IX(iim, kkp)];
            t = t + rf[IX(iim, kkm)];
            t = t + rf[IX(iim, kkp)];
            t = t + rf[IX(iim, kkm)];
            t = t * 0.015625;
            rc[IX(i, k)] = t;
        }
    }
    for (int k = 0; k <= n3c; ++k) {
        rc[IX(0, k)] = 0.0;
        rc[IX(n1c, k)] = 0.0;
        psic[IX(0, k)] = 0.0;
        psic[IX(n1c, k)] = 0.0;
        psif[IX(0, k)] = 0.0;
        psif[IX(n1c, k)] = 0.0;
    }
    for (int i = 0; i <= n1c; ++i) {
        /* The annulus corser (velvor2dnewsch3.4.f:2696-2704) leaves rc on the
         * seam lines k = 0 and k = n3c alone, so the coarse right-hand side of
         * line n3c keeps the fine residual stored there. */
        if (mg->variant != ORC_ANNULUS) {
            rc[IX(i, 0)] = 0.0;
            rc[IX(i, n3c)] = 0.0;
        }
        psic[IX(i, 0)] = 0.0;
        psic[IX(i, n3c)] = 0.0;
        psif[IX(i, 0)] = 0.0;
        psif[IX(i, n3c)] = 0.0;
    }
    trans1(mg, rc, mg->f[klev + 1], klev + 1);
}

/* Prolongation from level klev to klev-1 plus the saved fine solution,
 * finer PRB:2721-2803. */
void orc_finer(orc_mg_t *mg, int klev)
{
    const int ld = mg->ld;
    const int n1f = mg->n1[klev - 1], n3f = mg->n3[klev - 1];
    double *psic = mg->psic, *psif = mg->psif, *tempa = mg->tempa;
    trans2(mg, mg->v[klev], psic, klev);
    for (int i = 0; i <= n1f; ++i) {
        for (int k = 0; k <= n3f; ++k) {
            const int i1 = i / 2, k1 = k / 2;
            if (i1 * 2 == i) {
                if (k1 * 2 == k) psif[IX(i, k)] = psic[IX(i1, k1)];
                else psif[IX(i, k)] = (psic[IX(i1, k1)] + psic[IX(i1, k1 + 1)]) * 0.5;
            } else {
                if (k1 * 2 == k) psif[IX(i, k)] = (psic[IX(i1, k1)] + psic[IX(i1 + 1, k1)]) * 0.5;
                else psif[IX(i, k)] = (psic[IX(i1, k1)] + psic[IX(i1 + 1, k1)] +
                                       psic[IX(i1, k1 + 1)] + psic[IX(i1 + 1, k1 + 1)]) * 0.25;
            }
        }
    }
    trans2(mg, mg->v[klev - 1], tempa, klev - 1);
    for (int k = 0; k <= n3f; ++k) {
        for (int i = 0; i <= n1f; ++i) {
            psif[IX(i, k)] = psif[IX(i, k)] + tempa[IX(i, k)];
            psic[IX(i, k)] = 0.0;
        }
    }
}

/* poisson2 (PRB:1796-1927) / poisson3 (PRB:1930-2059): extrapolated initial
 * guess 2psi-psip, SOR of the whole-cycle change, FMG-flavoured schedule,
 * convergence on the level-1 max-norm residual.  Where the reference STOPs
 * the process after maxsweeps sweeps, this returns ORC_MAXSWEEPS and leaves
 * psi untouched. */
int orc_poisson(orc_mg_t *mg, int which, double *psi, double *psip,
                const double *rhs, int ld_io, int *sweeps)
{
    const int ld = mg->ld, nr = mg->nr, np = mg->np, nlev = mg->nlev;
    const int imax = (which == 2) ? nr + 1 : nr;
    double *psif = mg->psif, *psic = mg->psic, *rc = mg->rc, *rf = mg->rf;
    int nconv = 0;
#define IO(i, k) ((size_t)(i) + (size_t)ld_io * (size_t)(k))
    if (mg->zero_scratch) {
        if (!mg->scratch_v) {
            mg->scratch_v = (double *)malloc(sizeof(double) * (size_t)mg->mgen);
            mg->scratch_f = (double *)malloc(sizeof(double) * (size_t)mg->mgen);
        }
        for (long i = 0; i < mg->mgen; ++i) {
            mg->scratch_v[i] = 0.0;
            mg->scratch_f[i] = 0.0;
        }
    }
    for (int i = 0; i <= imax; ++i) {
        for (int k = 0; k <= np; ++k) {
            psic[IX(i, k)] = 0.0;
            psif[IX(i, k)] = 2.0 * psi[IO(i, k)] - psip[IO(i, k)];
            rc[IX(i, k)] = 0.0;
            rf[IX(i, k)] = rhs[IO(i, k)];
        }
    }
    trans1(mg, rf, mg->f[1], 1);
    trans1(mg, psif, mg->v[1], 1);
    for (int sweep = 1;; ++sweep) {
        if (sweep > mg->maxsweeps) {
            if (sweeps) *sweeps = sweep - 1;
            mg->last_sweeps = sweep - 1;
            return ORC_MAXSWEEPS;
        }
        if (sweep != 1) {
            for (int i = 0; i <= imax; ++i) {
                for (int k = 0; k <= np; ++k) {
                    psif[IX(i, k)] = psip[IO(i, k)] + mg->sor * (psif[IX(i, k)] - psip[IO(i, k)]);
                    psip[IO(i, k)] = psif[IX(i, k)];
                }
            }
            trans1(mg, psif, mg->v[1], 1);
        }
        if (sweep == 1 || nlev == 1) {
            orc_relax(mg, which, 1, 1, &nconv);
            for (int i = 0; i <= imax; ++i)
                for (int k = 0; k <= np; ++k) psip[IO(i, k)] = psif[IX(i, k)];
        }
        if (nlev > 1) {
            for (int l = 1; l <= nlev - 1; ++l) {
                orc_corser(mg, l);
                orc_relax(mg, which, 1, l + 1, &nconv);
            }
            for (int ifmg = 0; ifmg <= nlev - 2; ++ifmg) {
                for (int l = nlev; l >= nlev - ifmg; --l) {
                    orc_finer(mg, l);
                    orc_relax(mg, which, 1, l - 1, &nconv);
                }
                for (int l = nlev - ifmg - 1; l <= nlev - 1; ++l) {
                    orc_corser(mg, l);
                    orc_relax(mg, which, 1, l + 1, &nconv);
                }
            }
            for (int l = nlev; l >= 2; --l) {
                orc_finer(mg, l);
                orc_relax(mg, which, 1, l - 1, &nconv);
            }
        }
        if (mg->last_resmax != mg->last_resmax) {
            if (sweeps) *sweeps = sweep;
            mg->last_sweeps = sweep;
            return ORC_NAN;
        }
        if (nconv == 1) {
            for (int i = 0; i <= imax; ++i)
                for (int k = 0; k <= np; ++k) psip[IO(i, k)] = psi[IO(i, k)];
            /* the tank: v on k = 1..np-1, u on k = 1..np (velvor2dhorconvtank.f:1032, :1129) */
            const int k0 = mg->xwall ? 1 : 0, k1 = mg->xwall ? (which == 2 ? np - 1 : np) : np;
            for (int i = 1; i <= imax - 1; ++i)
                for (int k = k0; k <= k1; ++k) psi[IO(i, k)] = psif[IX(i, k)];
            for (int k = 0; k <= np; ++k) {
                psi[IO(0, k)] = 0.0;
                psi[IO(imax, k)] = 0.0;
            }
            if (mg->xwall)
                for (int i = 0; i <= imax; ++i) {
                    psi[IO(i, 0)] = 0.0;
                    psi[IO(i, which == 2 ? np : np + 1)] = 0.0;
                }
            if (sweeps) *sweeps = sweep;
            mg->last_sweeps = sweep;
            return ORC_OK;
        }
    }
#undef IO
}

/* ------------------------------------------------------------------------ */
/* Transport step                                                            */
/* ------------------------------------------------------------------------ */

int orc_prb_alloc(orc_prb_t *s, int nr, int np, int ld)
{
    memset(s, 0, sizeof(*s));
    if (ld < nr + 2) ld = nr + 2;
    s->nr = nr;
    s->np = np;
    s->ld = ld;
    size_t sz = (size_t)ld * (size_t)(np + 2);   /* the tank's T and u have a ghost column np+1 */
    double **f[] = {&s->An, &s->A, &s->Ap, &s->Bn, &s->B, &s->Bp, &s->Cn, &s->C, &s->Cp,
                    &s->thn, &s->th, &s->thp, &s->uel, &s->vel, &s->wel, &s->uelp,
                    &s->velp, &s->welp, &s->urh, &s->vrh};
    for (size_t i = 0; i < sizeof(f) / sizeof(f[0]); ++i) {
        *f[i] = (double *)calloc(sz, sizeof(double));
        if (!*f[i]) return ORC_INVALID;
    }
    s->r0 = 0.5;
    s->rmax = 1.0;
    s->xx = 3.0;
    return ORC_OK;
}

void orc_prb_free(orc_prb_t *s)
{
    double *f[] = {s->An, s->A, s->Ap, s->Bn, s->B, s->Bp, s->Cn, s->C, s->Cp, s->thn,
                   s->th, s->thp, s->uel, s->vel, s->wel, s->uelp, s->velp, s->welp,
                   s->urh, s->vrh};
    for (size_t i = 0; i < sizeof(f) / sizeof(f[0]); ++i) free(f[i]);
    memset(s, 0, sizeof(*s));
}

/* The (r, phi) plane of the annulus drivers (velvor2dnewsch3.4.f and the
 * Taylor-Couette velvor2dtaycouheat.f): radius terms everywhere. */
static int prb_polar(const orc_prb_t *s) { return s->variant == ORC_ANNULUS || s->variant == ORC_TAYCOU; }

/* The Taylor-Couette outer wall speed -(Ta**0.5) Ptl 0.5 rmax
 * (velvor2dtaycouheat.f:177, :1587, :1668); ** 0.5d0 through libm pow as
 * the compiled Fortran calls it. */
static double taycou_wall(const orc_prb_t *s) { return -(pow(s->Ta, 0.5) * s->Pr * 0.5 * s->rmax); }

/* REAL*4 constants of the reference's wall closures (PRB:865-872). */
static const double F23 = (double)(2.0f / 3.0f);
static const double F16 = (double)(1.0f / 6.0f);

/* Compact fourth-order derivatives shared by cvorticity1 and cvorticity
 * (PRB:608-704 / PRB:809-897): Cr -> A, Ch -> B, thr -> An, thh -> Bn. */
static void cvort_derivatives(orc_prb_t *s, double *wa, double *wb, double *wc,
                              double *wr, double *ws)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const double dri = 1.0 / s->dr, dpi = 1.0 / s->dp;
    const double *C = s->C, *th = s->th;
    /* Cr: tdma along r for each k */
    for (int k = 0; k <= np; ++k) {
        for (int i = 1; i <= nr - 1; ++i) {
            wa[i - 1] = 1.0; wb[i - 1] = 4.0; wc[i - 1] = 1.0;
            if (i == 1)
                wr[i - 1] = 3.0 * (C[IX(2, k)] - C[IX(0, k)]) * dri -
                            (-1.5 * C[IX(0, k)] + 2.0 * C[IX(1, k)] - 0.5 * C[IX(2, k)]) * dri;
            else if (i == nr - 1)
                wr[i - 1] = 3.0 * (C[IX(nr, k)] - C[IX(nr - 2, k)]) * dri -
                            (0.5 * C[IX(nr - 2, k)] - 2.0 * C[IX(nr - 1, k)] + 1.5 * C[IX(nr, k)]) * dri;
            else
                wr[i - 1] = 3.0 * (C[IX(i + 1, k)] - C[IX(i - 1, k)]) * dri;
        }
        orc_tdma(wa, wb, wc, ws, wr, nr - 1);
        for (int ii = 1; ii <= nr - 1; ++ii) s->A[IX(ii, k)] = ws[ii - 1];
    }
    /* Ch: periodic tdma along x for each i, n = np+1 */
    for (int i = 1; i <= nr - 1; ++i) {
        for (int k = 0; k <= np; ++k) {
            wa[k] = 1.0; wb[k] = 4.0; wc[k] = 1.0;
            if (k == np) wr[np] = 3.0 * (C[IX(i, 1)] - C[IX(i, np - 1)]) * dpi;
            else if (k == 0) wr[0] = 3.0 * (C[IX(i, 1)] - C[IX(i, np - 1)]) * dpi;
            else wr[k] = 3.0 * (C[IX(i, k + 1)] - C[IX(i, k - 1)]) * dpi;
        }
        orc_ptdma(wa, wb, wc, ws, wr, np + 1);
        for (int kk = 0; kk <= np; ++kk) s->B[IX(i, kk)] = ws[kk];
    }
    /* thr at C points: tdma along r, T averaged over k, k+1 */
    for (int k = 0; k <= np; ++k) {
        for (int i = 1; i <= nr - 1; ++i) {
            wa[i - 1] = 1.0; wb[i - 1] = 4.0; wc[i - 1] = 1.0;
            int ka = k + 1;
            if (k == np) ka = 1;
            if (i == 1)
                wr[i - 1] = 1.5 * (th[IX(2, k)] + th[IX(2, ka)] - th[IX(1, k)] - th[IX(1, ka)]) * dri -
                            (-F23 * (th[IX(0, k)] + th[IX(0, ka)]) + 0.5 * (th[IX(1, k)] + th[IX(1, ka)]) +
                             F16 * (th[IX(2, k)] + th[IX(2, ka)])) * dri;
            else if (i == nr - 1)
                wr[i - 1] = 1.5 * (th[IX(nr, k)] + th[IX(nr, ka)] - th[IX(nr - 1, k)] - th[IX(nr - 1, ka)]) * dri -
                            (-F16 * (th[IX(nr - 1, k)] + th[IX(nr - 1, ka)]) - 0.5 * (th[IX(nr, k)] + th[IX(nr, ka)]) +
                             F23 * (th[IX(nr + 1, k)] + th[IX(nr + 1, ka)])) * dri;
            else
                wr[i - 1] = 1.5 * (th[IX(i + 1, k)] + th[IX(i + 1, ka)] - th[IX(i, k)] - th[IX(i, ka)]) * dri;
        }
        orc_tdma(wa, wb, wc, ws, wr, nr - 1);
        for (int ii = 1; ii <= nr - 1; ++ii) s->An[IX(ii, k)] = ws[ii - 1];
    }
    /* thh at C points: periodic tdma along x */
    for (int i = 1; i <= nr - 1; ++i) {
        for (int k = 0; k <= np; ++k) {
            wa[k] = 1.0; wb[k] = 4.0; wc[k] = 1.0;
            int ka = k + 1;
            if (k == np) ka = 1;
            wr[k] = 1.5 * (th[IX(i + 1, ka)] + th[IX(i, ka)] - th[IX(i + 1, k)] - th[IX(i, k)]) * dpi;
        }
        orc_ptdma(wa, wb, wc, ws, wr, np + 1);
        for (int kk = 0; kk <= np; ++kk) s->Bn[IX(i, kk)] = ws[kk];
    }
}

/* Dufort-Frankel / leapfrog vorticity update, PRB:900-982 (first == 0) and
 * the forward first step, PRB:706-776 (first == 1).  The leapfrog RHS1 uses
 * C, not Cp (PRB:971), as the reference does.
 *
 * ORC_ANNULUS (velvor2dnewsch3.4.f:710-786, :911-993): radius r = r0 + i dr
 * of the C points, the (1/r) dC/dr term Cra*ri in RHS1, 0.5*Cp (not C) in
 * the leapfrog RHS1, and the rotational buoyancy term
 * 2 Ra (-thr u - thh v / r) / Re / Ptl in RHS2.
 *
 * ORC_OBLIQUE (mpkoks.f:769-770, :974-975): the layer with the buoyancy of
 * gravity along the diagonal, RHS2 = -Ra thr 0.707106781 (a REAL*4
 * literal). */
static void cvort_update(orc_prb_t *s, int first)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const int polar = prb_polar(s);
    const double dri = 1.0 / s->dr, dpi = 1.0 / s->dp;
    const double Ptl = s->Pr, dt = s->dt, Ra = s->Ra, Re = s->Re;
    const double *C = s->C, *Cp = s->Cp, *uel = s->uel, *vel = s->vel;
    for (int i = 1; i <= nr - 1; ++i) {
        for (int k = 0; k <= np; ++k) {
            const int ip = i + 1;
            int km = k - 1, ka = k + 1;
            if (k == 0) km = np - 1;
            if (k == np) ka = 1;
            const double r = polar ? s->r0 + (double)i * s->dr : 1.0, ri = 1.0 / r;
            const double u = (uel[IX(i, ka)] + uel[IX(i, k)]) * 0.5;
            const double v = (vel[IX(i, k)] + vel[IX(ip, k)]) * 0.5;
            const double thr = s->An[IX(i, k)];
            const double Chha = (C[IX(i, ka)] + C[IX(i, km)]) * (dpi * dpi);
            const double Ch = s->B[IX(i, k)];
            const double Crra = (C[IX(i - 1, k)] + C[IX(i + 1, k)]) * (dri * dri);
            const double cnr = -1.0 * (dri * dri);
            const double Cra = (C[IX(i + 1, k)] - C[IX(i - 1, k)]) * 0.5 * dri;
            const double Cr = s->A[IX(i, k)];
            const double thh = s->Bn[IX(i, k)];
            const double cnh = (-1.0 * (dpi * dpi)) * (ri * ri);
            double RHS1, RHS2, cf1;
            if (polar) {
                if (first) {
                    RHS1 = Crra + Cra * ri + Chha * (ri * ri) + C[IX(i, k)] / (Ptl * dt);
                    cf1 = 1.0 / (Ptl * dt) - cnr - cnh;
                } else {
                    RHS1 = Crra + Cra * ri + Chha * (ri * ri) + 0.5 * Cp[IX(i, k)] / (Ptl * dt);
                    cf1 = 0.5 / (Ptl * dt) - cnr - cnh;
                }
                RHS2 = -Ra * thh + 2.0 * Ra * (-thr * u - thh * v * ri) / Re / Ptl;
            } else {
                if (first) {
                    RHS1 = Crra + Chha * (ri * ri) + C[IX(i, k)] / (Ptl * dt);
                    cf1 = 1.0 / (Ptl * dt) - cnr - cnh;
                } else {
                    RHS1 = Crra + Chha * (ri * ri) + 0.5 * C[IX(i, k)] / (Ptl * dt);
                    cf1 = 0.5 / (Ptl * dt) - cnr - cnh;
                }
                RHS2 = s->variant == ORC_OBLIQUE ? -Ra * thr * (double)0.707106781f : -Ra * thh;
            }
            const double ULT = (u * Cr + v * Ch * ri) / Ptl;
            const double cf2 = cnr + cnh;
            s->Cn[IX(i, k)] = (cf2 * Cp[IX(i, k)] - ULT - RHS2 + RHS1) / cf1;
            if (!first) s->Ap[IX(i, k)] = s->Cn[IX(i, k)];
        }
    }
}

/* Robert filter coefficient: 0.02 in PRB (PRB:1041-1045), 0.05 in the
 * annulus driver (velvor2dnewsch3.4.f:1055, :1454). */
static double robert(const orc_prb_t *s)
{
    return s->variant == ORC_ANNULUS ? 0.05 : s->variant == ORC_TAYCOU ? 0.01 : 0.02;
}

static void *wbuf(int n, double **wa, double **wb, double **wc, double **wr, double **ws)
{
    double *b = (double *)malloc(sizeof(double) * (size_t)(n + 2) * 5);
    *wa = b; *wb = b + (n + 2); *wc = b + 2 * (n + 2); *wr = b + 3 * (n + 2); *ws = b + 4 * (n + 2);
    return b;
}

/* Cvorticity1, PRB:584-778: first (forward) step; no Robert filter. */
void orc_cvorticity1(orc_prb_t *s)
{
    double *wa, *wb, *wc, *wr, *ws;
    void *b = wbuf(s->np + s->nr + 2, &wa, &wb, &wc, &wr, &ws);
    cvort_derivatives(s, wa, wb, wc, wr, ws);
    cvort_update(s, 1);
    free(b);
}

/* Cvorticity, PRB:786-1048: leapfrog step followed by the Robert filter
 * C += 0.02 (Cn - 2C + Cp) on i=1..nr-1 (PRB:1041-1045). */
void orc_cvorticity(orc_prb_t *s)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    double *wa, *wb, *wc, *wr, *ws;
    void *b = wbuf(s->np + s->nr + 2, &wa, &wb, &wc, &wr, &ws);
    cvort_derivatives(s, wa, wb, wc, wr, ws);
    cvort_update(s, 0);
    for (int i = 1; i <= nr - 1; ++i)
        for (int k = 0; k <= np; ++k)
            s->C[IX(i, k)] = s->C[IX(i, k)] + robert(s) * (s->Cn[IX(i, k)] - 2.0 * s->C[IX(i, k)] + s->Cp[IX(i, k)]);
    free(b);
}

/* Compact derivatives of T at T points (PRB:1078-1120 / PRB:1244-1289):
 * thr -> A with third-order wall rows, thh -> B. */
static void temp_derivatives(orc_prb_t *s, double *wa, double *wb, double *wc,
                             double *wr, double *ws)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const double dri = 1.0 / s->dr, dpi = 1.0 / s->dp;
    const double *th = s->th;
    for (int k = 0; k <= np; ++k) {
        for (int i = 1; i <= nr; ++i) {
            wa[i - 1] = 1.0; wb[i - 1] = 4.0; wc[i - 1] = 1.0;
            if (i == 1) {
                wb[i - 1] = 1.0;
                wc[i - 1] = 2.0;
                wr[i - 1] = dri * (0.533333333 * th[IX(0, k)] - 3.6 * th[IX(1, k)] +
                                   2.966666667 * th[IX(2, k)] + 0.1 * th[IX(4, k)]);
            } else if (i == nr) {
                wa[i - 1] = 2.0;
                wb[i - 1] = 1.0;
                wr[i - 1] = dri * (-0.1 * th[IX(nr - 3, k)] - 2.966666667 * th[IX(nr - 1, k)] +
                                   3.6 * th[IX(nr, k)] - 0.533333333 * th[IX(nr + 1, k)]);
            } else {
                wr[i - 1] = 3.0 * (th[IX(i + 1, k)] - th[IX(i - 1, k)]) * dri;
            }
        }
        orc_tdma(wa, wb, wc, ws, wr, nr);
        for (int ii = 1; ii <= nr; ++ii) s->A[IX(ii, k)] = ws[ii - 1];
    }
    for (int i = 1; i <= nr; ++i) {
        for (int k = 0; k <= np; ++k) {
            wa[k] = 1.0; wb[k] = 4.0; wc[k] = 1.0;
            if (k == np) wr[np] = 3.0 * (th[IX(i, 1)] - th[IX(i, np - 1)]) * dpi;
            else if (k == 0) wr[0] = 3.0 * (th[IX(i, 1)] - th[IX(i, np - 1)]) * dpi;
            else wr[k] = 3.0 * (th[IX(i, k + 1)] - th[IX(i, k - 1)]) * dpi;
        }
        orc_ptdma(wa, wb, wc, ws, wr, np + 1);
        for (int kk = 0; kk <= np; ++kk) s->B[IX(i, kk)] = ws[kk];
    }
}

/* Temperature update, PRB:1292-1377 (first == 1, forward step) and
 * PRB:1292-1377 of `temperature` (first == 0, Dufort-Frankel).
 * ORC_ANNULUS (velvor2dnewsch3.4.f:1140-1223, :1308-1393): cell-centre
 * radius r = r0 + (i-1/2) dr and the (1/r) dT/dr term thra*ri in RHS1. */
static void temp_update(orc_prb_t *s, int first)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const int polar = prb_polar(s);
    const double dri = 1.0 / s->dr, dpi = 1.0 / s->dp, dt = s->dt;
    const double *th = s->th, *thp = s->thp, *uel = s->uel, *vel = s->vel;
    for (int i = 1; i <= nr; ++i) {
        for (int k = 0; k <= np; ++k) {
            const int im = i - 1;
            int km = k - 1, ka = k + 1;
            if (k == 0) km = np - 1;
            if (k == np) ka = 1;
            const double r = polar ? s->r0 + ((double)i - 0.5) * s->dr : 1.0, ri = 1.0 / r;
            const double u = (uel[IX(i, k)] + uel[IX(im, k)]) * 0.5;
            const double v = (vel[IX(i, k)] + vel[IX(i, km)]) * 0.5;
            double thrra, thra, cnr;
            const double thr = s->A[IX(i, k)];
            if (i == 1) {
                thrra = (3.2 * th[IX(i - 1, k)] + 2.0 * th[IX(i + 1, k)] - 0.2 * th[IX(i + 2, k)]) * (dri * dri);
                thra = (-4.0 * th[IX(i - 1, k)] / 3.0 + th[IX(i + 1, k)] / 3.0) * dri;
                cnr = -2.5 * (dri * dri) + 0.5 * dri * ri;
            } else if (i == nr) {
                thrra = (3.2 * th[IX(i + 1, k)] + 2.0 * th[IX(i - 1, k)] - 0.2 * th[IX(i - 2, k)]) * (dri * dri);
                thra = (-th[IX(i - 1, k)] / 3.0 + 4.0 * th[IX(i + 1, k)] / 3.0) * dri;
                cnr = -2.5 * (dri * dri) - 0.5 * dri * ri;
            } else {
                thrra = (th[IX(i - 1, k)] + th[IX(i + 1, k)]) * (dri * dri);
                thra = (th[IX(i + 1, k)] - th[IX(i - 1, k)]) * 0.5 * dri;
                cnr = -1.0 * (dri * dri);
            }
            const double thhha = (th[IX(i, ka)] + th[IX(i, km)]) * (dpi * dpi);
            const double thh = s->B[IX(i, k)];
            const double cnp = -(1.0 * (dpi * dpi)) * (ri * ri);
            double RHS1, cf1;
            if (polar) {
                if (first) {
                    RHS1 = thrra + thra * ri + thhha * (ri * ri) + th[IX(i, k)] / dt;
                    cf1 = 1.0 / dt - cnr - cnp;
                } else {
                    RHS1 = thrra + thra * ri + thhha * (ri * ri) + 0.5 * thp[IX(i, k)] / dt;
                    cf1 = 0.5 / dt - cnr - cnp;
                }
            } else if (first) {
                RHS1 = thrra + thhha * (ri * ri) + th[IX(i, k)] / dt;
                cf1 = 1.0 / dt - cnr - cnp;
            } else {
                RHS1 = thrra + thhha * (ri * ri) + 0.5 * thp[IX(i, k)] / dt;
                cf1 = 0.5 / dt - cnr - cnp;
            }
            const double ULT = u * thr + v * thh * ri;
            const double cf2 = cnr + cnp;
            s->thn[IX(i, k)] = (cf2 * thp[IX(i, k)] - ULT + RHS1) / cf1;
            if (!first) s->Ap[IX(i, k)] = s->thn[IX(i, k)];
        }
    }
}

/* temperature1, PRB:1056-1212. */
void orc_temperature1(orc_prb_t *s)
{
    double *wa, *wb, *wc, *wr, *ws;
    void *b = wbuf(s->np + s->nr + 2, &wa, &wb, &wc, &wr, &ws);
    temp_derivatives(s, wa, wb, wc, wr, ws);
    temp_update(s, 1);
    free(b);
}

/* temperature, PRB:1220-1443, Robert filter PRB:1435-1440. */
void orc_temperature(orc_prb_t *s)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    double *wa, *wb, *wc, *wr, *ws;
    void *b = wbuf(s->np + s->nr + 2, &wa, &wb, &wc, &wr, &ws);
    temp_derivatives(s, wa, wb, wc, wr, ws);
    temp_update(s, 0);
    for (int i = 1; i <= nr; ++i)
        for (int k = 0; k <= np; ++k)
            s->th[IX(i, k)] = s->th[IX(i, k)] + robert(s) * (s->thn[IX(i, k)] - 2.0 * s->th[IX(i, k)] + s->thp[IX(i, k)]);
    free(b);
}

/* Wall heat fluxes, heat PRB:1452-1500: five-point one-sided derivative at
 * each wall, trapezoid over k = 1..np. */
void orc_heat(const orc_prb_t *s, double *trans1, double *trans2)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const double dri = 1.0 / s->dr, dp = s->dp;
    const double *th = s->th;
    double t1 = 0.0, t2 = 0.0;
    for (int k = 1; k <= np; ++k) {
        int ka = k + 1;
        if (k == np) ka = 1;
        t1 = t1 + 0.5 * dp * (-3.35238095 * th[IX(0, k)] + 4.375 * th[IX(1, k)] - 1.45833333 * th[IX(2, k)] +
                              0.525 * th[IX(3, k)] - 0.08928571 * th[IX(4, k)]) * dri +
             0.5 * dp * (-3.35238095 * th[IX(0, ka)] + 4.375 * th[IX(1, ka)] - 1.45833333 * th[IX(2, ka)] +
                         0.525 * th[IX(3, ka)] - 0.08928571 * th[IX(4, ka)]) * dri;
        t2 = t2 + 0.5 * dp * (-3.35238095 * th[IX(nr + 1, k)] + 4.375 * th[IX(nr, k)] - 1.45833333 * th[IX(nr - 1, k)] +
                              0.525 * th[IX(nr - 2, k)] - 0.08928571 * th[IX(nr - 3, k)]) * dri +
             0.5 * dp * (-3.35238095 * th[IX(nr + 1, ka)] + 4.375 * th[IX(nr, ka)] - 1.45833333 * th[IX(nr - 1, ka)] +
                         0.525 * th[IX(nr - 2, ka)] - 0.08928571 * th[IX(nr - 3, ka)]) * dri;
    }
    *trans1 = t1;
    *trans2 = t2;
}

/* update, PRB:1557-1626: wall vorticity from the new v, T walls, time-level
 * rotation over i = 0..nr+1 and the clamp of T to (0.01, 0.99). */
void orc_update(orc_prb_t *s)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const double dr = s->dr;
    for (int k = 0; k <= np; ++k) {
        s->Bn[IX(0, k)] = -(3.0 * s->wel[IX(1, k)] - s->wel[IX(2, k)] / 3.0) / dr;
        s->Bn[IX(nr, k)] = -(s->wel[IX(nr - 1, k)] / 3.0 - 3.0 * s->wel[IX(nr, k)]) / dr;
    }
    for (int k = 0; k <= np; ++k) {
        if (s->variant == ORC_TAYCOU) {
            /* velvor2dtaycouheat.f:1587-1590: the moving outer wall */
            s->vel[IX(nr + 1, k)] = taycou_wall(s);
            s->Cn[IX(0, k)] = (3.0 * s->vel[IX(1, k)] - s->vel[IX(2, k)] / 3.0) / dr;
            s->Cn[IX(nr, k)] = (8.0 / 3.0 * s->vel[IX(nr + 1, k)] + s->vel[IX(nr - 1, k)] / 3.0 -
                                3.0 * s->vel[IX(nr, k)]) / dr + s->vel[IX(nr + 1, k)] / s->rmax;
            continue;
        }
        s->Cn[IX(0, k)] = (3.0 * s->vel[IX(1, k)] - s->vel[IX(2, k)] / 3.0) / dr;
        s->Cn[IX(nr, k)] = (s->vel[IX(nr - 1, k)] / 3.0 - 3.0 * s->vel[IX(nr, k)]) / dr;
    }
    for (int k = 0; k <= np; ++k) {
        s->thn[IX(0, k)] = 0.0;
        s->thn[IX(nr + 1, k)] = 1.0;
    }
    for (int i = 0; i <= nr + 1; ++i) {
        for (int k = 0; k <= np; ++k) {
            s->Cp[IX(i, k)] = s->C[IX(i, k)];
            s->C[IX(i, k)] = s->Cn[IX(i, k)];
            s->thp[IX(i, k)] = s->th[IX(i, k)];
            if (s->thn[IX(i, k)] > 1.0) { s->thn[IX(i, k)] = 0.99; s->clamp_count++; }
            if (s->thn[IX(i, k)] < 0.0) { s->thn[IX(i, k)] = 0.01; s->clamp_count++; }
            s->th[IX(i, k)] = s->thn[IX(i, k)];
        }
    }
}

/* rhsv, PRB:1629-1676: v-equation source dCn/dr on i = 1..nr with the
 * one-sided rows of the reference at i = 1 and i = nr.  ORC_ANNULUS
 * (velvor2dnewsch3.4.f:1666-1686) adds the polar terms Cn/r at the
 * cell-centre radius r = r0 + (i-1/2) dr. */
void orc_rhsv(orc_prb_t *s)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const double dr = s->dr;
    const int polar = prb_polar(s);
    for (int i = 1; i <= nr; ++i) {
        for (int k = 0; k <= np; ++k) {
            const double Cr = (s->Cn[IX(i, k)] - s->Cn[IX(i - 1, k)]) / dr;
            if (polar) {
                const double r = s->r0 + ((double)i - 0.5) * dr;
                if (i == 1) s->vrh[IX(i, k)] = s->Cn[IX(1, k)] / dr + s->Cn[IX(1, k)] / r;
                else if (i == nr) {
                    s->vrh[IX(i, k)] = -s->Cn[IX(nr - 1, k)] / dr + s->Cn[IX(nr - 1, k)] / r;
                    if (s->variant == ORC_TAYCOU) {
                        /* velvor2dtaycouheat.f:1668-1670, hhri = hri**2.d0, rvali**2.d0 */
                        const double velo = taycou_wall(s), rvali = 1.0 / s->rmax, hri = 1.0 / dr;
                        const double hhri = hri * hri;
                        s->vrh[IX(i, k)] = s->vrh[IX(i, k)] - 8.0 / 15.0 * velo * hhri + rvali * hri * velo -
                                           4.0 / 3.0 * velo * hri * rvali + velo * (rvali * rvali);
                    }
                }
                else s->vrh[IX(i, k)] = Cr + (s->Cn[IX(i, k)] + s->Cn[IX(i - 1, k)]) / r;
            } else if (i == 1) s->vrh[IX(i, k)] = s->Cn[IX(1, k)] / dr;
            else if (i == nr) s->vrh[IX(i, k)] = -s->Cn[IX(nr - 1, k)] / dr;
            else s->vrh[IX(i, k)] = Cr;
        }
    }
}

/* rhsu, PRB:1679-1721: u-equation source -dCn/dx / r on i = 1..nr-1, with
 * r = 1 in PRB and the face radius r = r0 + i dr in the annulus
 * (velvor2dnewsch3.4.f:1710-1730). */
void orc_rhsu(orc_prb_t *s)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const int polar = prb_polar(s);
    for (int i = 1; i <= nr - 1; ++i) {
        for (int k = 0; k <= np; ++k) {
            int km = k - 1;
            if (k == 0) km = np - 1;
            const double r = polar ? s->r0 + (double)i * s->dr : 1.0;
            const double Ch = (s->Cn[IX(i, k)] - s->Cn[IX(i, km)]) / s->dp;
            s->urh[IX(i, k)] = -Ch / r;
        }
    }
}

/* The annulus solves never stop the run: after nvs sweeps poisson2 and
 * poisson3 return with psi untouched and the step goes on
 * (velvor2dnewsch3.4.f:1853-1936, :1984-2068). */
static int solve_failed(const orc_prb_t *s, int st)
{
    return st != ORC_OK && !(s->variant == ORC_ANNULUS && st == ORC_MAXSWEEPS);
}

static int tank_step(orc_prb_t *s, orc_mg_t *mgv, orc_mg_t *mgu, int kt, double *nu, int *sweeps)
{
    double t1, t2;
    int sv = 0, su = 0, st;
    orc_tank_cvorticity(s, kt == 1);
    orc_tank_temperature(s, kt == 1);
    orc_tank_heat(s, &t1, &t2);
    orc_tank_rhsv(s);
    st = orc_poisson(mgv, 2, s->vel, s->velp, s->vrh, s->ld, &sv);
    if (st != ORC_OK) { if (sweeps) { sweeps[0] = sv; sweeps[1] = 0; } return st; }
    orc_tank_rhsu(s);
    st = orc_poisson(mgu, 3, s->uel, s->uelp, s->urh, s->ld, &su);
    if (st != ORC_OK) { if (sweeps) { sweeps[0] = sv; sweeps[1] = su; } return st; }
    orc_tank_update(s);
    if (nu) {
        /* velvor2dhorconvtank.f:197-198, :209-210: the first step overwrites
         * httrans with 2 trans2 and leaves httrans2 at zero; the DVD cavity
         * (velvor2ddvdbenchmark.f:197-210) the same without the factor 2 */
        const double c = s->variant == ORC_DVD ? 1.0 : 2.0;
        if (kt == 1) {
            nu[0] = s->variant == ORC_DVD ? t2 : t2 * c;
            nu[1] = 0.0;
        } else {
            nu[0] = s->variant == ORC_DVD ? t1 : t1 * c;
            nu[1] = s->variant == ORC_DVD ? t2 : t2 * c;
        }
    }
    if (sweeps) { sweeps[0] = sv; sweeps[1] = su; }
    return ORC_OK;
}

int orc_prb_step(orc_prb_t *s, orc_mg_t *mgv, orc_mg_t *mgu, int kt, double *nu, int *sweeps)
{
    double t1, t2;
    int sv = 0, su = 0, st;
    if (s->variant == ORC_TANK || s->variant == ORC_DVD) return tank_step(s, mgv, mgu, kt, nu, sweeps);
    if (kt == 1) {
        orc_cvorticity1(s);
        orc_temperature1(s);
    } else {
        orc_cvorticity(s);
        orc_temperature(s);
    }
    orc_heat(s, &t1, &t2);
    orc_rhsv(s);
    st = orc_poisson(mgv, 2, s->vel, s->velp, s->vrh, s->ld, &sv);
    if (solve_failed(s, st)) { if (sweeps) { sweeps[0] = sv; sweeps[1] = 0; } return st; }
    orc_rhsu(s);
    st = orc_poisson(mgu, 3, s->uel, s->uelp, s->urh, s->ld, &su);
    if (solve_failed(s, st)) { if (sweeps) { sweeps[0] = sv; sweeps[1] = su; } return st; }
    orc_update(s);
    if (nu) {
        if (prb_polar(s)) {
            /* httrans, httrans2 of velvor2dnewsch3.4.f:386-387 (velvor2dtaycouheat.f alike) */
            const double pi = acos(-1.0), L = log(s->r0 / s->rmax);
            nu[0] = -s->r0 * L * t1 / (2.0 * pi);
            nu[1] = -s->rmax * L * t2 / (2.0 * pi);
        } else {
            nu[0] = t1 * (s->rmax - s->r0) / s->xx;
            nu[1] = t2 * (s->rmax - s->r0) / s->xx;
        }
    }
    if (sweeps) { sweeps[0] = sv; sweeps[1] = su; }
    return ORC_OK;
}

/* Running means of the zonal-mean time-mean diagnostics (PRB:404-416).  The
 * reference keeps them in borrowed arrays (weln, welp, Bp, vrms); x**2.d0 is
 * x*x. */
void orc_prb_diag_accum(const orc_prb_t *s, int kt, double *msqT, double *mT, double *msqU, double *msqV)
{
    if (kt < 2) return;
    const int ld = s->ld;
    const double tkti = 1.0 / (double)(kt - 1);
    const double w = (double)(kt - 2);
    for (int i = 0; i <= s->nr + 1; ++i)
        for (int k = 0; k <= s->np; ++k) {
            const size_t c = (size_t)i + (size_t)ld * (size_t)k;
            const double th = s->th[c], u = s->uel[c], v = s->vel[c];
            msqT[c] = tkti * msqT[c] * w + tkti * (th * th);
            mT[c] = tkti * mT[c] * w + tkti * th;
            msqU[c] = tkti * msqU[c] * w + tkti * (u * u);
            msqV[c] = tkti * msqV[c] * w + tkti * (v * v);
        }
}

/* CFL scans (PRB:420-459; the annulus radius of velvor2dnewsch3.4.f:437-445). */
void orc_prb_cfl(const orc_prb_t *s, double *cflu, double *cflv)
{
    const int ld = s->ld;
    double mu = 0.0, mv = 0.0;
    for (int i = 1; i <= s->nr; ++i)
        for (int k = 0; k <= s->np; ++k) {
            const double cfl = fabs(s->uel[(size_t)i + (size_t)ld * (size_t)k] * s->dt / s->dr);
            if (cfl > mu) mu = cfl;
        }
    for (int i = 1; i <= s->nr - 1; ++i) {
        const double r = prb_polar(s) ? s->r0 + ((double)i - 0.5) * s->dr : 1.0;
        for (int k = 0; k <= s->np; ++k) {
            const double cfl = fabs(s->vel[(size_t)i + (size_t)ld * (size_t)k] * s->dt / (r * s->dp));
            if (cfl > mv) mv = cfl;
        }
    }
    *cflu = mu;
    *cflv = mv;
}

/* Zonal means written to zmtmtempvar.dat (PRB:474-493). */
void orc_prb_zmtm(const orc_prb_t *s, const double *msqT, const double *mT, const double *msqU,
                  const double *msqV, double *out)
{
    const int ld = s->ld;
    const double n = (double)(s->np + 1);
    for (int i = 0; i <= s->nr + 1; ++i) {
        double a = 0.0, b = 0.0, cu = 0.0, cv = 0.0;
        for (int k = 0; k <= s->np; ++k) {
            const size_t c = (size_t)i + (size_t)ld * (size_t)k;
            a = a + msqT[c];
            b = b + mT[c] * mT[c];
            cu = cu + msqU[c];
            cv = cv + msqV[c];
        }
        out[3 * i + 0] = (a - b) / n;
        out[3 * i + 1] = pow(cu / n, 0.5);
        out[3 * i + 2] = pow(cv / n, 0.5);
    }
}

/* splitmix64 (Steele, Lea, Flood 2014), used for the seeded noise. */
static unsigned long long splitmix64(unsigned long long *state)
{
    unsigned long long z = (*state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

void orc_prb_initial(orc_prb_t *s, int kind, unsigned long long seed, double amp)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const double r0 = s->r0, rmax = s->rmax, dr = s->dr;
    unsigned long long st = seed;
    for (int k = 0; k <= np; ++k) {
        for (int i = 0; i <= nr + 1; ++i) {
            double r;
            if (i == 0) r = r0;
            else if (i == nr + 1) r = rmax;
            else r = r0 + ((double)i - 0.5) * dr;
            s->An[IX(i, k)] = s->Bn[IX(i, k)] = s->Cn[IX(i, k)] = 0.0;
            s->A[IX(i, k)] = s->B[IX(i, k)] = s->C[IX(i, k)] = 0.0;
            s->uel[IX(i, k)] = s->vel[IX(i, k)] = s->wel[IX(i, k)] = 0.0;
            if (kind == 0 && prb_polar(s)) {
                /* velvor2dnewsch3.4.f:130-178: conduction profile 1 - ln r / ln r0
                 * with walls 0 and 1 and the ripple 0.7 T (r-rmax)/rmax (2 randno - 1),
                 * randno = 1/2 + sin(2 pi k/150)/2.  The blobs of :185-220 have
                 * amplitude -0.0 and leave T unchanged. */
                const double pi = acos(-1.0);
                double t = 1.0 - log(r) / log(r0);
                if (i == 0) t = 0.0;
                else if (i == nr + 1) t = 1.0;
                else {
                    double randno = 0.5 + 0.5 * sin((double)k / 150.0 * 2.0 * pi);
                    t = t + (r - rmax) / rmax * ((randno * 2.0) - 1.0) * 0.7 * t;
                }
                s->th[IX(i, k)] = t;
            } else if (kind == 0) {
                /* PRB:156-186: T = 2(r-r0) plus a deterministic sine ripple whose
                 * 0.01 is a REAL*4 literal.  The Gaussian blobs of PRB:193-227 have
                 * amplitude -0.0 and leave T unchanged. */
                double t = 2.0 * (r - r0);
                if (i == 0) t = 0.0;
                else if (i == nr + 1) t = 1.0;
                else {
                    double randno = 0.5 + 0.5 * sin((double)k / (double)np);
                    t = t + (r - r0) / rmax * (double)0.01f * ((randno * 2.0) - 1.0);
                }
                s->th[IX(i, k)] = t;
            }
        }
    }
    if (kind == 1) {
        for (int k = 0; k <= np; ++k) {
            for (int i = 0; i <= nr + 1; ++i) {
                double r = r0 + ((double)i - 0.5) * dr;
                double t;
                if (i == 0) t = 0.0;
                else if (i == nr + 1) t = 1.0;
                else if (k == np) t = s->th[IX(i, 0)];
                else {
                    double u = (double)(splitmix64(&st) >> 11) * (1.0 / 9007199254740992.0);
                    if (prb_polar(s)) t = 1.0 - log(r) / log(r0) + amp * (2.0 * u - 1.0);
                    else t = (r - r0) / (rmax - r0) + amp * (2.0 * u - 1.0);
                }
                s->th[IX(i, k)] = t;
            }
        }
    }
    if (s->variant == ORC_TAYCOU)   /* the moving outer wall of the start, velvor2dtaycouheat.f:177 */
        for (int k = 0; k <= np; ++k) s->vel[IX(nr + 1, k)] = taycou_wall(s);
    for (int k = 0; k <= np; ++k) {
        for (int i = 0; i <= nr + 1; ++i) {
            s->Ap[IX(i, k)] = s->A[IX(i, k)];
            s->Bp[IX(i, k)] = s->B[IX(i, k)];
            s->Cp[IX(i, k)] = s->C[IX(i, k)];
            s->thp[IX(i, k)] = s->th[IX(i, k)];
            s->uelp[IX(i, k)] = s->uel[IX(i, k)];
            s->velp[IX(i, k)] = s->vel[IX(i, k)];
            s->welp[IX(i, k)] = 0.0;
        }
    }
}
