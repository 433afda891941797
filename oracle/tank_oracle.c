/*
 * CPU oracle for the horizontal-convection tank of
 * monashubuntudir_velvor2dhorconvtankdir/velvor2dhorconvtank.f ("TANK"):
 * the 2D layer's scheme closed by side walls at x = 0 and x = xx (3.1).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of tests/; never linked into the
 * product.  PARITY PINNED: reproduces bit for bit velvor2dhorconvtank.f and
 * velvor2ddvdbenchmark.f run through the translator tests/golden/f77.py
 * (tests/test_reference_runs.py).
 * Double precision, the reference's order, -ffp-contract=off; REAL*4
 * literals (1./6., 4./3.) are the floats they round to.
 *
 * Staggering in x: C and v on faces k = 0..np (walls k = 0, np), T and u on
 * cells k = 1..np with ghost columns k = 0 and np+1 (the fields carry
 * np+2 columns).  What differs from the periodic layer (PRB):
 *   Cvorticity1/Cvorticity (:334-575): x-derivatives by the plain Thomas
 *     algorithm over k = 1..np-1 (no periodic closure); dT/dr at the C
 *     points with 3 (not 1.5) times the differences and no wall correction
 *     at i = 1; the update on k = 1..np-1; the leapfrog RHS1 takes 0.5 Cp
 *     (PRB takes C); Robert filter 0.02 on i = 1..nr-1, k = 1..np-1;
 *   temperature1/temperature (:582-770): k = 1..np, Thomas over np cells in
 *     x, the insulated-wall row -8 T0 + 6 T1 + 1.9 T2 + 0.1 T4 at i = 1,
 *     no 0.5 dr^-1 / r term in cnr at the wall rows, Robert filter on
 *     i = 0..nr, k = 1..np;
 *   heat (:778-799): the PRB flux formula over k = np/2..np-1;
 *   update (:812-845): wall vorticity on k = 1..np-1, C = 0 on the side
 *     walls, T at i = 0 from the insulated closure, T = k/np at i = nr+1,
 *     T ghosts 4/3 T(1) - 1/3 T(2) on both sides, no B wall rows;
 *   rhsv on k = 1..np-1, rhsu on k = 1..np (:867-910);
 *   poisson2/poisson3 and relax2/relax3: see the xwall field of orc_mg_t;
 *   main (:188-210): Nu = 2 trans; the first step stores 2 trans2 in
 *     httrans and leaves httrans2 at zero.
 *
 * ORC_DVD, the differentially heated cavity of
 * monashubuntudir_velvor2ddvdbenchmarkdir/velvor2ddvdbenchmark.f, is the
 * same scheme with: xx = 1; the start T = 0.5 inside, 0 at i = 0, 1 at
 * i = nr+1; the wall correction -(-4/3 (T0) + 1.5 (T1) - 1/6 (T2)) dr^-1 of
 * dT/dr at the C points at i = 1 (:382-383, REAL*4 4./3. and 1./6.);
 * buoyancy RHS2 = -Ra thr (:437, :560); the T derivative's wall row
 * 0.5333333333 T0 - 3.6 T1 + 2.9666666667 T2 + 0.1 T4 at i = 1 (:601,
 * :696); the Robert filter of T on i = 1..nr (:763); heat over
 * k = 2..np-1 (:780); the side-wall vorticities -u(1)/dp and u(np)/dp
 * (:819-820); T = 0 and 1 on the bottom and top rows including the ghost
 * columns, and the insulated closure on the side ghosts (:822-830);
 * Nu = trans.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "prb_oracle.h"

#define IX(i, k) ((size_t)(i) + (size_t)ld * (size_t)(k))

static const double F16 = (double)(1.0f / 6.0f);
static const double F43 = (double)(4.0f / 3.0f);

static int is_dvd(const orc_prb_t *s) { return s->variant == ORC_DVD; }

static double *tank_buf(int n, double **wa, double **wb, double **wc, double **wr, double **ws)
{
    double *b = (double *)malloc(sizeof(double) * 5 * (size_t)(n + 2));
    *wa = b;
    *wb = b + (n + 2);
    *wc = b + 2 * (n + 2);
    *wr = b + 3 * (n + 2);
    *ws = b + 4 * (n + 2);
    return b;
}

/* Cvorticity1 (first = 1, :334-455) and Cvorticity (first = 0, :457-575). */
void orc_tank_cvorticity(orc_prb_t *s, int first)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const double dri = 1.0 / s->dr, dpi = 1.0 / s->dp;
    const double Ptl = s->Pr, dt = s->dt, Ra = s->Ra;
    double *wa, *wb, *wc, *wr, *ws;
    double *buf = tank_buf(nr > np ? nr : np, &wa, &wb, &wc, &wr, &ws);
    const double *C = s->C, *Cp = s->Cp, *th = s->th, *uel = s->uel, *vel = s->vel;
    /* Cr -> A: tdma along r, k = 1..np-1 */
    for (int k = 1; k <= np - 1; ++k) {
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
    /* Ch -> B: tdma along x over k = 1..np-1 */
    for (int i = 1; i <= nr - 1; ++i) {
        for (int k = 1; k <= np - 1; ++k) {
            wa[k - 1] = 1.0; wb[k - 1] = 4.0; wc[k - 1] = 1.0;
            wr[k - 1] = 3.0 * (C[IX(i, k + 1)] - C[IX(i, k - 1)]) * dpi;
        }
        orc_tdma(wa, wb, wc, ws, wr, np - 1);
        for (int kk = 1; kk <= np - 1; ++kk) s->B[IX(i, kk)] = ws[kk - 1];
    }
    /* thr at the C points -> An */
    for (int k = 1; k <= np - 1; ++k) {
        const int ka = k + 1;
        for (int i = 1; i <= nr - 1; ++i) {
            wa[i - 1] = 1.0; wb[i - 1] = 4.0; wc[i - 1] = 1.0;
            if (i == 1 && is_dvd(s))
                wr[i - 1] = 3.0 * (th[IX(2, k)] + th[IX(2, ka)] - th[IX(1, k)] - th[IX(1, ka)]) * dri -
                            (-F43 * (th[IX(0, k)] + th[IX(0, ka)]) + 1.5 * (th[IX(1, k)] + th[IX(1, ka)]) -
                             F16 * (th[IX(2, k)] + th[IX(2, ka)])) * dri;
            else if (i == 1)
                wr[i - 1] = 3.0 * (th[IX(2, k)] + th[IX(2, ka)] - th[IX(1, k)] - th[IX(1, ka)]) * dri;
            else if (i == nr - 1)
                wr[i - 1] = 3.0 * (th[IX(nr, k)] + th[IX(nr, ka)] - th[IX(nr - 1, k)] - th[IX(nr - 1, ka)]) * dri -
                            (F16 * (th[IX(nr - 1, k)] + th[IX(nr - 1, ka)]) - 1.5 * (th[IX(nr, k)] + th[IX(nr, ka)]) +
                             F43 * (th[IX(nr + 1, k)] + th[IX(nr + 1, ka)])) * dri;
            else
                wr[i - 1] = 3.0 * (th[IX(i + 1, k)] + th[IX(i + 1, ka)] - th[IX(i, k)] - th[IX(i, ka)]) * dri;
        }
        orc_tdma(wa, wb, wc, ws, wr, nr - 1);
        for (int ii = 1; ii <= nr - 1; ++ii) s->An[IX(ii, k)] = ws[ii - 1];
    }
    /* thh at the C points -> Bn: tdma along x over k = 1..np-1 */
    for (int i = 1; i <= nr - 1; ++i) {
        for (int k = 1; k <= np - 1; ++k) {
            const int ka = k + 1;
            wa[k - 1] = 1.0; wb[k - 1] = 4.0; wc[k - 1] = 1.0;
            wr[k - 1] = 3.0 * (th[IX(i + 1, ka)] + th[IX(i, ka)] - th[IX(i + 1, k)] - th[IX(i, k)]) * dpi;
        }
        orc_tdma(wa, wb, wc, ws, wr, np - 1);
        for (int kk = 1; kk <= np - 1; ++kk) s->Bn[IX(i, kk)] = ws[kk - 1];
    }
    free(buf);
    /* the update on k = 1..np-1, r = 1 */
    for (int k = 1; k <= np - 1; ++k)
        for (int i = 1; i <= nr - 1; ++i) {
            const int ip = i + 1, km = k - 1, ka = k + 1;
            const double ri = 1.0 / 1.0;
            const double u = (uel[IX(i, ka)] + uel[IX(i, k)]) * 0.5;
            const double v = (vel[IX(i, k)] + vel[IX(ip, k)]) * 0.5;
            const double Chha = (C[IX(i, ka)] + C[IX(i, km)]) * (dpi * dpi);
            const double Ch = s->B[IX(i, k)];
            const double Crra = (C[IX(i - 1, k)] + C[IX(i + 1, k)]) * (dri * dri);
            const double cnr = -1.0 * (dri * dri);
            const double Cr = s->A[IX(i, k)];
            const double thh = s->Bn[IX(i, k)];
            const double cnh = (-1.0 * (dpi * dpi)) * (ri * ri);
            double RHS1, cf1;
            if (first) {
                RHS1 = Crra + Chha * (ri * ri) + C[IX(i, k)] / (Ptl * dt);
                cf1 = 1.0 / (Ptl * dt) - cnr - cnh;
            } else {
                RHS1 = Crra + Chha * (ri * ri) + 0.5 * Cp[IX(i, k)] / (Ptl * dt);
                cf1 = 0.5 / (Ptl * dt) - cnr - cnh;
            }
            const double ULT = (u * Cr + v * Ch * ri) / Ptl;
            const double RHS2 = is_dvd(s) ? -Ra * s->An[IX(i, k)] : -Ra * thh;
            const double cf2 = cnr + cnh;
            s->Cn[IX(i, k)] = (cf2 * Cp[IX(i, k)] - ULT - RHS2 + RHS1) / cf1;
            if (!first) s->Ap[IX(i, k)] = s->Cn[IX(i, k)];
        }
    if (!first)
        for (int i = 1; i <= nr - 1; ++i)
            for (int k = 1; k <= np - 1; ++k)
                s->C[IX(i, k)] = s->C[IX(i, k)] + 0.02 * (s->Cn[IX(i, k)] - 2.0 * s->C[IX(i, k)] + s->Cp[IX(i, k)]);
}

/* temperature1 (first = 1, :582-675) and temperature (first = 0, :677-770). */
void orc_tank_temperature(orc_prb_t *s, int first)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const double dri = 1.0 / s->dr, dpi = 1.0 / s->dp, dt = s->dt;
    double *wa, *wb, *wc, *wr, *ws;
    double *buf = tank_buf(nr > np ? nr : np, &wa, &wb, &wc, &wr, &ws);
    const double *th = s->th, *thp = s->thp, *uel = s->uel, *vel = s->vel;
    /* thr -> A: tdma along r over i = 1..nr, k = 1..np */
    for (int k = 1; k <= np; ++k) {
        for (int i = 1; i <= nr; ++i) {
            wa[i - 1] = 1.0; wb[i - 1] = 4.0; wc[i - 1] = 1.0;
            if (i == 1) {
                wb[i - 1] = 1.0;
                wc[i - 1] = 2.0;
                if (is_dvd(s))
                    wr[i - 1] = dri * (0.5333333333 * th[IX(0, k)] - 3.6 * th[IX(1, k)] + 2.9666666667 * th[IX(2, k)] +
                                       0.1 * th[IX(4, k)]);
                else
                    wr[i - 1] = dri * (-8.0 * th[IX(0, k)] + 6.0 * th[IX(1, k)] + 1.9 * th[IX(2, k)] + 0.1 * th[IX(4, k)]);
            } else if (i == nr) {
                wa[i - 1] = 2.0;
                wb[i - 1] = 1.0;
                wr[i - 1] = dri * (-0.1 * th[IX(nr - 3, k)] - 2.966666667 * th[IX(nr - 1, k)] + 3.6 * th[IX(nr, k)] -
                                   0.533333333 * th[IX(nr + 1, k)]);
            } else {
                wr[i - 1] = 3.0 * (th[IX(i + 1, k)] - th[IX(i - 1, k)]) * dri;
            }
        }
        orc_tdma(wa, wb, wc, ws, wr, nr);
        for (int ii = 1; ii <= nr; ++ii) s->A[IX(ii, k)] = ws[ii - 1];
    }
    /* thh -> B: tdma along x over k = 1..np */
    for (int i = 1; i <= nr; ++i) {
        for (int k = 1; k <= np; ++k) {
            wa[k - 1] = 1.0; wb[k - 1] = 4.0; wc[k - 1] = 1.0;
            wr[k - 1] = 3.0 * (th[IX(i, k + 1)] - th[IX(i, k - 1)]) * dpi;
        }
        orc_tdma(wa, wb, wc, ws, wr, np);
        for (int kk = 1; kk <= np; ++kk) s->B[IX(i, kk)] = ws[kk - 1];
    }
    free(buf);
    for (int k = 1; k <= np; ++k)
        for (int i = 1; i <= nr; ++i) {
            const int ip = i + 1, im = i - 1, km = k - 1, ka = k + 1;
            const double ri = 1.0 / 1.0;
            const double u = (uel[IX(i, k)] + uel[IX(im, k)]) * 0.5;
            const double v = (vel[IX(i, k)] + vel[IX(i, km)]) * 0.5;
            double thrra, cnr;
            if (i == 1) {
                thrra = (3.2 * th[IX(i - 1, k)] + 2.0 * th[IX(i + 1, k)] - 0.2 * th[IX(i + 2, k)]) * (dri * dri);
                cnr = -2.5 * (dri * dri);
            } else if (i == nr) {
                thrra = (3.2 * th[IX(i + 1, k)] + 2.0 * th[IX(i - 1, k)] - 0.2 * th[IX(i - 2, k)]) * (dri * dri);
                cnr = -2.5 * (dri * dri);
            } else {
                thrra = (th[IX(i - 1, k)] + th[IX(ip, k)]) * (dri * dri);
                cnr = -1.0 * (dri * dri);
            }
            const double thr = s->A[IX(i, k)];
            const double thhha = (th[IX(i, ka)] + th[IX(i, km)]) * (dpi * dpi);
            const double thh = s->B[IX(i, k)];
            const double cnp = -(1.0 * (dpi * dpi)) * (ri * ri);
            double RHS1, cf1;
            if (first) {
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
    if (!first)
        for (int k = 1; k <= np; ++k)
            for (int i = is_dvd(s) ? 1 : 0; i <= nr; ++i)
                s->th[IX(i, k)] = s->th[IX(i, k)] + 0.02 * (s->thn[IX(i, k)] - 2.0 * s->th[IX(i, k)] + s->thp[IX(i, k)]);
}

/* heat (:778-799): the layer's flux formula over k = np/2..np-1. */
void orc_tank_heat(const orc_prb_t *s, double *trans1, double *trans2)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const double dp = s->dp, dri = 1.0 / s->dr;
    const double *th = s->th;
    double t1 = 0.0, t2 = 0.0;
    for (int k = is_dvd(s) ? 2 : np / 2; k <= np - 1; ++k) {
        const int ka = k + 1;
        t1 = t1 + 0.5 * dp *
                      (-3.35238095 * th[IX(0, k)] + 4.375 * th[IX(1, k)] - 1.45833333 * th[IX(2, k)] +
                       0.525 * th[IX(3, k)] - 0.08928571 * th[IX(4, k)]) * dri +
             0.5 * dp *
                 (-3.35238095 * th[IX(0, ka)] + 4.375 * th[IX(1, ka)] - 1.45833333 * th[IX(2, ka)] +
                  0.525 * th[IX(3, ka)] - 0.08928571 * th[IX(4, ka)]) * dri;
        t2 = t2 + 0.5 * dp *
                      (-3.35238095 * th[IX(nr + 1, k)] + 4.375 * th[IX(nr, k)] - 1.45833333 * th[IX(nr - 1, k)] +
                       0.525 * th[IX(nr - 2, k)] - 0.08928571 * th[IX(nr - 3, k)]) * dri +
             0.5 * dp *
                 (-3.35238095 * th[IX(nr + 1, ka)] + 4.375 * th[IX(nr, ka)] - 1.45833333 * th[IX(nr - 1, ka)] +
                  0.525 * th[IX(nr - 2, ka)] - 0.08928571 * th[IX(nr - 3, ka)]) * dri;
    }
    *trans1 = t1;
    *trans2 = t2;
}

/* update (:812-845). */
void orc_tank_update(orc_prb_t *s)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const double dr = s->dr;
    for (int k = 1; k <= np - 1; ++k) {
        s->Cn[IX(0, k)] = (3.0 * s->vel[IX(1, k)] - s->vel[IX(2, k)] / 3.0) / dr;
        s->Cn[IX(nr, k)] = (s->vel[IX(nr - 1, k)] / 3.0 - 3.0 * s->vel[IX(nr, k)]) / dr;
    }
    for (int i = 0; i <= nr; ++i) {
        s->Cn[IX(i, 0)] = is_dvd(s) ? -s->uel[IX(i, 1)] / s->dp : 0.0;
        s->Cn[IX(i, np)] = is_dvd(s) ? s->uel[IX(i, np)] / s->dp : 0.0;
    }
    if (is_dvd(s)) {
        for (int k = 0; k <= np + 1; ++k) {
            s->thn[IX(0, k)] = 0.0;
            s->thn[IX(nr + 1, k)] = 1.0;
        }
        for (int i = 1; i <= nr; ++i) {
            s->thn[IX(i, 0)] = -30.0 / 92.0 * (-3.75 * s->thn[IX(i, 1)] + 5.0 / 6.0 * s->thn[IX(i, 2)] -
                                               3.0 / 20.0 * s->thn[IX(i, 3)]);
            s->thn[IX(i, np + 1)] = -30.0 / 92.0 * (-3.75 * s->thn[IX(i, np)] + 5.0 / 6.0 * s->thn[IX(i, np - 1)] -
                                                    3.0 / 20.0 * s->thn[IX(i, np - 2)]);
        }
    } else for (int k = 0; k <= np; ++k) {
        s->thn[IX(0, k)] = -30.0 / 92.0 * (-3.75 * s->thn[IX(1, k)] + 5.0 / 6.0 * s->thn[IX(2, k)] -
                                           3.0 / 20.0 * s->thn[IX(3, k)]);
        s->thn[IX(nr + 1, k)] = (double)k / (double)np * 1.0;
    }
    if (!is_dvd(s))
        for (int i = 0; i <= nr + 1; ++i) {
            s->thn[IX(i, 0)] = 2.0 / 1.5 * s->thn[IX(i, 1)] - 1.0 / 3.0 * s->thn[IX(i, 2)];
            s->thn[IX(i, np + 1)] = 2.0 / 1.5 * s->thn[IX(i, np)] - 1.0 / 3.0 * s->thn[IX(i, np - 1)];
        }
    for (int i = 0; i <= nr + 1; ++i) {
        s->thp[IX(i, np + 1)] = s->th[IX(i, np + 1)];
        s->th[IX(i, np + 1)] = s->thn[IX(i, np + 1)];
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

/* rhsv (:867-885) and rhsu (:887-910). */
void orc_tank_rhsv(orc_prb_t *s)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    const double dr = s->dr;
    for (int i = 1; i <= nr; ++i)
        for (int k = 1; k <= np - 1; ++k) {
            const double Cr = (s->Cn[IX(i, k)] - s->Cn[IX(i - 1, k)]) / dr;
            if (i == 1) s->vrh[IX(i, k)] = s->Cn[IX(1, k)] / dr;
            else if (i == nr) s->vrh[IX(i, k)] = -s->Cn[IX(nr - 1, k)] / dr;
            else s->vrh[IX(i, k)] = Cr;
        }
}

void orc_tank_rhsu(orc_prb_t *s)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    for (int i = 1; i <= nr - 1; ++i)
        for (int k = 1; k <= np; ++k) {
            const double Ch = (s->Cn[IX(i, k)] - s->Cn[IX(i, k - 1)]) / s->dp;
            s->urh[IX(i, k)] = -Ch / 1.0;
        }
}

/* The tank's start (:70-140): T = 0.5 everywhere including the ghost column
 * np+1 and the bottom wall, T = k/np on the top wall (i = nr+1), all else
 * zero; the blobs there have amplitude -0.0 and leave T unchanged.  The
 * previous time level is the current one. */
void orc_tank_initial(orc_prb_t *s)
{
    const int ld = s->ld, nr = s->nr, np = s->np;
    for (int i = 0; i <= nr + 1; ++i) {
        s->th[IX(i, np + 1)] = 0.5;
        for (int k = 0; k <= np; ++k) {
            s->An[IX(i, k)] = s->Bn[IX(i, k)] = s->Cn[IX(i, k)] = 0.0;
            s->A[IX(i, k)] = s->B[IX(i, k)] = s->C[IX(i, k)] = 0.0;
            s->uel[IX(i, k)] = s->vel[IX(i, k)] = s->wel[IX(i, k)] = 0.0;
            if (is_dvd(s))   /* velvor2ddvdbenchmark.f:92-96 */
                s->th[IX(i, k)] = i == 0 ? 0.0 : i == nr + 1 ? 1.0 : 0.5;
            else
                s->th[IX(i, k)] = i == nr + 1 ? (double)k / (double)np * 1.0 : 0.5;
        }
    }
    for (int i = 0; i <= nr + 1; ++i)
        for (int k = 0; k <= np + 1; ++k) {
            s->Ap[IX(i, k)] = s->A[IX(i, k)];
            s->Bp[IX(i, k)] = s->B[IX(i, k)];
            s->Cp[IX(i, k)] = s->C[IX(i, k)];
            s->thp[IX(i, k)] = s->th[IX(i, k)];
            s->uelp[IX(i, k)] = s->uel[IX(i, k)];
            s->velp[IX(i, k)] = s->vel[IX(i, k)];
            s->welp[IX(i, k)] = 0.0;
        }
}
