/*
 * CPU oracle: restatement of rotann2.f's axisymmetric rotating-annulus step
 * ("AXI").  TEST INFRASTRUCTURE ONLY; parity as in axi_oracle.h.
 * Every expression keeps the reference's left-to-right evaluation order;
 * build with -ffp-contract=off.
 */
#include "axi_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "prb_oracle.h"   /* orc_tdma: the same tdma as rotann2.f:971-1004 */

#define AX(i, j) ((size_t)(i) + (size_t)ld * (size_t)(j))

static double *zalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

/* the stretched-grid forms (end of this file) */
static void axs_vort_vel(orc_axi_t *s, int what);
static void axs_temperature(orc_axi_t *s);
static double axs_heat(const orc_axi_t *s);
static void axs_update(orc_axi_t *s);
static int axs_poisson(orc_axi_t *s, int *sweeps);

int orc_axi_init(orc_axi_t *s, int nr, int nz, double dt, double r0, double rmax, double zmax,
                 double Ra, double Re, double Ptl)
{
    memset(s, 0, sizeof(*s));
    /* level count, poissoninit rotann2.f:563-580: halvings while both nr
     * and nz stay even, capped at 6 */
    int nlev = 0, it = nr, it2 = nr, jt = nz, jt2 = nz;
    for (int i = 2; i <= 8; ++i) {
        it = it / 2;
        jt = jt / 2;
        if (it * 2 - it2 == 0 && jt * 2 - jt2 == 0) {
            nlev = nlev + 1;
            it2 = it;
            jt2 = jt;
        } else {
            break;
        }
    }
    if (nlev > 6) nlev = 6;
    if (nlev < 1 || nr < 4 || nz < 2) return ORC_INVALID;
    s->nr = nr;
    s->nz = nz;
    s->ld = nr + 1;
    s->dt = dt;
    s->r0 = r0;
    s->rmax = rmax;
    s->zmax = zmax;
    s->Ra = Ra;
    s->Re = Re;
    s->Ptl = Ptl;
    /* constants, rotann2.f:62-69 */
    s->dr = (rmax - r0) / (double)nr;
    s->dz = zmax / (double)nz;
    const double dr = s->dr, dz = s->dz;
    s->cf1 = 1.0 / (2.0 * Ptl * dt) + 1.0 / (dr * dr) + 1.0 / (dz * dz);
    s->cf2 = 1.0 / (2.0 * Ptl * dt) - 1.0 / (dr * dr) - 1.0 / (dz * dz);
    s->cf3 = 1.0 / (2.0 * dt) + 1.0 / (dr * dr) + 1.0 / (dz * dz);
    s->cf4 = 1.0 / (2.0 * dt) - 1.0 / (dr * dr) - 1.0 / (dz * dz);
    const size_t full = (size_t)(nr + 1) * (size_t)(nz + 1);
    double **fl[] = {&s->phi, &s->omegn, &s->omeg, &s->omegp, &s->veln, &s->vel, &s->velp,
                     &s->thetan, &s->theta, &s->thetap, &s->psic, &s->psif, &s->rc, &s->rf, &s->tempa};
    for (size_t q = 0; q < sizeof(fl) / sizeof(fl[0]); ++q) *fl[q] = zalloc(full);
    s->rval = zalloc((size_t)nr + 1);
    s->nlev = nlev;
    /* level sizes, rotann2.f:583-594 */
    for (int l = 1; l <= nlev; ++l) {
        s->n1[l] = nr * 2 / (1 << l);
        s->n2[l] = nz * 2 / (1 << l);
        s->hr[l] = dr * (double)(1 << l) / 2.0;
        s->hz[l] = dz * (double)(1 << l) / 2.0;
        s->hhr[l] = s->hr[l] * s->hr[l];
        s->hhz[l] = s->hz[l] * s->hz[l];
        const size_t sz = (size_t)(s->n1[l] + 1) * (size_t)(s->n2[l] + 1);
        s->v[l] = zalloc(sz);
        s->f[l] = zalloc(sz);
    }
    s->tolcon = 1.0e-6;
    s->nrel = 2;
    s->maxsweeps = 10000;
    s->mode = AXI_LEX;
    return ORC_OK;
}

void orc_axi_free(orc_axi_t *s)
{
    double *fl[] = {s->phi, s->omegn, s->omeg, s->omegp, s->veln, s->vel, s->velp, s->thetan, s->theta,
                    s->thetap, s->psic, s->psif, s->rc, s->rf, s->tempa, s->rval};
    for (size_t q = 0; q < sizeof(fl) / sizeof(fl[0]); ++q) free(fl[q]);
    for (int l = 1; l <= s->nlev; ++l) {
        free(s->v[l]);
        free(s->f[l]);
    }
    memset(s, 0, sizeof(*s));
}

static unsigned long long axi_splitmix64(unsigned long long *state)
{
    unsigned long long z = (*state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

void orc_axi_initial(orc_axi_t *s, int kind, unsigned long long seed, double amp)
{
    const int ld = s->ld, nr = s->nr, nz = s->nz;
    unsigned long long st = seed;
    for (int j = 0; j <= nz; ++j) {
        for (int i = 0; i <= nr; ++i) {
            const double r = s->sg ? s->sg->r[1][i] : s->r0 + (double)i * s->dr;
            s->omeg[AX(i, j)] = 0.0;
            s->phi[AX(i, j)] = 0.0;
            s->vel[AX(i, j)] = 0.0;
            double t = 1.0 - log(r / s->rmax) / log(s->r0 / s->rmax);
            if (kind == 1 && i >= 1 && i <= nr - 1) {
                double u = (double)(axi_splitmix64(&st) >> 11) * (1.0 / 9007199254740992.0);
                t = t + amp * (2.0 * u - 1.0);
            }
            s->theta[AX(i, j)] = t;
        }
    }
    if (kind == 0) s->theta[AX(nr / 4, nz / 4)] = s->theta[AX(nr / 4, nz / 4)] + 0.01;
    for (size_t q = 0; q < (size_t)ld * (size_t)(nz + 1); ++q) {
        s->omegp[q] = s->omeg[q];
        s->velp[q] = s->vel[q];
        s->thetap[q] = s->theta[q];
        s->omegn[q] = s->veln[q] = s->thetan[q] = 0.0;
    }
}

/* arakawa, rotann2.f:432-459 (interior points only) */
void orc_axi_arakawa(const orc_axi_t *s, double *arak, const double *psi, const double *th)
{
    const int ld = s->ld, nx = s->nr, ny = s->nz;
    const double hx = s->dr, hy = s->dz;
    for (int i = 1; i <= nx - 1; ++i) {
        for (int j = 1; j <= ny - 1; ++j) {
            const int ip = i + 1, im = i - 1;
            double a = (psi[AX(ip, j)] - psi[AX(im, j)]) * (th[AX(i, j + 1)] - th[AX(i, j - 1)]) -
                       (psi[AX(i, j + 1)] - psi[AX(i, j - 1)]) * (th[AX(ip, j)] - th[AX(im, j)]) +
                       psi[AX(ip, j)] * (th[AX(ip, j + 1)] - th[AX(ip, j - 1)]) -
                       psi[AX(im, j)] * (th[AX(im, j + 1)] - th[AX(im, j - 1)]) -
                       psi[AX(i, j + 1)] * (th[AX(ip, j + 1)] - th[AX(im, j + 1)]) +
                       psi[AX(i, j - 1)] * (th[AX(ip, j - 1)] - th[AX(im, j - 1)]) +
                       th[AX(i, j + 1)] * (psi[AX(ip, j + 1)] - psi[AX(im, j + 1)]) -
                       th[AX(i, j - 1)] * (psi[AX(ip, j - 1)] - psi[AX(im, j - 1)]) -
                       th[AX(ip, j)] * (psi[AX(ip, j + 1)] - psi[AX(ip, j - 1)]) +
                       th[AX(im, j)] * (psi[AX(im, j + 1)] - psi[AX(im, j - 1)]);
            arak[AX(i, j)] = a / (12.0 * hx * hy);
        }
    }
}

/* vorticity, rotann2.f:268-316 */
void orc_axi_vorticity(orc_axi_t *s)
{
    if (s->sg) {
        axs_vort_vel(s, 1);
        return;
    }
    const int ld = s->ld, nr = s->nr, nz = s->nz;
    const double dr = s->dr, dz = s->dz, Ptl = s->Ptl, Ra = s->Ra, Re = s->Re;
    const double *omeg = s->omeg, *omegp = s->omegp, *phi = s->phi, *vel = s->vel, *theta = s->theta;
    double *arak = zalloc((size_t)ld * (size_t)(nz + 1));
    orc_axi_arakawa(s, arak, phi, omeg);
    const double RRP = Ra / Re / Ptl;
    for (int i = 1; i <= nr - 1; ++i) {
        for (int j = 1; j <= nz - 1; ++j) {
            const int ip = i + 1, im = i - 1, jp = j + 1, jm = j - 1;
            const double r = s->r0 + (double)i * dr;
            const double A = s->cf1 + 1.0 / (2.0 * (r * r));
            const double AA = s->cf2 - 1.0 / (2.0 * (r * r));
            const double B = (1.0 / (2.0 * Ptl * r * dz)) *
                             (phi[AX(i, j)] * (omeg[AX(i, jp)] - omeg[AX(i, jm)]) +
                              omeg[AX(i, j)] * (phi[AX(i, jp)] - phi[AX(i, jm)]));
            const double C = (1.0 / (Ptl * r * dz)) * vel[AX(i, j)] * (vel[AX(i, jp)] - vel[AX(i, jm)]);
            const double D = Re * (vel[AX(i, jp)] - vel[AX(i, jm)]) / dz;
            const double E = r * Ra * (theta[AX(i, jp)] - theta[AX(i, jm)]) / (2.0 * dz);
            const double EE = RRP * vel[AX(i, j)] * (theta[AX(i, jp)] - theta[AX(i, jm)]) / dz +
                              RRP * theta[AX(i, j)] * (vel[AX(i, jp)] - vel[AX(i, jm)]) / dz;
            const double F = (omeg[AX(ip, j)] + omeg[AX(im, j)]) / (dr * dr);
            const double G = (1.0 / (2.0 * r * dr)) * (omeg[AX(ip, j)] - omeg[AX(im, j)]);
            const double H = (omeg[AX(i, jp)] + omeg[AX(i, jm)]) / (dz * dz);
            s->omegn[AX(i, j)] = (AA * omegp[AX(i, j)] + arak[AX(i, j)] / Ptl + B + C + D - E - EE + F + G + H) / A;
        }
    }
    free(arak);
}

/* velocity, rotann2.f:324-370 */
void orc_axi_velocity(orc_axi_t *s)
{
    if (s->sg) {
        axs_vort_vel(s, 2);
        return;
    }
    const int ld = s->ld, nr = s->nr, nz = s->nz;
    const double dr = s->dr, dz = s->dz, Ptl = s->Ptl, Ra = s->Ra, Re = s->Re;
    const double *phi = s->phi, *vel = s->vel, *velp = s->velp, *theta = s->theta;
    double *arak = zalloc((size_t)ld * (size_t)(nz + 1));
    orc_axi_arakawa(s, arak, phi, vel);
    const double RRP = Ra / Re / Ptl;
    for (int i = 1; i <= nr - 1; ++i) {
        for (int j = 1; j <= nz - 1; ++j) {
            const int ip = i + 1, im = i - 1, jp = j + 1, jm = j - 1;
            const double r = s->r0 + (double)i * dr;
            const double A = s->cf1 + 1.0 / (2.0 * (r * r));
            const double AA = s->cf2 - 1.0 / (2.0 * (r * r));
            const double B = (1.0 / (2.0 * Ptl * r * dz)) *
                             (vel[AX(i, j)] * (phi[AX(i, jp)] - phi[AX(i, jm)]) -
                              phi[AX(i, j)] * (vel[AX(i, jp)] - vel[AX(i, jm)]));
            const double C = Re * (phi[AX(i, jp)] - phi[AX(i, jm)]) / dz;
            const double CC = -RRP * theta[AX(i, j)] * (phi[AX(i, jp)] - phi[AX(i, jm)]) / dz;
            const double D = (vel[AX(ip, j)] + vel[AX(im, j)]) / (dr * dr);
            const double E = (1.0 / (2.0 * r * dr)) * (vel[AX(ip, j)] - vel[AX(im, j)]);
            const double F = (vel[AX(i, jp)] + vel[AX(i, jm)]) / (dz * dz);
            s->veln[AX(i, j)] = (AA * velp[AX(i, j)] + arak[AX(i, j)] / Ptl - B - C - CC + D + E + F) / A;
        }
    }
    free(arak);
}

/* temperature, rotann2.f:379-424: rows j = 0 and nz mirror j-1 / j+1
 * (adiabatic top and bottom) and take no Jacobian. */
void orc_axi_temperature(orc_axi_t *s)
{
    if (s->sg) {
        axs_temperature(s);
        return;
    }
    const int ld = s->ld, nr = s->nr, nz = s->nz;
    const double dr = s->dr, dz = s->dz;
    const double *phi = s->phi, *theta = s->theta, *thetap = s->thetap;
    double *arak = zalloc((size_t)ld * (size_t)(nz + 1));
    orc_axi_arakawa(s, arak, phi, theta);
    for (int i = 1; i <= nr - 1; ++i) {
        for (int j = 0; j <= nz; ++j) {
            const int ip = i + 1, im = i - 1;
            int jp = j + 1, jm = j - 1;
            const double r = s->r0 + (double)i * dr;
            if (j == 0) {
                jm = jp;
                arak[AX(i, j)] = 0.0;
            }
            if (j == nz) {
                jp = jm;
                arak[AX(i, j)] = 0.0;
            }
            const double B = (1.0 / (2.0 * r * dz)) * phi[AX(i, j)] * (theta[AX(i, jp)] - theta[AX(i, jm)]);
            const double C = (theta[AX(ip, j)] + theta[AX(im, j)]) / (dr * dr);
            const double D = (1.0 / (2.0 * r * dr)) * (theta[AX(ip, j)] - theta[AX(im, j)]);
            const double E = (theta[AX(i, jp)] + theta[AX(i, jm)]) / (dz * dz);
            s->thetan[AX(i, j)] = (s->cf4 * thetap[AX(i, j)] + arak[AX(i, j)] + B + C + D + E) / s->cf3;
        }
    }
    free(arak);
}

/* heat, rotann2.f:468-487: fourth-order one-sided d/dr at the inner wall,
 * trapezoid in z. */
double orc_axi_heat(const orc_axi_t *s)
{
    if (s->sg) return axs_heat(s);
    const int ld = s->ld, nz = s->nz;
    const double dr = s->dr, dz = s->dz;
    const double *th = s->theta;
    double trans = dz * (-25.0 * th[AX(0, 0)] + 48.0 * th[AX(1, 0)] - 36.0 * th[AX(2, 0)] + 16.0 * th[AX(3, 0)] -
                         3.0 * th[AX(4, 0)]) / (24.0 * dr);
    trans = trans + dz * (-25.0 * th[AX(0, nz)] + 48.0 * th[AX(1, nz)] - 36.0 * th[AX(2, nz)] +
                          16.0 * th[AX(3, nz)] - 3.0 * th[AX(4, nz)]) / (24.0 * dr);
    for (int j = 1; j <= nz - 1; ++j)
        trans = trans + dz * (-25.0 * th[AX(0, j)] + 48.0 * th[AX(1, j)] - 36.0 * th[AX(2, j)] +
                              16.0 * th[AX(3, j)] - 3.0 * th[AX(4, j)]) / (12.0 * dr);
    return trans;
}

/* update, rotann2.f:497-539: Thom wall vorticity 2 psi_1 / h^2 (the r-walls
 * written last, so they own the corners), walls of v and T, time levels. */
void orc_axi_update(orc_axi_t *s)
{
    if (s->sg) {
        axs_update(s);
        return;
    }
    const int ld = s->ld, nr = s->nr, nz = s->nz;
    const double dr = s->dr, dz = s->dz;
    for (int i = 0; i <= nr; ++i) {
        s->omegn[AX(i, 0)] = 2.0 * s->phi[AX(i, 1)] / (dz * dz);
        s->veln[AX(i, 0)] = 0.0;
        s->omegn[AX(i, nz)] = 2.0 * s->phi[AX(i, nz - 1)] / (dz * dz);
        s->veln[AX(i, nz)] = 0.0;
    }
    for (int j = 0; j <= nz; ++j) {
        s->omegn[AX(0, j)] = 2.0 * s->phi[AX(1, j)] / (dr * dr);
        s->veln[AX(0, j)] = 0.0;
        s->thetan[AX(0, j)] = 0.0;
        s->omegn[AX(nr, j)] = 2.0 * s->phi[AX(nr - 1, j)] / (dr * dr);
        s->veln[AX(nr, j)] = 0.0;
        s->thetan[AX(nr, j)] = 1.0;
    }
    for (size_t q = 0; q < (size_t)ld * (size_t)(nz + 1); ++q) {
        s->omegp[q] = s->omeg[q];
        s->omeg[q] = s->omegn[q];
        s->velp[q] = s->vel[q];
        s->vel[q] = s->veln[q];
        s->thetap[q] = s->theta[q];
        s->theta[q] = s->thetan[q];
    }
}

/* trans1 / trans2 (rotann2.f:856-880): level region <-> packed slot */
static void axi_pack(const orc_axi_t *s, const double *a2, double *a1, int l)
{
    const int ld = s->ld, n1 = s->n1[l], n2 = s->n2[l];
    for (int j = 0; j <= n2; ++j)
        for (int i = 0; i <= n1; ++i) a1[(size_t)j * (n1 + 1) + i] = a2[AX(i, j)];
}

static void axi_unpack(const orc_axi_t *s, const double *a1, double *a2, int l)
{
    const int ld = s->ld, n1 = s->n1[l], n2 = s->n2[l];
    for (int j = 0; j <= n2; ++j)
        for (int i = 0; i <= n1; ++i) a2[AX(i, j)] = a1[(size_t)j * (n1 + 1) + i];
}

static void r_line(orc_axi_t *s, int klev, int j, double *wa, double *wb, double *wc, double *wr, double *ws)
{
    const int ld = s->ld, n1 = s->n1[klev], lf = (1 << klev) / 2;
    const double hhr = s->hhr[klev], hhz = s->hhz[klev], hr = s->hr[klev];
    double *psif = s->psif;
    for (int i = 1; i <= n1 - 1; ++i) {
        const double rv = s->rval[i * lf];
        wa[i - 1] = 1.0 / hhr - 0.5 / hr / rv;
        wc[i - 1] = 1.0 / hhr + 0.5 / hr / rv;
        wb[i - 1] = -2.0 / hhr - 2.0 / hhz - 1.0 / (rv * rv);
        wr[i - 1] = -(psif[AX(i, j + 1)] + psif[AX(i, j - 1)]) / hhz + s->rf[AX(i, j)];
    }
    orc_tdma(wa, wb, wc, ws, wr, n1 - 1);
    for (int i = 1; i <= n1 - 1; ++i) psif[AX(i, j)] = ws[i - 1];
}

static void z_line(orc_axi_t *s, int klev, int i, double *wa, double *wb, double *wc, double *wr, double *ws)
{
    const int ld = s->ld, n2 = s->n2[klev], lf = (1 << klev) / 2;
    const double hhr = s->hhr[klev], hhz = s->hhz[klev], hr = s->hr[klev];
    double *psif = s->psif;
    const double rv = s->rval[i * lf];
    for (int j = 1; j <= n2 - 1; ++j) {
        wa[j - 1] = 1.0 / hhz;
        wc[j - 1] = 1.0 / hhz;
        wb[j - 1] = -2.0 / hhr - 2.0 / hhz - 1.0 / (rv * rv);
        wr[j - 1] = -(psif[AX(i + 1, j)] + psif[AX(i - 1, j)]) / hhr + s->rf[AX(i, j)] -
                    (psif[AX(i + 1, j)] - psif[AX(i - 1, j)]) * 0.5 / rv / hr;
    }
    orc_tdma(wa, wb, wc, ws, wr, n2 - 1);
    for (int j = 1; j <= n2 - 1; ++j) psif[AX(i, j)] = ws[j - 1];
}

/* relax, rotann2.f:668-753 */
void orc_axi_relax(orc_axi_t *s, int nrel, int klev, int *nconv)
{
    const int ld = s->ld, n1 = s->n1[klev], n2 = s->n2[klev], lf = (1 << klev) / 2;
    const double hhr = s->hhr[klev], hhz = s->hhz[klev], hr = s->hr[klev];
    double *psif = s->psif, *rf = s->rf, *rc = s->rc;
    *nconv = 0;
    axi_unpack(s, s->f[klev], rf, klev);
    axi_unpack(s, s->v[klev], psif, klev);
    const double drdz = 2.0 * (1.0 / hhr + 1.0 / hhz);
    const int nmax = (n1 > n2 ? n1 : n2) + 2;
    double *buf = zalloc((size_t)nmax * 5);
    double *wa = buf, *wb = wa + nmax, *wc = wb + nmax, *wr = wc + nmax, *ws = wr + nmax;
    double resmax = 0.0;
    for (int irel = 1; irel <= nrel; ++irel) {
        if (s->mode == AXI_LEX) {
            for (int j = 1; j <= n2 - 1; ++j) r_line(s, klev, j, wa, wb, wc, wr, ws);
            for (int i = 1; i <= n1 - 1; ++i) z_line(s, klev, i, wa, wb, wc, wr, ws);
        } else {
            for (int par = 1; par >= 0; --par)
                for (int j = 1; j <= n2 - 1; ++j)
                    if ((j & 1) == par) r_line(s, klev, j, wa, wb, wc, wr, ws);
            for (int par = 1; par >= 0; --par)
                for (int i = 1; i <= n1 - 1; ++i)
                    if ((i & 1) == par) z_line(s, klev, i, wa, wb, wc, wr, ws);
        }
        resmax = 0.0;
        for (int i = 1; i <= n1 - 1; ++i) {
            const double rv = s->rval[i * lf];
            for (int j = 1; j <= n2 - 1; ++j) {
                double temp = (psif[AX(i + 1, j)] + psif[AX(i - 1, j)]) / hhr +
                              (psif[AX(i + 1, j)] - psif[AX(i - 1, j)]) * 0.5 / hr / rv -
                              psif[AX(i, j)] / (rv * rv) + (psif[AX(i, j + 1)] + psif[AX(i, j - 1)]) / hhz -
                              psif[AX(i, j)] * drdz;
                temp = rf[AX(i, j)] - temp;
                rc[AX(i, j)] = temp;
                temp = fabs(temp);
                if (temp > resmax) resmax = temp;
            }
        }
    }
    free(buf);
    axi_pack(s, psif, s->v[klev], klev);
    if (klev == 1) s->last_resmax = resmax;
    if (klev == 1 && resmax < s->tolcon) *nconv = 1;
}

/* corser, rotann2.f:755-801: nine-point restriction; the boundary rows and
 * columns cleared use n1 of the coarse level for both directions, as the
 * reference does (no effect when nr = nz). */
void orc_axi_corser(orc_axi_t *s, int klev)
{
    const int ld = s->ld, n1 = s->n1[klev], n2 = s->n2[klev];
    const int n1c = s->n1[klev + 1], n2c = s->n2[klev + 1];
    double *rc = s->rc, *rf = s->rf, *psic = s->psic;
    for (int j = 0; j <= n2; ++j)
        for (int i = 0; i <= n1; ++i) rf[AX(i, j)] = rc[AX(i, j)];
    for (int i = 1; i <= n1c - 1; ++i) {
        for (int j = 1; j <= n2c - 1; ++j) {
            const int ii = i + i, jj = j + j;
            double temp = rf[AX(ii, jj)];
            temp = temp * 2.0 + rf[AX(ii + 1, jj)] + rf[AX(ii - 1, jj)];
            temp = temp + rf[AX(ii, jj + 1)] + rf[AX(ii, jj - 1)];
            temp = temp * 2.0 + rf[AX(ii + 1, jj + 1)] + rf[AX(ii - 1, jj - 1)];
            temp = temp + rf[AX(ii + 1, jj - 1)] + rf[AX(ii - 1, jj + 1)];
            temp = temp / 16.0;
            rc[AX(i, j)] = temp;
            psic[AX(i, j)] = 0.0;
        }
    }
    for (int i = 0; i <= n1c; ++i) {
        rc[AX(i, 0)] = 0.0;
        rc[AX(i, n1c)] = 0.0;
        psic[AX(i, 0)] = 0.0;
        psic[AX(i, n1c)] = 0.0;
    }
    for (int j = 0; j <= n1c; ++j) {
        rc[AX(0, j)] = 0.0;
        rc[AX(n1c, j)] = 0.0;
        psic[AX(0, j)] = 0.0;
        psic[AX(n1c, j)] = 0.0;
    }
    axi_pack(s, rc, s->f[klev + 1], klev + 1);
    axi_pack(s, psic, s->v[klev + 1], klev + 1);
}

/* finer, rotann2.f:803-854 */
void orc_axi_finer(orc_axi_t *s, int klev)
{
    const int ld = s->ld;
    const int n1f = s->n1[klev - 1], n2f = s->n2[klev - 1];
    double *psic = s->psic, *psif = s->psif, *tempa = s->tempa;
    axi_unpack(s, s->v[klev], psic, klev);
    for (int i = 0; i <= n1f; ++i) {
        for (int j = 0; j <= n2f; ++j) {
            const int i1 = i / 2, j1 = j / 2;
            if (i1 * 2 == i) {
                if (j1 * 2 == j) psif[AX(i, j)] = psic[AX(i1, j1)];
                else psif[AX(i, j)] = (psic[AX(i1, j1)] + psic[AX(i1, j1 + 1)]) * 0.5;
            } else {
                if (j1 * 2 == j) {
                    psif[AX(i, j)] = (psic[AX(i1, j1)] + psic[AX(i1 + 1, j1)]) * 0.5;
                } else {
                    double temp = psic[AX(i1, j1)] + psic[AX(i1 + 1, j1 + 1)];
                    temp = temp + psic[AX(i1, j1 + 1)] + psic[AX(i1 + 1, j1)];
                    psif[AX(i, j)] = temp * 0.25;
                }
            }
        }
    }
    axi_unpack(s, s->v[klev - 1], tempa, klev - 1);
    for (int i = 0; i <= n1f; ++i) {
        for (int j = 0; j <= n2f; ++j) {
            psif[AX(i, j)] = psif[AX(i, j)] + tempa[AX(i, j)];
            psic[AX(i, j)] = 0.0;
        }
    }
    axi_pack(s, psic, s->v[klev], klev);
    axi_pack(s, psif, s->v[klev - 1], klev - 1);
}

/* poisson, rotann2.f:598-666 */
int orc_axi_poisson(orc_axi_t *s, double *psi, const double *rhs, int *sweeps)
{
    if (s->sg) {
        /* the stretched solve works on the state's phi and omegn */
        if (psi != s->phi || rhs != s->omegn) return ORC_INVALID;
        return axs_poisson(s, sweeps);
    }
    const int ld = s->ld, nlev = s->nlev, n1 = s->n1[1], n2 = s->n2[1];
    int nconv = 0;
    for (int i = 0; i <= n1; ++i) {
        s->rval[i] = (double)i * s->hr[1] + s->r0;
        for (int j = 0; j <= n2; ++j) {
            s->psic[AX(i, j)] = 0.0;
            s->psif[AX(i, j)] = psi[AX(i, j)];
            s->rc[AX(i, j)] = 0.0;
            s->rf[AX(i, j)] = rhs[AX(i, j)];
        }
    }
    axi_pack(s, s->rf, s->f[1], 1);
    axi_pack(s, s->psif, s->v[1], 1);
    for (int sweep = 1; sweep <= s->maxsweeps; ++sweep) {
        if (sweep == 1 || nlev == 1) orc_axi_relax(s, s->nrel, 1, &nconv);
        if (nlev > 1) {
            for (int l = 1; l <= nlev - 1; ++l) {
                orc_axi_corser(s, l);
                orc_axi_relax(s, s->nrel, l + 1, &nconv);
            }
            for (int l = nlev; l >= 2; --l) {
                orc_axi_finer(s, l);
                orc_axi_relax(s, s->nrel, l - 1, &nconv);
            }
        }
        if (nconv == 1) {
            for (int i = 0; i <= n1; ++i)
                for (int j = 0; j <= n2; ++j) psi[AX(i, j)] = s->psif[AX(i, j)];
            if (sweeps) *sweeps = sweep;
            s->last_sweeps = sweep;
            return 0;
        }
    }
    if (sweeps) *sweeps = s->maxsweeps;
    s->last_sweeps = s->maxsweeps;
    return 1;
}

int orc_axi_step(orc_axi_t *s, double *nu, int *sweeps, int *converged)
{
    const int ld = s->ld, nr = s->nr, nz = s->nz;
    orc_axi_vorticity(s);
    orc_axi_velocity(s);
    orc_axi_temperature(s);
    const int st = orc_axi_poisson(s, s->phi, s->omegn, sweeps);
    orc_axi_update(s);
    const double trans = orc_axi_heat(s);
    if (nu) *nu = -s->r0 * log(s->r0 / s->rmax) * trans / (s->zmax * s->rmax);
    if (converged) {
        double e1 = 0.0, e2 = 0.0, e3 = 0.0;
        for (int i = 0; i <= nr; ++i) {
            for (int j = 0; j <= nz; ++j) {
                const double a = fabs(s->omeg[AX(i, j)] - s->omegp[AX(i, j)]);
                const double b = fabs(s->vel[AX(i, j)] - s->velp[AX(i, j)]);
                const double c = fabs(s->theta[AX(i, j)] - s->thetap[AX(i, j)]);
                if (a > e1) e1 = a;
                if (b > e2) e2 = b;
                if (c > e3) e3 = c;
            }
        }
        const double tol = (double)1e-6f;   /* REAL*4 literal of rotann2.f:191 */
        *converged = (e1 < tol && e2 < tol && e3 < tol);
    }
    return st;
}

/* ------------------------------------------------------------------------
 * Stretched grid (see axi_oracle.h): rotann2.f's physics with grid.f's
 * level-1 weights and rcsc.f's stretched multigrid.  Every expression is
 * evaluated in the order written here, which the device kernels follow.
 * ------------------------------------------------------------------------ */
#define SR(i) (g->r[1][(i)])
#define SZ(j) (g->z[1][(j)])
#define SCR(i, k) (g->cr[1][3 * ((i) - 1) + (k) - 1])
#define SCRR(i, k) (g->crr[1][4 * ((i) - 1) + (k) - 1])
#define SCZ(j, k) (g->cz[1][3 * ((j) - 1) + (k) - 1])
#define SCZZ(j, k) (g->czz[1][4 * ((j) - 1) + (k) - 1])

int orc_axi_set_stretched(orc_axi_t *s, const orc_str_grid_t *g, orc_str_mg_t *m)
{
    if (!g || !m || g->nlev < 1 || g->n1[1] != s->nr || g->n2[1] != s->nz || s->nr < 4) return ORC_INVALID;
    double w[25];
    if (orc_str_fdif(5, 1, 0, g->r[1], w)) return ORC_INVALID;
    for (int q = 0; q < 5; ++q) s->hw[q] = w[5 + q];
    s->sg = g;
    s->smg = m;
    return ORC_OK;
}

static double axs_dr_off(const orc_str_grid_t *g, const double *x, int ld, int i, int j)
{
    return SCR(i, 1) * x[AX(i - 1, j)] + SCR(i, 3) * x[AX(i + 1, j)];
}
static double axs_drr_off(const orc_str_grid_t *g, const double *x, int ld, int i, int j, int nr)
{
    if (i <= nr / 2) return SCRR(i, 1) * x[AX(i - 1, j)] + SCRR(i, 3) * x[AX(i + 1, j)] + SCRR(i, 4) * x[AX(i + 2, j)];
    return SCRR(i, 1) * x[AX(i - 2, j)] + SCRR(i, 2) * x[AX(i - 1, j)] + SCRR(i, 4) * x[AX(i + 1, j)];
}
static double axs_crrc(const orc_str_grid_t *g, int i, int nr) { return i <= nr / 2 ? SCRR(i, 2) : SCRR(i, 3); }
static double axs_dz(const orc_str_grid_t *g, const double *x, int ld, int i, int j)
{
    return SCZ(j, 1) * x[AX(i, j - 1)] + SCZ(j, 2) * x[AX(i, j)] + SCZ(j, 3) * x[AX(i, j + 1)];
}
static double axs_dzz_off(const orc_str_grid_t *g, const double *x, int ld, int i, int j, int nz)
{
    if (j <= nz / 2) return SCZZ(j, 1) * x[AX(i, j - 1)] + SCZZ(j, 3) * x[AX(i, j + 1)] + SCZZ(j, 4) * x[AX(i, j + 2)];
    return SCZZ(j, 1) * x[AX(i, j - 2)] + SCZZ(j, 2) * x[AX(i, j - 1)] + SCZZ(j, 4) * x[AX(i, j + 1)];
}
static double axs_czzc(const orc_str_grid_t *g, int j, int nz) { return j <= nz / 2 ? SCZZ(j, 2) : SCZZ(j, 3); }

/* the Arakawa sum of rotann2.f:432-459 over the local metric */
static double axs_arakawa(const orc_str_grid_t *g, const double *psi, const double *th, int ld, int i, int j)
{
    const int ip = i + 1, im = i - 1;
    const double a = (psi[AX(ip, j)] - psi[AX(im, j)]) * (th[AX(i, j + 1)] - th[AX(i, j - 1)]) -
                     (psi[AX(i, j + 1)] - psi[AX(i, j - 1)]) * (th[AX(ip, j)] - th[AX(im, j)]) +
                     psi[AX(ip, j)] * (th[AX(ip, j + 1)] - th[AX(ip, j - 1)]) -
                     psi[AX(im, j)] * (th[AX(im, j + 1)] - th[AX(im, j - 1)]) -
                     psi[AX(i, j + 1)] * (th[AX(ip, j + 1)] - th[AX(im, j + 1)]) +
                     psi[AX(i, j - 1)] * (th[AX(ip, j - 1)] - th[AX(im, j - 1)]) +
                     th[AX(i, j + 1)] * (psi[AX(ip, j + 1)] - psi[AX(im, j + 1)]) -
                     th[AX(i, j - 1)] * (psi[AX(ip, j - 1)] - psi[AX(im, j - 1)]) -
                     th[AX(ip, j)] * (psi[AX(ip, j + 1)] - psi[AX(ip, j - 1)]) +
                     th[AX(im, j)] * (psi[AX(im, j + 1)] - psi[AX(im, j - 1)]);
    return a / (3.0 * (SR(ip) - SR(im)) * (SZ(j + 1) - SZ(j - 1)));
}

static void axs_vort_vel(orc_axi_t *s, int what)
{
    const orc_str_grid_t *g = s->sg;
    const int ld = s->ld, nr = s->nr, nz = s->nz;
    const double Ptl = s->Ptl, Ra = s->Ra, Re = s->Re, dt = s->dt;
    const double *omeg = s->omeg, *phi = s->phi, *vel = s->vel, *theta = s->theta;
    const double RRP = Ra / Re / Ptl;
    for (int i = 1; i <= nr - 1; ++i) {
        for (int j = 1; j <= nz - 1; ++j) {
            const double r = SR(i);
            const double sigma = axs_crrc(g, i, nr) + SCR(i, 2) / r + axs_czzc(g, j, nz);
            const double A = 1.0 / (2.0 * Ptl * dt) - sigma / 2.0 + 1.0 / (2.0 * (r * r));
            const double AA = 1.0 / (2.0 * Ptl * dt) + sigma / 2.0 - 1.0 / (2.0 * (r * r));
            const double dz_phi = axs_dz(g, phi, ld, i, j), dz_v = axs_dz(g, vel, ld, i, j);
            if (what & 1) {
                const double arak = axs_arakawa(g, phi, omeg, ld, i, j);
                const double dz_om = axs_dz(g, omeg, ld, i, j), dz_th = axs_dz(g, theta, ld, i, j);
                const double B = (phi[AX(i, j)] * dz_om + omeg[AX(i, j)] * dz_phi) / (Ptl * r);
                const double C = 2.0 * vel[AX(i, j)] * dz_v / (Ptl * r);
                const double D = 2.0 * Re * dz_v;
                const double E = r * Ra * dz_th;
                const double EE = 2.0 * RRP * vel[AX(i, j)] * dz_th + 2.0 * RRP * theta[AX(i, j)] * dz_v;
                const double F = axs_drr_off(g, omeg, ld, i, j, nr);
                const double G = axs_dr_off(g, omeg, ld, i, j) / r;
                const double H = axs_dzz_off(g, omeg, ld, i, j, nz);
                s->omegn[AX(i, j)] = (AA * s->omegp[AX(i, j)] + arak / Ptl + B + C + D - E - EE + F + G + H) / A;
            }
            if (what & 2) {
                const double arak = axs_arakawa(g, phi, vel, ld, i, j);
                const double B = (vel[AX(i, j)] * dz_phi - phi[AX(i, j)] * dz_v) / (Ptl * r);
                const double C = 2.0 * Re * dz_phi;
                const double CC = -2.0 * RRP * theta[AX(i, j)] * dz_phi;
                const double D = axs_drr_off(g, vel, ld, i, j, nr);
                const double E = axs_dr_off(g, vel, ld, i, j) / r;
                const double F = axs_dzz_off(g, vel, ld, i, j, nz);
                s->veln[AX(i, j)] = (AA * s->velp[AX(i, j)] + arak / Ptl - B - C - CC + D + E + F) / A;
            }
        }
    }
}

static void axs_temperature(orc_axi_t *s)
{
    const orc_str_grid_t *g = s->sg;
    const int ld = s->ld, nr = s->nr, nz = s->nz;
    const double dt = s->dt;
    const double *phi = s->phi, *theta = s->theta;
    const double h1 = SZ(1) - SZ(0), hn = SZ(nz) - SZ(nz - 1);
    for (int i = 1; i <= nr - 1; ++i) {
        for (int j = 0; j <= nz; ++j) {
            const double r = SR(i);
            double arak, B, E, czzc;
            if (j == 0) {
                arak = 0.0;
                B = 0.0;
                E = 2.0 * theta[AX(i, 1)] / (h1 * h1);
                czzc = -2.0 / (h1 * h1);
            } else if (j == nz) {
                arak = 0.0;
                B = 0.0;
                E = 2.0 * theta[AX(i, nz - 1)] / (hn * hn);
                czzc = -2.0 / (hn * hn);
            } else {
                arak = axs_arakawa(g, phi, theta, ld, i, j);
                B = phi[AX(i, j)] * axs_dz(g, theta, ld, i, j) / r;
                E = axs_dzz_off(g, theta, ld, i, j, nz);
                czzc = axs_czzc(g, j, nz);
            }
            const double sigma = axs_crrc(g, i, nr) + SCR(i, 2) / r + czzc;
            const double cf3 = 1.0 / (2.0 * dt) - sigma / 2.0;
            const double cf4 = 1.0 / (2.0 * dt) + sigma / 2.0;
            const double C = axs_drr_off(g, theta, ld, i, j, nr);
            const double D = axs_dr_off(g, theta, ld, i, j) / r;
            s->thetan[AX(i, j)] = (cf4 * s->thetap[AX(i, j)] + arak + B + C + D + E) / cf3;
        }
    }
}

static double axs_heat(const orc_axi_t *s)
{
    const orc_str_grid_t *g = s->sg;
    const int ld = s->ld, nz = s->nz;
    const double *th = s->theta;
    const double *w = s->hw;
#define AXS_DTDR(j) (w[0] * th[AX(0, j)] + w[1] * th[AX(1, j)] + w[2] * th[AX(2, j)] + w[3] * th[AX(3, j)] + \
                     w[4] * th[AX(4, j)])
    double trans = (SZ(1) - SZ(0)) / 2.0 * AXS_DTDR(0);
    trans = trans + (SZ(nz) - SZ(nz - 1)) / 2.0 * AXS_DTDR(nz);
    for (int j = 1; j <= nz - 1; ++j) trans = trans + (SZ(j + 1) - SZ(j - 1)) / 2.0 * AXS_DTDR(j);
#undef AXS_DTDR
    return trans;
}

static void axs_update(orc_axi_t *s)
{
    const orc_str_grid_t *g = s->sg;
    const int ld = s->ld, nr = s->nr, nz = s->nz;
    const double hz1 = SZ(1) - SZ(0), hzn = SZ(nz) - SZ(nz - 1);
    const double hr1 = SR(1) - SR(0), hrn = SR(nr) - SR(nr - 1);
    for (int i = 0; i <= nr; ++i) {
        s->omegn[AX(i, 0)] = 2.0 * s->phi[AX(i, 1)] / (hz1 * hz1);
        s->veln[AX(i, 0)] = 0.0;
        s->omegn[AX(i, nz)] = 2.0 * s->phi[AX(i, nz - 1)] / (hzn * hzn);
        s->veln[AX(i, nz)] = 0.0;
    }
    for (int j = 0; j <= nz; ++j) {
        s->omegn[AX(0, j)] = 2.0 * s->phi[AX(1, j)] / (hr1 * hr1);
        s->veln[AX(0, j)] = 0.0;
        s->thetan[AX(0, j)] = 0.0;
        s->omegn[AX(nr, j)] = 2.0 * s->phi[AX(nr - 1, j)] / (hrn * hrn);
        s->veln[AX(nr, j)] = 0.0;
        s->thetan[AX(nr, j)] = 1.0;
    }
    for (size_t q = 0; q < (size_t)ld * (size_t)(nz + 1); ++q) {
        s->omegp[q] = s->omeg[q];
        s->omeg[q] = s->omegn[q];
        s->velp[q] = s->vel[q];
        s->vel[q] = s->veln[q];
        s->thetap[q] = s->theta[q];
        s->theta[q] = s->thetan[q];
    }
}

/* the stretched multigrid with the AXI state's tolerance, relaxation count,
 * sweep limit and line order (AXI_ZEBRA: rcsc.f's four colours) */
static int axs_poisson(orc_axi_t *s, int *sweeps)
{
    orc_str_mg_t *m = s->smg;
    m->tolcon = s->tolcon;
    m->nrel = s->nrel;
    m->maxsweeps = s->maxsweeps;
    m->mode = s->mode;
    int sw = 0;
    const int st = orc_str_poisson(m, s->phi, s->omegn, &sw);
    s->last_sweeps = sw;
    if (sweeps) *sweeps = sw;
    return st;
}
