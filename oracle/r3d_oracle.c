/*
 * CPU oracle: restatement of the 3D rotating-annulus hot path of rot3dmg.f
 * (R3D).  TEST INFRASTRUCTURE ONLY -- the checker of tests/, smoke() and the
 * CPU legs of bench.py; never linked into the product.  PARITY PINNED: it
 * reproduces bit for bit rot3dmg.f and rot3dmghor.f run as their main
 * programs through the translator tests/golden/f77.py (every field, Nusselt
 * number and sweep count; tests/test_reference_runs.py), besides its own
 * invariants (manufactured solutions of the three velocity operators, the
 * conduction state, agreement of the two line orderings).
 *
 * Every expression keeps the reference's left-to-right evaluation order;
 * x**2 is x*x as the Fortran compiler expands it.  Build with
 * -ffp-contract=off (see Makefile).
 */
#include "r3d_oracle.h"
#include "prb_oracle.h"   /* orc_tdma, orc_ptdma, orc_pdma (the same solvers, rot3dmg.f:2570-2689) */

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* REAL*4 literal 0.2 mixed into REAL*8 arithmetic */
static const double F02 = (double)0.2f;

#define FX(a, i, j, k) ((a)[(size_t)(i) + (size_t)s->ni * ((size_t)(j) + (size_t)s->nj * (size_t)(k))])

static size_t field_size(const orc_r3d_t *s) { return (size_t)s->ni * (size_t)s->nj * (size_t)s->nk; }
static size_t level_size(const orc_r3d_t *s, int l)
{
    return (size_t)(s->n1[l] + 1) * (size_t)(s->n2[l] + 1) * (size_t)(s->n3[l] + 1);
}

/* ------------------------------------------------------------------------ */
/* Set-up (rot3dmg.f:92-96, poissoninit :1153-1213)                          */
/* ------------------------------------------------------------------------ */

int orc_r3d_init(orc_r3d_t *s, int nr, int nz, int np, double dt, double r0, double rmax, double zmax,
                 double Ra, double Re, double Gr, double Ptl)
{
    memset(s, 0, sizeof(*s));
    if (nr < 4 || nz < 4 || np < 4) return R3D_INVALID;
    s->nr = nr;
    s->nz = nz;
    s->np = np;
    s->ni = nr + 2;
    s->nj = nz + 2;
    s->nk = np + 1;
    s->dt = dt;
    s->r0 = r0;
    s->rmax = rmax;
    s->zmax = zmax;
    s->Ra = Ra;
    s->Re = Re;
    s->Gr = Gr;
    s->Ptl = Ptl;
    s->pi = acos(-1.0);
    s->dr = (rmax - r0) / (double)nr;
    s->dz = zmax / (double)nz;
    s->dp = 2.0 * s->pi / (double)np;
    s->tolcon = 1e-5;
    s->sor = 1.2;
    s->nrel = 2;
    s->maxsweeps = 500;
    s->mode = R3D_LEX;

    /* level count: halvings of nr and nz while both halve exactly, counted
     * while both are still >= 4, capped at 4 (rot3dmg.f:1172-1192) */
    int nlev = 0, itest = nr, itest2 = nr, jtest = nz, jtest2 = nz;
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
    if (nlev > 4) nlev = 4;
    if (nlev < 1) nlev = 1;
    s->nlev = nlev;
    if (np % (1 << nlev) != 0 || np / (1 << (nlev - 1)) < 4) return R3D_INVALID;
    for (int l = 1; l <= nlev; ++l) {
        const int p2 = 1 << l;
        s->n1[l] = nr * 2 / p2;
        s->n2[l] = nz * 2 / p2;
        s->n3[l] = np * 2 / p2;
        s->hr[l] = s->dr * (double)p2 * 0.5;
        s->hz[l] = s->dz * (double)p2 * 0.5;
        s->hp[l] = s->dp * (double)p2 * 0.5;
        s->hhr[l] = s->hr[l] * s->hr[l];
        s->hhz[l] = s->hz[l] * s->hz[l];
        s->hhp[l] = s->hp[l] * s->hp[l];
        const size_t n = level_size(s, l);
        s->v[l] = (double *)calloc(n, sizeof(double));
        s->f[l] = (double *)calloc(n, sizeof(double));
        s->res[l] = (double *)calloc(n, sizeof(double));
        if (!s->v[l] || !s->f[l] || !s->res[l]) return R3D_INVALID;
    }
    const size_t nf = field_size(s);
    double **fields[] = {&s->An, &s->A, &s->Ap, &s->Bn, &s->B, &s->Bp, &s->Cn, &s->C, &s->Cp,
                         &s->thn, &s->th, &s->thp, &s->uel, &s->vel, &s->wel, &s->uelp, &s->velp, &s->welp,
                         &s->urh, &s->vrh, &s->wrh};
    for (size_t q = 0; q < sizeof(fields) / sizeof(fields[0]); ++q) {
        *fields[q] = (double *)calloc(nf, sizeof(double));
        if (!*fields[q]) return R3D_INVALID;
    }
    return R3D_OK;
}

void orc_r3d_free(orc_r3d_t *s)
{
    double *fields[] = {s->An, s->A, s->Ap, s->Bn, s->B, s->Bp, s->Cn, s->C, s->Cp, s->thn, s->th, s->thp,
                        s->uel, s->vel, s->wel, s->uelp, s->velp, s->welp, s->urh, s->vrh, s->wrh};
    for (size_t q = 0; q < sizeof(fields) / sizeof(fields[0]); ++q) free(fields[q]);
    for (int l = 1; l < R3D_MAXLEV; ++l) {
        free(s->v[l]);
        free(s->f[l]);
        free(s->res[l]);
    }
    free(s->sinth);
    free(s->costh);
    memset(s, 0, sizeof(*s));
}

int orc_r3d_set_horizontal(orc_r3d_t *s)
{
    s->horizontal = 1;
    s->tolcon = 1e-6;
    free(s->sinth);
    free(s->costh);
    s->sinth = (double *)calloc((size_t)s->np + 1, sizeof(double));
    s->costh = (double *)calloc((size_t)s->np + 1, sizeof(double));
    if (!s->sinth || !s->costh) return R3D_INVALID;
    for (int k = 0; k <= s->np; ++k) {
        const double theta = 6.283185307 / (double)s->np * (double)k;
        s->sinth[k] = sin(theta);
        s->costh[k] = cos(theta);
    }
    return R3D_OK;
}

void orc_r3d_initial(orc_r3d_t *s, int nval, double amp)
{
    const int nr = s->nr, nz = s->nz, np = s->np;
    const size_t nf = field_size(s);
    double *zero[] = {s->An, s->A, s->Bn, s->B, s->Cn, s->C, s->uel, s->vel, s->wel, s->thn};
    for (size_t q = 0; q < sizeof(zero) / sizeof(zero[0]); ++q) memset(zero[q], 0, nf * sizeof(double));
    for (int i = 0; i <= nr + 1; ++i) {
        double r;
        if (i == 0) r = s->r0;
        else if (i == nr + 1) r = s->rmax;
        else r = s->r0 + ((double)i - 0.5) * s->dr;
        for (int j = 0; j <= nz + 1; ++j)
            for (int k = 0; k <= np; ++k) {
                const double phi = 8.0 * atan(1.0) * (double)k / (double)np;
                const double base = s->horizontal ? log(r) / log(s->r0) : 1.0 - log(r) / log(s->r0);
                FX(s->th, i, j, k) = base + amp * (s->rmax - r) * (r - s->r0) * cos((double)nval * phi);
            }
    }
    const int ic = s->horizontal ? nr / 2 : nr / 4, jc = s->horizontal ? nz / 2 : nz / 4;
    FX(s->th, ic, jc, np / 2) = FX(s->th, ic, jc, np / 2) - 0.5 * FX(s->th, ic, jc, np / 2);
    memcpy(s->Ap, s->A, nf * sizeof(double));
    memcpy(s->Bp, s->B, nf * sizeof(double));
    memcpy(s->Cp, s->C, nf * sizeof(double));
    memcpy(s->thp, s->th, nf * sizeof(double));
    memcpy(s->uelp, s->uel, nf * sizeof(double));
    memcpy(s->velp, s->vel, nf * sizeof(double));
    memcpy(s->welp, s->wel, nf * sizeof(double));
}

/* ------------------------------------------------------------------------ */
/* Transport (rot3dmg.f:341-873)                                             */
/* ------------------------------------------------------------------------ */

/* Avorticity, rot3dmg.f:341-469: i = 1..nr (r = r0 + (i - 1/2) dr),
 * j = 1..nz-1, k = 0..np. */
void orc_r3d_avorticity(orc_r3d_t *s)
{
    const int nr = s->nr, nz = s->nz, np = s->np;
    const double dr = s->dr, dz = s->dz, dp = s->dp, dt = s->dt, Ptl = s->Ptl;
    const double Ra = s->Ra, Re = s->Re, Gr = s->Gr;
    const double *A = s->A, *Ap = s->Ap, *B = s->B, *C = s->C, *th = s->th;
    const double *uel = s->uel, *vel = s->vel, *wel = s->wel;
    double *An = s->An;
    for (int i = 1; i <= nr; ++i)
        for (int j = 1; j <= nz - 1; ++j)
            for (int k = 0; k <= np; ++k) {
                const int im = i - 1, jp = j + 1;
                const int km = k == 0 ? np - 1 : k - 1;
                const int ka = k == np ? 1 : k + 1;
                const double r = s->r0 + ((double)i - 0.5) * dr;
                const double u = (FX(uel, i, j, k) + FX(uel, i, jp, k) + FX(uel, i, j, ka) + FX(uel, i, jp, ka) +
                                  FX(uel, im, j, k) + FX(uel, im, jp, k) + FX(uel, im, j, ka) + FX(uel, im, jp, ka)) *
                                 0.125;
                const double v = (FX(vel, i, jp, k) + FX(vel, i, j, k)) * 0.5;
                const double w = (FX(wel, i, j, ka) + FX(wel, i, j, k)) * 0.5;
                const double tem = (FX(th, i, j, k) + FX(th, i, j, ka) + FX(th, i, jp, k) + FX(th, i, jp, ka)) * 0.25;
                const double BB = (FX(B, i, j, k) + FX(B, im, j, k) + FX(B, i, j, ka) + FX(B, im, j, ka)) * 0.25;
                const double CC = (FX(C, i, j, k) + FX(C, i, jp, k) + FX(C, im, j, k) + FX(C, im, jp, k)) * 0.25;
                double Arra, Ara, Ar, cnr;
                if (i == 1) {
                    Arra = (3.2 * FX(A, i - 1, j, k) + 2.0 * FX(A, i + 1, j, k) - 0.2 * FX(A, i + 2, j, k)) / (dr * dr);
                    Ara = (-4.0 * FX(A, i - 1, j, k) / 3.0 + FX(A, i + 1, j, k) / 3.0) / dr;
                    Ar = (-4.0 * FX(A, i - 1, j, k) / 3.0 + FX(A, i, j, k) + FX(A, i + 1, j, k) / 3.0) / dr;
                    cnr = -2.5 / (dr * dr) + 0.5 / dr / r;
                } else if (i == nr) {
                    Arra = (3.2 * FX(A, i + 1, j, k) + 2.0 * FX(A, i - 1, j, k) - 0.2 * FX(A, i - 2, j, k)) / (dr * dr);
                    Ara = (-FX(A, i - 1, j, k) / 3.0 + 4.0 * FX(A, i + 1, j, k) / 3.0) / dr;
                    /* the inner-wall formula again (rot3dmg.f:390) */
                    Ar = (-4.0 * FX(A, i - 1, j, k) / 3.0 + FX(A, i, j, k) + FX(A, i + 1, j, k) / 3.0) / dr;
                    cnr = -2.5 / (dr * dr) - 0.5 / dr / r;
                } else {
                    Arra = (FX(A, i - 1, j, k) + FX(A, i + 1, j, k)) / (dr * dr);
                    Ara = (FX(A, i + 1, j, k) - FX(A, i - 1, j, k)) * 0.5 / dr;
                    Ar = Ara;
                    cnr = -1.0 / (dr * dr);
                    const double Pe = fabs(u * dr / Ptl);
                    if (Pe > 2.0) {
                        if (u > 0.0) Ar = (FX(A, i, j, k) - FX(A, i - 1, j, k)) / dr;
                        else if (u < 0.0) Ar = (FX(A, i + 1, j, k) - FX(A, i, j, k)) / dr;
                    }
                }
                const double uelr = ((FX(uel, i, j, k) + FX(uel, i, jp, k) + FX(uel, i, j, ka) + FX(uel, i, jp, ka)) * 0.25 -
                                     (FX(uel, im, j, k) + FX(uel, im, jp, k) + FX(uel, im, j, ka) + FX(uel, im, jp, ka)) *
                                         0.25) /
                                    dr;
                const double Azza = (FX(A, i, j - 1, k) + FX(A, i, j + 1, k)) / (dz * dz);
                double Az = (FX(A, i, j + 1, k) - FX(A, i, j - 1, k)) * 0.5 / dz;
                {
                    const double Pe = fabs(w * dz / Ptl);
                    if (Pe > 2.0) {
                        if (w > 0.0) Az = (FX(A, i, j, k) - FX(A, i, j - 1, k)) / dz;
                        else if (w < 0.0) Az = (FX(A, i, j + 1, k) - FX(A, i, j, k)) / dz;
                    }
                }
                const double uelz = ((FX(uel, i, jp, k) + FX(uel, i, jp, ka) + FX(uel, im, jp, k) + FX(uel, im, jp, ka)) * 0.25 -
                                     (FX(uel, i, j, k) + FX(uel, i, j, ka) + FX(uel, im, j, k) + FX(uel, im, j, ka)) * 0.25) /
                                    dz;
                const double thz = (FX(th, i, jp, k) + FX(th, i, jp, ka) - FX(th, i, j, k) - FX(th, i, j, ka)) * 0.5 / dz;
                const double thh = (FX(th, i, j, ka) + FX(th, i, jp, ka) - FX(th, i, j, k) - FX(th, i, jp, k)) * 0.5 / dp;
                const double Ahha = (FX(A, i, j, ka) + FX(A, i, j, km)) / (dp * dp);
                double Ah = (FX(A, i, j, ka) - FX(A, i, j, km)) * 0.5 / dp;
                {
                    const double Pe = fabs(v * dp * r / Ptl);
                    if (Pe > 2.0) {
                        if (v > 0.0) Ah = (FX(A, i, j, k) - FX(A, i, j, km)) / dp;
                        else if (v < 0.0) Ah = (FX(A, i, j, ka) - FX(A, i, j, k)) / dp;
                    }
                }
                const double Bh = (FX(B, i, j, ka) + FX(B, im, j, ka) - FX(B, i, j, k) - FX(B, im, j, k)) * 0.5 / dp;
                const double uelh = ((FX(uel, i, j, ka) + FX(uel, i, jp, ka) + FX(uel, im, j, ka) + FX(uel, im, jp, ka)) * 0.25 -
                                     (FX(uel, i, j, k) + FX(uel, i, jp, k) + FX(uel, im, j, k) + FX(uel, im, jp, k)) * 0.25) /
                                    dp;
                const double cnz = -1.0 / (dz * dz);
                const double cnh = -1.0 / (dp * dp) / (r * r);
                const double RHS1 = Arra + Ara / r + Ahha / (r * r) + Azza - 2.0 * Bh / (r * r) + FX(A, i, j, k) / (Ptl * dt);
                const double ULT = (u * Ar + v * Ah / r + w * Az - uelh * BB / r - uelz * CC) / Ptl;
                const double RHS2 = s->horizontal ? s->sinth[k] * Gr * Ptl * thz
                                                  : -2.0 * Re * uelz + 2.0 * Ra * (tem * uelz + thz * u) / Re / Ptl -
                                                        Gr * Ptl / r * thh;
                const double cf1 = 1.0 / (Ptl * dt) - uelr / (2.0 * Ptl) + 1.0 / (2.0 * (r * r)) - cnr - cnz - cnh;
                const double cf2 = uelr / (2.0 * Ptl) - 1.0 / (2.0 * (r * r)) + cnr + cnz + cnh;
                FX(An, i, j, k) = (cf2 * FX(Ap, i, j, k) - ULT - RHS2 + RHS1) / cf1;
            }
}

/* Bvorticity, rot3dmg.f:477-593: i = 1..nr-1 (r = r0 + i dr), j = 1..nz-1,
 * k = 0..np. */
void orc_r3d_bvorticity(orc_r3d_t *s)
{
    const int nr = s->nr, nz = s->nz, np = s->np;
    const double dr = s->dr, dz = s->dz, dp = s->dp, dt = s->dt, Ptl = s->Ptl;
    const double Ra = s->Ra, Re = s->Re, Gr = s->Gr;
    const double *A = s->A, *B = s->B, *Bp = s->Bp, *C = s->C, *th = s->th;
    const double *uel = s->uel, *vel = s->vel, *wel = s->wel;
    double *Bn = s->Bn;
    for (int i = 1; i <= nr - 1; ++i)
        for (int j = 1; j <= nz - 1; ++j)
            for (int k = 0; k <= np; ++k) {
                const int ip = i + 1, jp = j + 1;
                const int km = k == 0 ? np - 1 : k - 1;
                const int ka = k == np ? 1 : k + 1;
                const double r = s->r0 + (double)i * dr;
                const double u = (FX(uel, i, j, k) + FX(uel, i, jp, k)) * 0.5;
                const double v = (FX(vel, i, j, km) + FX(vel, i, jp, km) + FX(vel, i, j, k) + FX(vel, i, jp, k) +
                                  FX(vel, ip, j, km) + FX(vel, ip, jp, km) + FX(vel, ip, j, k) + FX(vel, ip, jp, k)) *
                                 0.125;
                const double w = (FX(wel, i, j, k) + FX(wel, ip, j, k)) * 0.5;
                const double tem = (FX(th, i, jp, k) + FX(th, ip, jp, k) + FX(th, i, j, k) + FX(th, ip, j, k)) * 0.25;
                const double AA = (FX(A, i, j, k) + FX(A, ip, j, k) + FX(A, i, j, km) + FX(A, ip, j, km)) * 0.25;
                const double CC = (FX(C, i, j, k) + FX(C, i, jp, k) + FX(C, i, j, km) + FX(C, i, jp, km)) * 0.25;
                const double Brra = (FX(B, i - 1, j, k) + FX(B, i + 1, j, k)) / (dr * dr);
                const double Bra = (FX(B, i + 1, j, k) - FX(B, i - 1, j, k)) * 0.5 / dr;
                double Br = Bra;
                {
                    const double Pe = fabs(u * dr / Ptl);
                    if (Pe > 2.0) {
                        if (u > 0.0) Br = (FX(B, i, j, k) - FX(B, i - 1, j, k)) / dr;
                        else if (u < 0.0) Br = (FX(B, i + 1, j, k) - FX(B, i, j, k)) / dr;
                    }
                }
                const double velr = ((FX(vel, ip, j, km) + FX(vel, ip, jp, km) + FX(vel, ip, j, k) + FX(vel, ip, jp, k)) * 0.25 -
                                     (FX(vel, i, j, km) + FX(vel, i, jp, km) + FX(vel, i, j, k) + FX(vel, i, jp, k)) * 0.25) /
                                    dr;
                const double Bzza = (FX(B, i, j - 1, k) + FX(B, i, j + 1, k)) / (dz * dz);
                double Bz = (FX(B, i, j + 1, k) - FX(B, i, j - 1, k)) * 0.5 / dz;
                {
                    const double Pe = fabs(w * dz / Ptl);
                    if (Pe > 2.0) {
                        if (w > 0.0) Bz = (FX(B, i, j, k) - FX(B, i, j - 1, k)) / dz;
                        else if (w < 0.0) Bz = (FX(B, i, j + 1, k) - FX(B, i, j, k)) / dz;
                    }
                }
                const double velz = ((FX(vel, i, jp, km) + FX(vel, ip, jp, km) + FX(vel, i, jp, k) + FX(vel, ip, jp, k)) * 0.25 -
                                     (FX(vel, i, j, km) + FX(vel, ip, j, km) + FX(vel, i, j, k) + FX(vel, ip, j, k)) * 0.25) /
                                    dz;
                const double thz = (FX(th, i, jp, k) + FX(th, ip, jp, k) - FX(th, i, j, k) - FX(th, ip, j, k)) * 0.5 / dz;
                const double thr = (FX(th, ip, jp, k) + FX(th, ip, j, k) - FX(th, i, jp, k) - FX(th, i, j, k)) * 0.5 / dr;
                const double Bhha = (FX(B, i, j, ka) + FX(B, i, j, km)) / (dp * dp);
                double Bh = (FX(B, i, j, ka) - FX(B, i, j, km)) * 0.5 / dp;
                {
                    const double Pe = fabs(v * dp * r / Ptl);
                    if (Pe > 2.0) {
                        if (v > 0.0) Bh = (FX(B, i, j, k) - FX(B, i, j, km)) / dp;
                        else if (v < 0.0) Bh = (FX(B, i, j, ka) - FX(B, i, j, k)) / dp;
                    }
                }
                const double Ah = (FX(A, i, j, k) + FX(A, ip, j, k) - FX(A, i, j, km) - FX(A, ip, j, km)) * 0.5 / dp;
                const double velh = ((FX(vel, i, j, k) + FX(vel, ip, j, k) + FX(vel, i, jp, k) + FX(vel, ip, jp, k)) * 0.25 -
                                     (FX(vel, i, j, km) + FX(vel, ip, j, km) + FX(vel, i, jp, km) + FX(vel, ip, jp, km)) *
                                         0.25) /
                                    dp;
                const double cnr = -1.0 / (dr * dr);
                const double cnz = -1.0 / (dz * dz);
                const double cnh = -1.0 / (dp * dp) / (r * r);
                const double RHS1 = Brra + Bra / r + Bhha / (r * r) + Bzza + 2.0 * Ah / (r * r) + FX(B, i, j, k) / (Ptl * dt);
                const double ULT = (u * Br + v * Bh / r + w * Bz - (velr - v / r) * AA - velz * CC) / Ptl;
                const double RHS2 =
                    s->horizontal ? s->costh[k] * Gr * Ptl * thz
                                  : -2.0 * Re * velz + r * Ra * thz + 2.0 * Ra * (tem * velz + thz * v) / Re / Ptl +
                                        Gr * Ptl * thr;
                const double cf1 = 1.0 / (Ptl * dt) - (u / r + velh / r) / (2.0 * Ptl) + 1.0 / (2.0 * (r * r)) - cnr - cnz - cnh;
                const double cf2 = (u / r + velh / r) / (2.0 * Ptl) - 1.0 / (2.0 * (r * r)) + cnr + cnz + cnh;
                FX(Bn, i, j, k) = (cf2 * FX(Bp, i, j, k) - ULT - RHS2 + RHS1) / cf1;
            }
}

/* Cvorticity, rot3dmg.f:601-728: i = 1..nr-1 (r = r0 + i dr), j = 1..nz,
 * k = 0..np; one-sided z stencils at j = 1 and j = nz. */
void orc_r3d_cvorticity(orc_r3d_t *s)
{
    const int nr = s->nr, nz = s->nz, np = s->np;
    const double dr = s->dr, dz = s->dz, dp = s->dp, dt = s->dt, Ptl = s->Ptl;
    const double Ra = s->Ra, Re = s->Re;
    const double *A = s->A, *B = s->B, *C = s->C, *Cp = s->Cp, *th = s->th;
    const double *uel = s->uel, *vel = s->vel, *wel = s->wel;
    double *Cn = s->Cn;
    for (int i = 1; i <= nr - 1; ++i)
        for (int j = 1; j <= nz; ++j)
            for (int k = 0; k <= np; ++k) {
                const int ip = i + 1, im = i - 1, jm = j - 1;
                const int km = k == 0 ? np - 1 : k - 1;
                const int ka = k == np ? 1 : k + 1;
                const double r = s->r0 + (double)i * dr;
                const double u = (FX(uel, i, j, ka) + FX(uel, i, j, k)) * 0.5;
                const double v = (FX(vel, i, j, k) + FX(vel, ip, j, k)) * 0.5;
                const double w = (FX(wel, i, j, k) + FX(wel, ip, j, k) + FX(wel, i, j, ka) + FX(wel, ip, j, ka) +
                                  FX(wel, i, jm, k) + FX(wel, ip, jm, k) + FX(wel, i, jm, ka) + FX(wel, ip, jm, ka)) *
                                 0.125;
                const double AA = (FX(A, i, j, k) + FX(A, i, jm, k) + FX(A, ip, j, k) + FX(A, ip, jm, k)) * 0.25;
                const double BB = (FX(B, i, j, k) + FX(B, i, jm, k) + FX(B, i, j, ka) + FX(B, i, jm, ka)) * 0.25;
                const double tem = (FX(th, i, j, k) + FX(th, ip, j, k) + FX(th, ip, j, ka) + FX(th, i, j, ka)) * 0.25;
                const double Crra = (FX(C, i - 1, j, k) + FX(C, i + 1, j, k)) / (dr * dr);
                const double Cra = (FX(C, i + 1, j, k) - FX(C, i - 1, j, k)) * 0.5 / dr;
                double Cr = Cra;
                {
                    const double Pe = fabs(u * dr / Ptl);
                    if (Pe > 2.0) {
                        if (u > 0.0) Cr = (FX(C, i, j, k) - FX(C, i - 1, j, k)) / dr;
                        else if (u < 0.0) Cr = (FX(C, i + 1, j, k) - FX(C, i, j, k)) / dr;
                    }
                }
                const double welr = ((FX(wel, ip, j, k) + FX(wel, ip, j, ka) + FX(wel, ip, jm, k) + FX(wel, ip, jm, ka)) * 0.25 -
                                     (FX(wel, i, j, k) + FX(wel, i, j, ka) + FX(wel, i, jm, k) + FX(wel, i, jm, ka)) * 0.25) /
                                    dr;
                const double uelr = (FX(uel, ip, j, k) + FX(uel, ip, j, ka) - FX(uel, im, j, k) - FX(uel, im, j, ka)) * 0.25 / dr;
                const double thr = (FX(th, ip, j, k) + FX(th, ip, j, ka) - FX(th, i, j, k) - FX(th, i, j, ka)) * 0.5 / dr;
                (void)uelr;
                double Czza, Cz, cnz;
                if (j == 1) {
                    Czza = (3.2 * FX(C, i, j - 1, k) + 2.0 * FX(C, i, j + 1, k) - 0.2 * FX(C, i, j + 2, k)) / (dz * dz);
                    Cz = (-4.0 * FX(C, i, j - 1, k) / 3.0 + FX(C, i, j, k) + FX(C, i, j + 1, k) / 3.0) / dz;
                    cnz = -2.5 / (dz * dz);
                } else if (j == nz) {
                    Czza = (3.2 * FX(C, i, j + 1, k) + 2.0 * FX(C, i, j - 1, k) - 0.2 * FX(C, i, j - 2, k)) / (dz * dz);
                    Cz = (-FX(C, i, j - 1, k) / 3.0 - FX(C, i, j, k) + 4.0 * FX(C, i, j + 1, k) / 3.0) / dz;
                    cnz = -2.5 / (dz * dz);
                } else {
                    Czza = (FX(C, i, j - 1, k) + FX(C, i, j + 1, k)) / (dz * dz);
                    Cz = (FX(C, i, j + 1, k) - FX(C, i, j - 1, k)) * 0.5 / dz;
                    const double Pe = fabs(w * dz / Ptl);
                    if (Pe > 2.0) {
                        if (w > 0.0) Cz = (FX(C, i, j, k) - FX(C, i, j - 1, k)) / dz;
                        else if (w < 0.0) Cz = (FX(C, i, j + 1, k) - FX(C, i, j, k)) / dz;
                    }
                    cnz = -1.0 / (dz * dz);
                }
                const double welz = ((FX(wel, i, j, k) + FX(wel, ip, j, k) + FX(wel, i, j, ka) + FX(wel, ip, j, ka)) * 0.25 -
                                     (FX(wel, i, jm, k) + FX(wel, ip, jm, k) + FX(wel, i, jm, ka) + FX(wel, ip, jm, ka)) * 0.25) /
                                    dz;
                const double Chha = (FX(C, i, j, ka) + FX(C, i, j, km)) / (dp * dp);
                double Ch = (FX(C, i, j, ka) - FX(C, i, j, km)) * 0.5 / dp;
                {
                    const double Pe = fabs(v * dp * r / Ptl);
                    if (Pe > 2.0) {
                        if (v > 0.0) Ch = (FX(C, i, j, k) - FX(C, i, j, km)) / dp;
                        else if (v < 0.0) Ch = (FX(C, i, j, ka) - FX(C, i, j, k)) / dp;
                    }
                }
                const double welh = ((FX(wel, i, j, ka) + FX(wel, ip, j, ka) + FX(wel, i, jm, ka) + FX(wel, ip, jm, ka)) * 0.25 -
                                     (FX(wel, i, j, k) + FX(wel, ip, j, k) + FX(wel, i, jm, k) + FX(wel, ip, jm, k)) * 0.25) /
                                    dp;
                const double velh = (FX(vel, i, j, ka) + FX(vel, ip, j, ka) - FX(vel, i, j, km) - FX(vel, ip, j, km)) * 0.25 / dp;
                const double thh = (FX(th, i, j, ka) + FX(th, ip, j, ka) - FX(th, i, j, k) - FX(th, ip, j, k)) * 0.5 / dp;
                (void)velh;
                const double cnr = -1.0 / (dr * dr);
                const double cnh = -1.0 / (dp * dp) / (r * r);
                const double RHS1 = Crra + Cra / r + Chha / (r * r) + Czza + FX(C, i, j, k) / (Ptl * dt);
                const double ULT = (u * Cr + v * Ch / r + w * Cz - welr * AA - welh * BB / r) / Ptl;
                const double RHS2 =
                    s->horizontal ? -(1.0 / r * s->Gr * Ptl * s->costh[k] * thh) - s->Gr * Ptl * s->sinth[k] * thr
                                  : -2.0 * Re * welz - Ra * thh + 2.0 * Ra * (tem * welz - thr * u - thh * v / r) / Re / Ptl;
                const double cf1 = 1.0 / (Ptl * dt) - welz / (2.0 * Ptl) - cnr - cnz - cnh;
                const double cf2 = welz / (2.0 * Ptl) + cnr + cnz + cnh;
                FX(Cn, i, j, k) = (cf2 * FX(Cp, i, j, k) - ULT - RHS2 + RHS1) / cf1;
            }
}

/* temperature, rot3dmg.f:736-873: i = 1..nr (r = r0 + (i - 1/2) dr),
 * j = 0..nz+1 (the end-wall rows j = 0, nz+1 with zero velocity and the
 * adiabatic stencil 8 th(j+-1)/dz^2), k = 0..np. */
void orc_r3d_temperature(orc_r3d_t *s)
{
    const int nr = s->nr, nz = s->nz, np = s->np;
    const double dr = s->dr, dz = s->dz, dp = s->dp, dt = s->dt, Ptl = s->Ptl;
    const double *th = s->th, *thp = s->thp, *uel = s->uel, *vel = s->vel, *wel = s->wel;
    double *thn = s->thn;
    for (int i = 1; i <= nr; ++i)
        for (int j = 0; j <= nz + 1; ++j)
            for (int k = 0; k <= np; ++k) {
                const int im = i - 1, jm = j - 1;
                const int km = k == 0 ? np - 1 : k - 1;
                const int ka = k == np ? 1 : k + 1;
                const double r = s->r0 + ((double)i - 0.5) * dr;
                double u, v, w;
                if (j == 0 || j == nz + 1) {
                    u = 0.0;
                    v = 0.0;
                    w = 0.0;
                } else {
                    u = (FX(uel, i, j, k) + FX(uel, im, j, k)) * 0.5;
                    v = (FX(vel, i, j, k) + FX(vel, i, j, km)) * 0.5;
                    w = (FX(wel, i, j, k) + FX(wel, i, jm, k)) * 0.5;
                }
                double thrra, thra, thr, cnr;
                if (i == 1) {
                    thrra = (3.2 * FX(th, i - 1, j, k) + 2.0 * FX(th, i + 1, j, k) - 0.2 * FX(th, i + 2, j, k)) / (dr * dr);
                    thra = (-4.0 * FX(th, i - 1, j, k) / 3.0 + FX(th, i + 1, j, k) / 3.0) / dr;
                    thr = (-4.0 * FX(th, i - 1, j, k) / 3.0 + FX(th, i, j, k) + FX(th, i + 1, j, k) / 3.0) / dr;
                    cnr = -2.5 / (dr * dr) + 0.5 / dr / r;
                } else if (i == nr) {
                    thrra = (3.2 * FX(th, i + 1, j, k) + 2.0 * FX(th, i - 1, j, k) - 0.2 * FX(th, i - 2, j, k)) / (dr * dr);
                    thra = (-FX(th, i - 1, j, k) / 3.0 + 4.0 * FX(th, i + 1, j, k) / 3.0) / dr;
                    thr = (-FX(th, i - 1, j, k) / 3.0 - FX(th, i, j, k) + 4.0 * FX(th, i + 1, j, k) / 3.0) / dr;
                    cnr = -2.5 / (dr * dr) - 0.5 / dr / r;
                } else {
                    thrra = (FX(th, i - 1, j, k) + FX(th, i + 1, j, k)) / (dr * dr);
                    thra = (FX(th, i + 1, j, k) - FX(th, i - 1, j, k)) * 0.5 / dr;
                    thr = thra;
                    const double Pe = fabs(u * dr / Ptl);
                    if (Pe > 2.0) {
                        if (u > 0.0) thr = (FX(th, i, j, k) - FX(th, i - 1, j, k)) / dr;
                        else if (u < 0.0) thr = (FX(th, i + 1, j, k) - FX(th, i, j, k)) / dr;
                    }
                    cnr = -1.0 / (dr * dr);
                }
                double thzza, thz, cnz;
                if (j == 1) {
                    thzza = (3.2 * FX(th, i, j - 1, k) + 2.0 * FX(th, i, j + 1, k) - 0.2 * FX(th, i, j + 2, k)) / (dz * dz);
                    thz = (-4.0 * FX(th, i, j - 1, k) / 3.0 + FX(th, i, j, k) + FX(th, i, j + 1, k) / 3.0) / dz;
                    cnz = -2.5 / (dz * dz);
                } else if (j == nz) {
                    thzza = (3.2 * FX(th, i, j + 1, k) + 2.0 * FX(th, i, j - 1, k) - 0.2 * FX(th, i, j - 2, k)) / (dz * dz);
                    thz = (-FX(th, i, j - 1, k) / 3.0 - FX(th, i, j, k) + 4.0 * FX(th, i, j + 1, k) / 3.0) / dz;
                    cnz = -2.5 / (dz * dz);
                } else if (j == 0) {
                    thzza = 8.0 * FX(th, i, j + 1, k) / (dz * dz);
                    thz = 0.0;
                    cnz = -4.0 / (dz * dz);
                } else if (j == nz + 1) {
                    thzza = 8.0 * FX(th, i, j - 1, k) / (dz * dz);
                    thz = 0.0;
                    cnz = -4.0 / (dz * dz);
                } else {
                    thzza = (FX(th, i, j - 1, k) + FX(th, i, j + 1, k)) / (dz * dz);
                    thz = (FX(th, i, j + 1, k) - FX(th, i, j - 1, k)) * 0.5 / dz;
                    const double Pe = fabs(w * dz / Ptl);
                    if (Pe > 2.0) {
                        if (w > 0.0) thz = (FX(th, i, j, k) - FX(th, i, j - 1, k)) / dz;
                        else if (w < 0.0) thz = (FX(th, i, j + 1, k) - FX(th, i, j, k)) / dz;
                    }
                    cnz = -1.0 / (dz * dz);
                }
                const double thhha = (FX(th, i, j, ka) + FX(th, i, j, km)) / (dp * dp);
                double thh = (FX(th, i, j, ka) - FX(th, i, j, km)) * 0.5 / dp;
                {
                    const double Pe = fabs(v * dp * r / Ptl);
                    if (Pe > 2.0) {
                        if (v > 0.0) thh = (FX(th, i, j, k) - FX(th, i, j, km)) / dp;
                        else if (v < 0.0) thh = (FX(th, i, j, ka) - FX(th, i, j, k)) / dp;
                    }
                }
                const double cnp = -1.0 / (dp * dp) / (r * r);
                const double RHS1 = thrra + thra / r + thhha / (r * r) + thzza + FX(th, i, j, k) / dt;
                const double ULT = u * thr + v * thh / r + w * thz;
                const double cf1 = 1.0 / dt - cnr - cnz - cnp;
                const double cf2 = cnr + cnz + cnp;
                FX(thn, i, j, k) = (cf2 * FX(thp, i, j, k) - ULT + RHS1) / cf1;
            }
}

/* heat, rot3dmg.f:882-909: the inner-wall flux, four-point one-sided
 * derivative, trapezoid-like weights 1/240, 1/80, 1/60 in z, summed over
 * k = 1..np. */
double orc_r3d_heat(const orc_r3d_t *s)
{
    const int nz = s->nz, np = s->np;
    const double dr = s->dr, dz = s->dz, dp = s->dp;
    const double *th = s->th;
    double trans1 = 0.0;
#define HT(j, k) ((-184.0 * FX(th, 0, j, k) + 225.0 * FX(th, 1, j, k) - 50.0 * FX(th, 2, j, k) + 9.0 * FX(th, 3, j, k)))
    for (int k = 1; k <= np; ++k) {
        double trans = dz * HT(0, k) / (240.0 * dr);
        trans = trans + dz * HT(1, k) / (80.0 * dr);
        trans = trans + dz * HT(nz, k) / (80.0 * dr);
        trans = trans + dz * HT(nz + 1, k) / (240.0 * dr);
        for (int j = 2; j <= nz - 1; ++j) trans = trans + dz * HT(j, k) / (60.0 * dr);
        trans1 = trans1 + trans * dp;
    }
#undef HT
    return trans1;
}

/* heat(trans1, trans2), rot3dmghor.f:913-945: both cylinders' fluxes over
 * the band j = nz/2-3 .. nz/2+3, weights 1/120 at its ends and 1/60 inside,
 * summed over k = 1..np. */
double orc_r3d_heat2(const orc_r3d_t *s, double *trans2)
{
    const int nr = s->nr, nz = s->nz, np = s->np;
    const double dr = s->dr, dz = s->dz, dp = s->dp;
    const double *th = s->th;
    const int nza = nz / 2 - 3, nzb = nz / 2 + 3;
    double trans1 = 0.0, t2 = 0.0;
#define HA(j, k) ((-184.0 * FX(th, 0, j, k) + 225.0 * FX(th, 1, j, k) - 50.0 * FX(th, 2, j, k) + 9.0 * FX(th, 3, j, k)))
#define HB(j, k) ((184.0 * FX(th, nr + 1, j, k) - 225.0 * FX(th, nr, j, k) + 50.0 * FX(th, nr - 1, j, k) - \
                   9.0 * FX(th, nr - 2, j, k)))
    for (int k = 1; k <= np; ++k) {
        double ta = dz * HA(nza, k) / (120.0 * dr);
        double tb = dz * HB(nza, k) / (120.0 * dr);
        ta = ta + dz * HA(nzb, k) / (120.0 * dr);
        tb = tb + dz * HB(nzb, k) / (120.0 * dr);
        for (int j = nza + 1; j <= nzb - 1; ++j) {
            ta = ta + dz * HA(j, k) / (60.0 * dr);
            tb = tb + dz * HB(j, k) / (60.0 * dr);
        }
        trans1 = trans1 + ta * dp;
        t2 = t2 + tb * dp;
    }
#undef HA
#undef HB
    if (trans2) *trans2 = t2;
    return trans1;
}

/* update, rot3dmg.f:964-1023: wall vorticities from the new velocities,
 * wall temperatures 0 (inner) and 1 (outer; reversed in rot3dmghor.f:1042),
 * then the time levels move. */
void orc_r3d_update(orc_r3d_t *s)
{
    const int nr = s->nr, nz = s->nz, np = s->np;
    const double dr = s->dr, dz = s->dz;
    const double *uel = s->uel, *vel = s->vel, *wel = s->wel;
    for (int i = 1; i <= nr; ++i)
        for (int k = 0; k <= np; ++k) {
            FX(s->An, i, 0, k) = -(3.0 * FX(vel, i, 1, k) - FX(vel, i, 2, k) / 3.0) / dz;
            FX(s->An, i, nz, k) = -(FX(vel, i, nz - 1, k) / 3.0 - 3.0 * FX(vel, i, nz, k)) / dz;
        }
    for (int i = 1; i <= nr - 1; ++i)
        for (int k = 0; k <= np; ++k) {
            FX(s->Bn, i, 0, k) = (3.0 * FX(uel, i, 1, k) - FX(uel, i, 2, k) / 3.0) / dz;
            FX(s->Bn, i, nz, k) = (-3.0 * FX(uel, i, nz, k) + FX(uel, i, nz - 1, k) / 3.0) / dz;
        }
    for (int j = 1; j <= nz - 1; ++j)
        for (int k = 0; k <= np; ++k) {
            FX(s->Bn, 0, j, k) = -(3.0 * FX(wel, 1, j, k) - FX(wel, 2, j, k) / 3.0) / dr;
            FX(s->Bn, nr, j, k) = -(FX(wel, nr - 1, j, k) / 3.0 - 3.0 * FX(wel, nr, j, k)) / dr;
        }
    for (int j = 1; j <= nz; ++j)
        for (int k = 0; k <= np; ++k) {
            FX(s->Cn, 0, j, k) = (3.0 * FX(vel, 1, j, k) - FX(vel, 2, j, k) / 3.0) / dr;
            FX(s->Cn, nr, j, k) = (FX(vel, nr - 1, j, k) / 3.0 - 3.0 * FX(vel, nr, j, k)) / dr;
        }
    for (int j = 0; j <= nz + 1; ++j)
        for (int k = 0; k <= np; ++k) {
            FX(s->thn, 0, j, k) = s->horizontal ? 1.0 : 0.0;
            FX(s->thn, nr + 1, j, k) = s->horizontal ? 0.0 : 1.0;
        }
    const size_t n = field_size(s) * sizeof(double);
    memcpy(s->Ap, s->A, n);
    memcpy(s->A, s->An, n);
    memcpy(s->Bp, s->B, n);
    memcpy(s->B, s->Bn, n);
    memcpy(s->Cp, s->C, n);
    memcpy(s->C, s->Cn, n);
    memcpy(s->thp, s->th, n);
    memcpy(s->th, s->thn, n);
}

/* rhsw, rot3dmg.f:1026-1063 */
void orc_r3d_rhsw(orc_r3d_t *s)
{
    const int nr = s->nr, nz = s->nz, np = s->np;
    const double dr = s->dr, dp = s->dp;
    const double *An = s->An, *Bn = s->Bn;
    for (int i = 1; i <= nr; ++i)
        for (int j = 1; j <= nz - 1; ++j)
            for (int k = 0; k <= np; ++k) {
                const int km = k == 0 ? np - 1 : k - 1;
                const double r = s->r0 + ((double)i - 0.5) * dr;
                const double Ah = (FX(An, i, j, k) - FX(An, i, j, km)) / dp;
                double w;
                if (i == 1) w = Ah / r - FX(Bn, 1, j, k) / dr - 0.5 * FX(Bn, 1, j, k) / r;
                else if (i == nr) w = Ah / r + FX(Bn, nr - 1, j, k) / dr - 0.5 * FX(Bn, nr - 1, j, k) / r;
                else {
                    const double Br = (FX(Bn, i, j, k) - FX(Bn, i - 1, j, k)) / dr;
                    w = Ah / r - Br - 0.5 * (FX(Bn, i, j, k) + FX(Bn, i - 1, j, k)) / r;
                }
                FX(s->wrh, i, j, k) = w;
            }
}

/* rhsv, rot3dmg.f:1066-1108 */
void orc_r3d_rhsv(orc_r3d_t *s)
{
    const int nr = s->nr, nz = s->nz, np = s->np;
    const double dr = s->dr, dz = s->dz;
    const double *An = s->An, *Cn = s->Cn;
    for (int i = 1; i <= nr; ++i)
        for (int j = 1; j <= nz; ++j)
            for (int k = 0; k <= np; ++k) {
                const double r = s->r0 + ((double)i - 0.5) * dr;
                double v;
                if (i == 1) v = FX(Cn, 1, j, k) / dr + FX(Cn, 1, j, k) / r;
                else if (i == nr) v = -FX(Cn, nr - 1, j, k) / dr + FX(Cn, nr - 1, j, k) / r;
                else {
                    const double Cr = (FX(Cn, i, j, k) - FX(Cn, i - 1, j, k)) / dr;
                    v = Cr + (FX(Cn, i, j, k) + FX(Cn, i - 1, j, k)) / r;
                }
                if (j == 1) v = v - FX(An, i, 1, k) / dz;
                else if (j == nz) v = v + FX(An, i, nz - 1, k) / dz;
                else {
                    const double Az = (FX(An, i, j, k) - FX(An, i, j - 1, k)) / dz;
                    v = v - Az;
                }
                FX(s->vrh, i, j, k) = v;
            }
}

/* rhsu, rot3dmg.f:1111-1150 */
void orc_r3d_rhsu(orc_r3d_t *s)
{
    const int nr = s->nr, nz = s->nz, np = s->np;
    const double dr = s->dr, dz = s->dz, dp = s->dp;
    const double *Bn = s->Bn, *Cn = s->Cn, *wel = s->wel;
    for (int i = 1; i <= nr - 1; ++i)
        for (int j = 1; j <= nz; ++j)
            for (int k = 0; k <= np; ++k) {
                const int km = k == 0 ? np - 1 : k - 1;
                const double r = s->r0 + (double)i * dr;
                const double welz =
                    0.5 * (FX(wel, i, j, k) + FX(wel, i + 1, j, k) - FX(wel, i, j - 1, k) - FX(wel, i + 1, j - 1, k)) / dz;
                const double Ch = (FX(Cn, i, j, k) - FX(Cn, i, j, km)) / dp;
                double u;
                if (j == 1) u = FX(Bn, i, 1, k) / dz - Ch / r - 2.0 * welz / r;
                else if (j == nz) u = -FX(Bn, i, nz - 1, k) / dz - Ch / r - 2.0 * welz / r;
                else {
                    const double Bz = (FX(Bn, i, j, k) - FX(Bn, i, j - 1, k)) / dz;
                    u = Bz - Ch / r - 2.0 * welz / r;
                }
                FX(s->urh, i, j, k) = u;
            }
}

/* ------------------------------------------------------------------------ */
/* Multigrid (rot3dmg.f:1216-2344)                                           */
/* ------------------------------------------------------------------------ */

typedef struct {
    int which, n1, n2, n3, L1, L2;
    double r0, hr, hz, hp, hhr, hhz, hhp;
    double *P;           /* psif of the level */
    const double *rf;    /* rhs of the level */
    double *wa, *wb, *wc, *wd, *we, *wr, *ws;
} lev_t;

#define PV(i, j, k) (L->P[(size_t)(i) + (size_t)L->L1 * ((size_t)(j) + (size_t)L->L2 * (size_t)(k))])
#define RF(i, j, k) (L->rf[(size_t)(i) + (size_t)L->L1 * ((size_t)(j) + (size_t)L->L2 * (size_t)(k))])

/* Unknown ranges of the three components on a level: w has i = 1..n1,
 * j = 1..n2-1; v has i = 1..n1, j = 1..n2; u has i = 1..n1-1, j = 1..n2. */
static int imax_of(const lev_t *L) { return L->which == 3 ? L->n1 - 1 : L->n1; }
static int jmax_of(const lev_t *L) { return L->which == 1 ? L->n2 - 1 : L->n2; }

/* r-line (j, k): relax1 :1572-1607 (pdma), relax2 :1770-1822 (pdma),
 * relax3 :2017-2051 (tdma). */
static void line_r(lev_t *L, int j, int k)
{
    const int n1 = L->n1, n2 = L->n2, n3 = L->n3;
    const double hr = L->hr, hhr = L->hhr, hhz = L->hhz, hhp = L->hhp;
    const int ka = k == n3 ? 1 : k + 1, km = k - 1;
    double *a = L->wa, *b = L->wb, *c = L->wc, *d = L->wd, *e = L->we, *rr = L->wr, *x = L->ws;
    if (L->which == 1) {
        for (int i = 1; i <= n1; ++i) {
            const double rval = L->r0 + ((double)i - 0.5) * hr;
            const int q = i - 1;
            if (i == 1) {
                a[q] = 0.0;
                b[q] = 0.0;
                c[q] = -2.0 / hhr - 1.0 / hr / rval * 0.5 - 2.0 / hhz - 2.0 / hhp / (rval * rval);
                d[q] = 5.0 / hhr / 3.0 + 1.0 / hr / rval * 0.5;
                e[q] = -0.2 / hhr;
            } else if (i == n1) {
                a[q] = -0.2 / hhr;
                b[q] = 5.0 / hhr / 3.0 - 1.0 / hr / rval * 0.5;
                c[q] = -2.0 / hhr + 1.0 / hr / rval * 0.5 - 2.0 / hhz - 2.0 / hhp / (rval * rval);
                d[q] = 0.0;
                e[q] = 0.0;
            } else {
                a[q] = 0.0;
                b[q] = 1.0 / hhr - 0.5 / hr / rval;
                c[q] = -(2.0 / hhr + 2.0 / hhz + 2.0 / hhp / (rval * rval));
                d[q] = 1.0 / hhr + 0.5 / hr / rval;
                e[q] = 0.0;
            }
            rr[q] = -(PV(i, j + 1, k) + PV(i, j - 1, k)) / hhz - (PV(i, j, ka) + PV(i, j, km)) / hhp / (rval * rval) +
                    RF(i, j, k);
        }
        orc_pdma(a, b, c, d, e, rr, x, n1);
        for (int i = 1; i <= n1; ++i) {
            PV(i, j, k) = x[i - 1];
            if (k == n3) PV(i, j, 0) = PV(i, j, k);
        }
    } else if (L->which == 2) {
        for (int i = 1; i <= n1; ++i) {
            const double rval = L->r0 + ((double)i - 0.5) * hr;
            const double rq = rval * rval;
            const int q = i - 1;
            if (i == 1) {
                a[q] = 0.0;
                b[q] = 0.0;
                c[q] = -2.0 / hhr - 2.0 / hhp / rq + 1.0 / rq;
                d[q] = 5.0 / 3.0 / hhr + 4.0 / 3.0 / hr / rval;
                e[q] = -0.2 / hhr;
            } else if (i == n1) {
                a[q] = -0.2 / hhr;
                b[q] = 5.0 / 3.0 / hhr - 4.0 / 3.0 / hr / rval;
                c[q] = -2.0 / hhr - 2.0 / hhp / rq + 1.0 / rq;
                d[q] = 0.0;
                e[q] = 0.0;
            } else {
                a[q] = 0.0;
                b[q] = 1.0 / hhr - 1.5 / hr / rval;
                c[q] = -(2.0 / hhr + 2.0 / hhp / rq) + 1.0 / rq;
                d[q] = 1.0 / hhr + 1.5 / hr / rval;
                e[q] = 0.0;
            }
            c[q] = c[q] - 2.0 / hhz;
            if (j == 1)
                rr[q] = -(5.0 / 3.0 * PV(i, j + 1, k) - F02 * PV(i, j + 2, k)) / hhz -
                        (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
            else if (j == n2)
                rr[q] = -(5.0 / 3.0 * PV(i, j - 1, k) - F02 * PV(i, j - 2, k)) / hhz -
                        (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
            else
                rr[q] = -(PV(i, j - 1, k) + PV(i, j + 1, k)) / hhz - (PV(i, j, ka) + PV(i, j, km)) / hhp / rq +
                        RF(i, j, k);
        }
        orc_pdma(a, b, c, d, e, rr, x, n1);
        for (int i = 1; i <= n1; ++i) {
            PV(i, j, k) = x[i - 1];
            if (k == n3) PV(i, j, 0) = PV(i, j, k);
        }
    } else {
        for (int i = 1; i <= n1 - 1; ++i) {
            const double rval = (double)i * hr + L->r0;
            const double rq = rval * rval;
            const int q = i - 1;
            a[q] = 1.0 / hhr - 1.5 / hr / rval;
            b[q] = -(2.0 / hhr - 1.0 / rq + 2.0 / hhp / rq);
            c[q] = 1.0 / hhr + 1.5 / hr / rval;
            b[q] = b[q] - 2.0 / hhz;
            if (j == 1)
                rr[q] = -(5.0 * PV(i, j + 1, k) / 3.0 - F02 * PV(i, j + 2, k)) / hhz -
                        (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
            else if (j == n2)
                rr[q] = -(5.0 * PV(i, j - 1, k) / 3.0 - F02 * PV(i, j - 2, k)) / hhz -
                        (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
            else
                rr[q] = -(PV(i, j - 1, k) + PV(i, j + 1, k)) / hhz - (PV(i, j, ka) + PV(i, j, km)) / hhp / rq +
                        RF(i, j, k);
        }
        orc_tdma(a, b, c, x, rr, n1 - 1);
        for (int i = 1; i <= n1 - 1; ++i) {
            PV(i, j, k) = x[i - 1];
            if (k == n3) PV(i, j, 0) = PV(i, j, k);
        }
    }
}

/* z-line (i, k): relax1 :1609-1646 (tdma), relax2 :1824-1884 (pdma),
 * relax3 :2053-2088 (pdma). */
static void line_z(lev_t *L, int i, int k)
{
    const int n1 = L->n1, n2 = L->n2, n3 = L->n3;
    const double hr = L->hr, hhr = L->hhr, hhz = L->hhz, hhp = L->hhp;
    const int ka = k == n3 ? 1 : k + 1, km = k - 1;
    double *a = L->wa, *b = L->wb, *c = L->wc, *d = L->wd, *e = L->we, *rr = L->wr, *x = L->ws;
    if (L->which == 1) {
        const double rval = L->r0 + ((double)i - 0.5) * hr;
        for (int j = 1; j <= n2 - 1; ++j) {
            const int q = j - 1;
            a[q] = 1.0 / hhz;
            b[q] = -(2.0 / hhz + 2.0 / hhp / (rval * rval));
            c[q] = 1.0 / hhz;
            if (i == 1) {
                b[q] = b[q] - 2.0 / hhr - 1.0 / hr / rval * 0.5;
                rr[q] = -(5.0 * PV(i + 1, j, k) / 3.0 - F02 * PV(i + 2, j, k)) / hhr - 1.0 * PV(i + 1, j, k) / hr / rval * 0.5 -
                        (PV(i, j, ka) + PV(i, j, km)) / hhp / (rval * rval) + RF(i, j, k);
            } else if (i == n1) {
                b[q] = b[q] - 2.0 / hhr + 1.0 / hr / rval * 0.5;
                rr[q] = -(5.0 * PV(i - 1, j, k) / 3.0 - F02 * PV(i - 2, j, k)) / hhr + 1.0 * PV(i - 1, j, k) / hr / rval * 0.5 -
                        (PV(i, j, ka) + PV(i, j, km)) / hhp / (rval * rval) + RF(i, j, k);
            } else {
                b[q] = b[q] - 2.0 / hhr;
                rr[q] = -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 0.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                        (PV(i, j, ka) + PV(i, j, km)) / hhp / (rval * rval) + RF(i, j, k);
            }
        }
        orc_tdma(a, b, c, x, rr, n2 - 1);
        for (int j = 1; j <= n2 - 1; ++j) {
            PV(i, j, k) = x[j - 1];
            if (k == n3) PV(i, j, 0) = PV(i, j, k);
        }
    } else if (L->which == 2) {
        const double rval = L->r0 + ((double)i - 0.5) * hr;
        const double rq = rval * rval;
        for (int j = 1; j <= n2; ++j) {
            const int q = j - 1;
            if (j == 1) {
                a[q] = 0.0;
                b[q] = 0.0;
                c[q] = -2.0 / hhz - 2.0 / hhp / rq + 1.0 / rq;
                d[q] = 5.0 / 3.0 / hhz;
                e[q] = -0.2 / hhz;
            } else if (j == n2) {
                a[q] = -0.2 / hhz;
                b[q] = 5.0 / 3.0 / hhz;
                c[q] = -2.0 / hhz - 2.0 / hhp / rq + 1.0 / rq;
                d[q] = 0.0;
                e[q] = 0.0;
            } else {
                a[q] = 0.0;
                b[q] = 1.0 / hhz;
                c[q] = -(2.0 / hhz + 2.0 / hhp / rq) + 1.0 / rq;
                d[q] = 1.0 / hhz;
                e[q] = 0.0;
            }
            c[q] = c[q] - 2.0 / hhr;
            if (i == 1)
                rr[q] = -(5.0 / 3.0 * PV(i + 1, j, k) - 0.2 * PV(i + 2, j, k)) / hhr - 4.0 / 3.0 * PV(i + 1, j, k) / hr / rval -
                        (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
            else if (i == n1)
                rr[q] = -(5.0 / 3.0 * PV(i - 1, j, k) - 0.2 * PV(i - 2, j, k)) / hhr + 4.0 / 3.0 * PV(i - 1, j, k) / hr / rval -
                        (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
            else
                rr[q] = -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                        (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
        }
        orc_pdma(a, b, c, d, e, rr, x, n2);
        for (int j = 1; j <= n2; ++j) {
            PV(i, j, k) = x[j - 1];
            if (k == n3) PV(i, j, 0) = PV(i, j, k);
        }
    } else {
        const double rval = (double)i * hr + L->r0;
        const double rq = rval * rval;
        for (int j = 1; j <= n2; ++j) {
            const int q = j - 1;
            if (j == 1) {
                a[q] = 0.0;
                b[q] = 0.0;
                c[q] = -2.0 / hhz - 2.0 / hhr + 1.0 / rq - 2.0 / hhp / rq;
                d[q] = 5.0 / hhz / 3.0;
                e[q] = -0.2 / hhz;
            } else if (j == n2) {
                a[q] = -0.2 / hhz;
                b[q] = 5.0 / hhz / 3.0;
                c[q] = -2.0 / hhz - 2.0 / hhr + 1.0 / rq - 2.0 / hhp / rq;
                d[q] = 0.0;
                e[q] = 0.0;
            } else {
                a[q] = 0.0;
                b[q] = 1.0 / hhz;
                c[q] = -(2.0 / hhz + 2.0 / hhr + 2.0 / hhp / rq) + 1.0 / rq;
                d[q] = 1.0 / hhz;
                e[q] = 0.0;
            }
            rr[q] = -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                    (PV(i, j, ka) + PV(i, j, km)) / hhp / rq + RF(i, j, k);
        }
        orc_pdma(a, b, c, d, e, rr, x, n2);
        for (int j = 1; j <= n2; ++j) {
            PV(i, j, k) = x[j - 1];
            if (k == n3) PV(i, j, 0) = PV(i, j, k);
        }
    }
}

/* phi-line (i, j), periodic tdma over k = 1..n3, plane 0 = plane n3:
 * relax1 :1648-1686, relax2 :1886-1933, relax3 :2090-2127. */
static void line_p(lev_t *L, int i, int j)
{
    const int n1 = L->n1, n2 = L->n2, n3 = L->n3;
    const double hr = L->hr, hhr = L->hhr, hhz = L->hhz, hhp = L->hhp;
    double *a = L->wa, *b = L->wb, *c = L->wc, *rr = L->wr, *x = L->ws;
    if (L->which == 1) {
        const double rval = L->r0 + ((double)i - 0.5) * hr;
        for (int k = 1; k <= n3; ++k) {
            const int q = k - 1;
            a[q] = 1.0 / hhp / (rval * rval);
            b[q] = -(2.0 / hhz + 2.0 / hhp / (rval * rval));
            c[q] = 1.0 / hhp / (rval * rval);
            if (i == 1) {
                b[q] = b[q] - 2.0 / hhr - 1.0 / hr / rval * 0.5;
                rr[q] = -(5.0 * PV(i + 1, j, k) / 3.0 - F02 * PV(i + 2, j, k)) / hhr - PV(i + 1, j, k) / hr / rval * 0.5 -
                        (PV(i, j + 1, k) + PV(i, j - 1, k)) / hhz + RF(i, j, k);
            } else if (i == n1) {
                b[q] = b[q] - 2.0 / hhr + 1.0 / hr / rval * 0.5;
                rr[q] = -(5.0 * PV(i - 1, j, k) / 3.0 - F02 * PV(i - 2, j, k)) / hhr + PV(i - 1, j, k) / hr / rval * 0.5 -
                        (PV(i, j + 1, k) + PV(i, j - 1, k)) / hhz + RF(i, j, k);
            } else {
                b[q] = b[q] - 2.0 / hhr;
                rr[q] = -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 0.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                        (PV(i, j + 1, k) + PV(i, j - 1, k)) / hhz + RF(i, j, k);
            }
        }
    } else if (L->which == 2) {
        const double rval = L->r0 + ((double)i - 0.5) * hr;
        const double rq = rval * rval;
        for (int k = 1; k <= n3; ++k) {
            const int q = k - 1;
            a[q] = 1.0 / hhp / rq;
            c[q] = 1.0 / hhp / rq;
            b[q] = -(2.0 / hhp / rq) + 1.0 / rq;
            if (i == 1) {
                b[q] = b[q] - 2.0 / hhr;
                rr[q] = -(5.0 / 3.0 * PV(i + 1, j, k) - 0.2 * PV(i + 2, j, k)) / hhr - 4.0 / 3.0 * PV(i + 1, j, k) / hr / rval;
            } else if (i == n1) {
                b[q] = b[q] - 2.0 / hhr;
                rr[q] = -(5.0 / 3.0 * PV(i - 1, j, k) - 0.2 * PV(i - 2, j, k)) / hhr + 4.0 / 3.0 * PV(i - 1, j, k) / hr / rval;
            } else {
                b[q] = b[q] - 2.0 / hhr;
                rr[q] = -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval;
            }
            if (j == 1) {
                b[q] = b[q] - 2.0 / hhz;
                rr[q] = rr[q] - (5.0 / 3.0 * PV(i, j + 1, k) - 0.2 * PV(i, j + 2, k)) / hhz + RF(i, j, k);
            } else if (j == n2) {
                b[q] = b[q] - 2.0 / hhz;
                rr[q] = rr[q] - (5.0 / 3.0 * PV(i, j - 1, k) - 0.2 * PV(i, j - 2, k)) / hhz + RF(i, j, k);
            } else {
                b[q] = b[q] - 2.0 / hhz;
                rr[q] = rr[q] - (PV(i, j - 1, k) + PV(i, j + 1, k)) / hhz + RF(i, j, k);
            }
        }
    } else {
        const double rval = (double)i * hr + L->r0;
        const double rq = rval * rval;
        for (int k = 1; k <= n3; ++k) {
            const int q = k - 1;
            a[q] = 1.0 / hhp / rq;
            b[q] = -(2.0 / hhr - 1.0 / rq + 2.0 / hhp / rq);
            c[q] = 1.0 / hhp / rq;
            b[q] = b[q] - 2.0 / hhz;
            if (j == 1)
                rr[q] = -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                        (5.0 * PV(i, j + 1, k) / 3.0 - F02 * PV(i, j + 2, k)) / hhz + RF(i, j, k);
            else if (j == n2)
                rr[q] = -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                        (5.0 * PV(i, j - 1, k) / 3.0 - F02 * PV(i, j - 2, k)) / hhz + RF(i, j, k);
            else
                rr[q] = -(PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr - 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval -
                        (PV(i, j + 1, k) + PV(i, j - 1, k)) / hhz + RF(i, j, k);
        }
    }
    orc_ptdma(a, b, c, x, rr, n3);
    for (int k = 0; k <= n3; ++k) PV(i, j, k) = k == 0 ? x[n3 - 1] : x[k - 1];
}

/* Residual rc = rf - A psif at the unknowns of the level and its max norm:
 * relax1 :1688-1720, relax2 :1935-1977, relax3 :2129-2160. */
static double residual(lev_t *L, double *rc, int *anynan)
{
    const int n1 = L->n1, n2 = L->n2, n3 = L->n3;
    const double hr = L->hr, hhr = L->hhr, hhz = L->hhz, hhp = L->hhp;
    double resmax = 0.0;
#define RC(i, j, k) (rc[(size_t)(i) + (size_t)L->L1 * ((size_t)(j) + (size_t)L->L2 * (size_t)(k))])
    const int im = imax_of(L), jm = jmax_of(L);
    for (int i = 1; i <= im; ++i) {
        const double rval = L->which == 3 ? (double)i * hr + L->r0 : L->r0 + ((double)i - 0.5) * hr;
        for (int j = 1; j <= jm; ++j)
            for (int k = 1; k <= n3; ++k) {
                const int ka = k == n3 ? 1 : k + 1, km = k - 1;
                double temp;
                if (L->which == 1) {
                    temp = (PV(i, j + 1, k) + PV(i, j - 1, k)) / hhz + (PV(i, j, ka) + PV(i, j, km)) / hhp / (rval * rval) -
                           PV(i, j, k) * (2.0 / hhz + 2.0 / hhp / (rval * rval));
                    if (i == 1)
                        temp = temp +
                               (-2.0 * PV(i, j, k) + 5.0 * PV(i + 1, j, k) / 3.0 - 0.2 * PV(i + 2, j, k)) / hhr +
                               0.5 * (-PV(i, j, k) + PV(i + 1, j, k)) / hr / rval;
                    else if (i == n1)
                        temp = temp +
                               (-2.0 * PV(i, j, k) + 5.0 * PV(i - 1, j, k) / 3.0 - 0.2 * PV(i - 2, j, k)) / hhr +
                               0.5 * (PV(i, j, k) - PV(i - 1, j, k)) / hr / rval;
                    else
                        temp = temp + (PV(i - 1, j, k) - 2.0 * PV(i, j, k) + PV(i + 1, j, k)) / hhr +
                               0.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval;
                } else if (L->which == 2) {
                    const double rq = rval * rval;
                    temp = (PV(i, j, ka) - 2.0 * PV(i, j, k) + PV(i, j, km)) / hhp / rq + PV(i, j, k) / rq;
                    if (i == 1)
                        temp = temp +
                               (-2.0 * PV(i, j, k) + 5.0 / 3.0 * PV(i + 1, j, k) - 0.2 * PV(i + 2, j, k)) / hhr +
                               4.0 / 3.0 * PV(i + 1, j, k) / hr / rval;
                    else if (i == n1)
                        temp = temp +
                               (-2.0 * PV(i, j, k) + 5.0 / 3.0 * PV(i - 1, j, k) - 0.2 * PV(i - 2, j, k)) / hhr -
                               4.0 / 3.0 * PV(i - 1, j, k) / hr / rval;
                    else
                        temp = temp + (PV(i - 1, j, k) - 2.0 * PV(i, j, k) + PV(i + 1, j, k)) / hhr +
                               1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval;
                    if (j == 1)
                        temp = temp + (-2.0 * PV(i, j, k) + 5.0 / 3.0 * PV(i, j + 1, k) - 0.2 * PV(i, j + 2, k)) / hhz;
                    else if (j == n2)
                        temp = temp + (-2.0 * PV(i, j, k) + 5.0 / 3.0 * PV(i, j - 1, k) - 0.2 * PV(i, j - 2, k)) / hhz;
                    else
                        temp = temp + (PV(i, j + 1, k) - 2.0 * PV(i, j, k) + PV(i, j - 1, k)) / hhz;
                } else {
                    const double rq = rval * rval;
                    temp = (PV(i + 1, j, k) + PV(i - 1, j, k)) / hhr + 1.5 * (PV(i + 1, j, k) - PV(i - 1, j, k)) / hr / rval +
                           PV(i, j, k) / rq + (PV(i, j, ka) + PV(i, j, km)) / hhp / rq -
                           PV(i, j, k) * (2.0 / hhr + 2.0 / hhp / rq);
                    if (j == 1)
                        temp = temp + (-2.0 * PV(i, j, k) + 5.0 * PV(i, j + 1, k) / 3.0 - 0.2 * PV(i, j + 2, k)) / hhz;
                    else if (j == n2)
                        temp = temp + (-2.0 * PV(i, j, k) + 5.0 * PV(i, j - 1, k) / 3.0 - 0.2 * PV(i, j - 2, k)) / hhz;
                    else
                        temp = temp + (PV(i, j + 1, k) - 2.0 * PV(i, j, k) + PV(i, j - 1, k)) / hhz;
                }
                temp = RF(i, j, k) - temp;
                RC(i, j, k) = temp;
                temp = fabs(temp);
                if (temp != temp) *anynan = 1;
                if (temp > resmax) resmax = temp;
            }
    }
#undef RC
    return resmax;
}

/* Which transverse index of a pass has one-sided rows (reads two lines
 * over): i for w and v, j for v and u. */
static int onesided_i(int which) { return which != 3; }
static int onesided_j(int which) { return which != 1; }

static int line_class(int p, int P, int p_os, int q, int Q, int q_os)
{
    return (p_os && (p == 1 || p == P)) + (q_os && (q == 1 || q == Q));
}

/* One direction of one relaxation sweep in the chosen order.  dir 0:
 * r-lines (p, q) = (j, k); 1: z-lines (i, k); 2: phi-lines (i, j). */
static void pass(lev_t *L, int dir, int mode)
{
    const int w = L->which;
    int P, Q, p_os, q_os;
    if (dir == 0) {
        P = jmax_of(L);
        Q = L->n3;
        p_os = onesided_j(w);
        q_os = 0;
    } else if (dir == 1) {
        P = imax_of(L);
        Q = L->n3;
        p_os = onesided_i(w);
        q_os = 0;
    } else {
        P = imax_of(L);
        Q = jmax_of(L);
        p_os = onesided_i(w);
        q_os = onesided_j(w);
    }
    for (int colour = 0; colour < (mode == R3D_LEX ? 1 : 2); ++colour)
        for (int cls = (mode == R3D_LEX ? 0 : 2); cls >= 0; --cls)
            for (int q = 1; q <= Q; ++q)
                for (int p = 1; p <= P; ++p) {
                    if (mode != R3D_LEX && (((p + q) & 1) != colour || line_class(p, P, p_os, q, Q, q_os) != cls))
                        continue;
                    if (dir == 0) line_r(L, p, q);
                    else if (dir == 1) line_z(L, p, q);
                    else line_p(L, p, q);
                }
}

static void level_ctx(orc_r3d_t *s, int which, int klev, lev_t *L, double *buf)
{
    L->which = which;
    L->n1 = s->n1[klev];
    L->n2 = s->n2[klev];
    L->n3 = s->n3[klev];
    L->L1 = L->n1 + 1;
    L->L2 = L->n2 + 1;
    L->r0 = s->r0;
    L->hr = s->hr[klev];
    L->hz = s->hz[klev];
    L->hp = s->hp[klev];
    L->hhr = s->hhr[klev];
    L->hhz = s->hhz[klev];
    L->hhp = s->hhp[klev];
    L->P = s->v[klev];
    L->rf = s->f[klev];
    const int nmax = (L->n1 > L->n2 ? (L->n1 > L->n3 ? L->n1 : L->n3) : (L->n2 > L->n3 ? L->n2 : L->n3)) + 2;
    L->wa = buf;
    L->wb = buf + nmax;
    L->wc = buf + 2 * nmax;
    L->wd = buf + 3 * nmax;
    L->we = buf + 4 * nmax;
    L->wr = buf + 5 * nmax;
    L->ws = buf + 6 * nmax;
}

void orc_r3d_relax(orc_r3d_t *s, int which, int nrel, int klev, int *nconv)
{
    lev_t L;
    const int nmax = (s->n1[klev] > s->n2[klev] ? s->n1[klev] : s->n2[klev]) + s->n3[klev] + 2;
    double *buf = (double *)malloc(sizeof(double) * (size_t)nmax * 7);
    level_ctx(s, which, klev, &L, buf);
    *nconv = 0;
    double resmax = 0.0;
    int anynan = 0;
    for (int irel = 1; irel <= nrel; ++irel) {
        pass(&L, 0, s->mode);
        pass(&L, 1, s->mode);
        pass(&L, 2, s->mode);
        anynan = 0;
        resmax = residual(&L, s->res[klev], &anynan);
    }
    free(buf);
    if (klev == 1) s->last_resmax = anynan ? NAN : resmax;
    if (klev == 1 && resmax < s->tolcon) *nconv = 1;
}

/* corser, rot3dmg.f:2176-2265: 27-point full weighting of the fine
 * residual onto the coarse interior planes k = 1..n3c-1, summed as the
 * centre, faces, edges and corners with a doubling between groups; faces
 * i = 0, n1c and j = 0, n2c zero.  The restriction never writes the planes
 * k = 0 and k = n3c: the coarse right-hand side there is what the shared
 * residual array holds, zero on plane 0 and the fine residual at fine
 * index (i, j, n3c) on plane n3c.  The coarse correction starts at zero. */
void orc_r3d_corser(orc_r3d_t *s, int klev)
{
    const int n1 = s->n1[klev], n2 = s->n2[klev];
    const int n1c = s->n1[klev + 1], n2c = s->n2[klev + 1], n3c = s->n3[klev + 1];
    const double *rf = s->res[klev];
    double *fc = s->f[klev + 1];
    const size_t F1 = (size_t)n1 + 1, F2 = (size_t)n2 + 1;
    const size_t C1 = (size_t)n1c + 1, C2 = (size_t)n2c + 1;
#define R(i, j, k) rf[(size_t)(i) + F1 * ((size_t)(j) + F2 * (size_t)(k))]
#define FC(i, j, k) fc[(size_t)(i) + C1 * ((size_t)(j) + C2 * (size_t)(k))]
    for (int k = 0; k <= n3c; ++k)
        for (int j = 0; j <= n2c; ++j)
            for (int i = 0; i <= n1c; ++i) {
                double val;
                if (i == 0 || i == n1c || j == 0 || j == n2c) {
                    val = 0.0;
                } else if (k == 0 || k == n3c) {
                    val = R(i, j, k);
                } else {
                    const int ii = i + i, jj = j + j, kk = k + k;
                    const int iip = ii + 1, iim = ii - 1, jjp = jj + 1, jjm = jj - 1, kkp = kk + 1, kkm = kk - 1;
                    double temp = R(ii, jj, kk);
                    temp = temp + temp + R(iip, jj, kk) + R(iim, jj, kk) + R(ii, jjp, kk) + R(ii, jjm, kk) +
                           R(ii, jj, kkp) + R(ii, jj, kkm);
                    temp = temp + temp + R(iip, jjp, kk) + R(iip, jjm, kk) + R(iim, jjp, kk) + R(iim, jjm, kk) +
                           R(iip, jj, kkp) + R(iip, jj, kkm) + R(iim, jj, kkp) + R(iim, jj, kkm) + R(ii, jjp, kkp) +
                           R(ii, jjp, kkm) + R(ii, jjm, kkp) + R(ii, jjm, kkm);
                    temp = temp + temp + R(iip, jjp, kkp) + R(iip, jjp, kkm) + R(iip, jjm, kkp) + R(iip, jjm, kkm) +
                           R(iim, jjm, kkp) + R(iim, jjm, kkm) + R(iim, jjp, kkp) + R(iim, jjp, kkm);
                    val = temp * 0.015625;
                }
                FC(i, j, k) = val;
            }
#undef R
#undef FC
    memset(s->v[klev + 1], 0, level_size(s, klev + 1) * sizeof(double));
}

/* finer, rot3dmg.f:2268-2344: trilinear prolongation of the coarse
 * correction (sums in the reference's order) added to the fine level; the
 * coarse correction is cleared. */
void orc_r3d_finer(orc_r3d_t *s, int klev)
{
    const int n1 = s->n1[klev - 1], n2 = s->n2[klev - 1], n3 = s->n3[klev - 1];
    const int n1c = s->n1[klev], n2c = s->n2[klev];
    const double *pc = s->v[klev];
    double *pf = s->v[klev - 1];
    const size_t F1 = (size_t)n1 + 1, F2 = (size_t)n2 + 1;
    const size_t C1 = (size_t)n1c + 1, C2 = (size_t)n2c + 1;
#define PC(i, j, k) pc[(size_t)(i) + C1 * ((size_t)(j) + C2 * (size_t)(k))]
    for (int k = 0; k <= n3; ++k)
        for (int j = 0; j <= n2; ++j)
            for (int i = 0; i <= n1; ++i) {
                const int i1 = i / 2, j1 = j / 2, k1 = k / 2;
                const int ie = (i1 * 2 == i), je = (j1 * 2 == j), ke = (k1 * 2 == k);
                double p;
                if (ie) {
                    if (je) {
                        if (ke) p = PC(i1, j1, k1);
                        else p = (PC(i1, j1, k1) + PC(i1, j1, k1 + 1)) * 0.5;
                    } else {
                        if (ke) p = (PC(i1, j1, k1) + PC(i1, j1 + 1, k1)) * 0.5;
                        else
                            p = (PC(i1, j1, k1) + PC(i1, j1 + 1, k1) + PC(i1, j1, k1 + 1) + PC(i1, j1 + 1, k1 + 1)) * 0.25;
                    }
                } else {
                    if (je) {
                        if (ke) p = (PC(i1, j1, k1) + PC(i1 + 1, j1, k1)) * 0.5;
                        else
                            p = (PC(i1, j1, k1) + PC(i1 + 1, j1, k1) + PC(i1, j1, k1 + 1) + PC(i1 + 1, j1, k1 + 1)) * 0.25;
                    } else {
                        if (ke)
                            p = (PC(i1, j1, k1) + PC(i1 + 1, j1, k1) + PC(i1, j1 + 1, k1) + PC(i1 + 1, j1 + 1, k1)) * 0.25;
                        else
                            p = (PC(i1, j1, k1) + PC(i1 + 1, j1, k1) + PC(i1, j1 + 1, k1) + PC(i1 + 1, j1 + 1, k1) +
                                 PC(i1, j1, k1 + 1) + PC(i1 + 1, j1, k1 + 1) + PC(i1, j1 + 1, k1 + 1) +
                                 PC(i1 + 1, j1 + 1, k1 + 1)) *
                                0.125;
                    }
                }
                double *t = &pf[(size_t)i + F1 * ((size_t)j + F2 * (size_t)k)];
                *t = p + *t;
            }
#undef PC
    memset(s->v[klev], 0, level_size(s, klev) * sizeof(double));
}

/* poisson1/2/3, rot3dmg.f:1216-1540: initial guess 2 psi - psip, relax on
 * the fine level on the first sweep only, then V-cycles (descent: corser,
 * relax nrel1; ascent: finer, relax nrel2) with SOR 1.2 between sweeps, until
 * the fine residual after the last relax is below tolcon.  On convergence
 * psip takes the old psi, psi the interior solution and zero walls. */
int orc_r3d_poisson(orc_r3d_t *s, int which, int *sweeps)
{
    const int nr = s->nr, nz = s->nz, np = s->np, nlev = s->nlev;
    double *psi, *psip, *rhs;
    if (which == 1) {
        psi = s->wel;
        psip = s->welp;
        rhs = s->wrh;
    } else if (which == 2) {
        psi = s->vel;
        psip = s->velp;
        rhs = s->vrh;
    } else {
        psi = s->uel;
        psip = s->uelp;
        rhs = s->urh;
    }
    const int imax = which == 3 ? nr : nr + 1;   /* psi's i range (rot3dmg.f:1247, 1356, 1465) */
    const int jmax = which == 1 ? nz : nz + 1;
    const int n1 = s->n1[1], n2 = s->n2[1];
    const size_t L1 = (size_t)n1 + 1, L2 = (size_t)n2 + 1;
    double *v1 = s->v[1], *f1 = s->f[1];
#define V1(i, j, k) v1[(size_t)(i) + L1 * ((size_t)(j) + L2 * (size_t)(k))]
#define F1(i, j, k) f1[(size_t)(i) + L1 * ((size_t)(j) + L2 * (size_t)(k))]
    for (int k = 0; k <= np; ++k)
        for (int j = 0; j <= n2; ++j)
            for (int i = 0; i <= n1; ++i) {
                F1(i, j, k) = FX(rhs, i, j, k);
                V1(i, j, k) = 2.0 * FX(psi, i, j, k) - FX(psip, i, j, k);
            }
    int nconv = 0;
    for (int sweep = 1;; ++sweep) {
        if (sweep > s->maxsweeps) {
            if (sweeps) *sweeps = sweep - 1;
            s->last_sweeps = sweep - 1;
            return R3D_MAXSWEEPS;
        }
        if (sweep != 1 && !s->horizontal) {
            for (int k = 0; k <= np; ++k)
                for (int j = 0; j <= n2; ++j)
                    for (int i = 0; i <= n1; ++i) {
                        V1(i, j, k) = FX(psip, i, j, k) + s->sor * (V1(i, j, k) - FX(psip, i, j, k));
                        FX(psip, i, j, k) = V1(i, j, k);
                    }
        }
        if (sweep == 1 || nlev == 1) {
            orc_r3d_relax(s, which, s->nrel, 1, &nconv);
            if (!s->horizontal)
                for (int k = 0; k <= np; ++k)
                    for (int j = 0; j <= n2; ++j)
                        for (int i = 0; i <= n1; ++i) FX(psip, i, j, k) = V1(i, j, k);
        }
        if (nlev > 1) {
            for (int l = 1; l <= nlev - 1; ++l) {
                orc_r3d_corser(s, l);
                orc_r3d_relax(s, which, s->nrel, l + 1, &nconv);
            }
            for (int l = nlev; l >= 2; --l) {
                orc_r3d_finer(s, l);
                orc_r3d_relax(s, which, s->nrel, l - 1, &nconv);
            }
        }
        if (s->last_resmax != s->last_resmax) {
            if (sweeps) *sweeps = sweep;
            s->last_sweeps = sweep;
            return R3D_NAN;
        }
        if (nconv == 1) {
            for (int k = 0; k <= np; ++k)
                for (int j = 0; j <= jmax; ++j)
                    for (int i = 0; i <= imax; ++i) FX(psip, i, j, k) = FX(psi, i, j, k);
            const int ii1 = which == 3 ? nr - 1 : nr;
            const int jj1 = which == 1 ? nz - 1 : nz;
            for (int k = 0; k <= np; ++k)
                for (int j = 1; j <= jj1; ++j)
                    for (int i = 1; i <= ii1; ++i) FX(psi, i, j, k) = V1(i, j, k);
            for (int k = 0; k <= np; ++k) {
                for (int i = 0; i <= imax; ++i) {
                    FX(psi, i, 0, k) = 0.0;
                    FX(psi, i, jmax, k) = 0.0;
                }
                for (int j = 0; j <= jmax; ++j) {
                    FX(psi, 0, j, k) = 0.0;
                    FX(psi, imax, j, k) = 0.0;
                }
            }
            if (sweeps) *sweeps = sweep;
            s->last_sweeps = sweep;
            return R3D_OK;
        }
    }
#undef V1
#undef F1
}

int orc_r3d_step(orc_r3d_t *s, double *nu, int *sweeps)
{
    int sw[3] = {0, 0, 0};
    orc_r3d_avorticity(s);
    orc_r3d_bvorticity(s);
    orc_r3d_cvorticity(s);
    orc_r3d_temperature(s);
    double trans2 = 0.0;
    const double trans1 = s->horizontal ? orc_r3d_heat2(s, &trans2) : orc_r3d_heat(s);
    orc_r3d_rhsw(s);
    int st = orc_r3d_poisson(s, 1, &sw[0]);
    if (st == R3D_OK) {
        orc_r3d_rhsv(s);
        st = orc_r3d_poisson(s, 2, &sw[1]);
    }
    if (st == R3D_OK) {
        orc_r3d_rhsu(s);
        st = orc_r3d_poisson(s, 3, &sw[2]);
    }
    if (sweeps) {
        sweeps[0] = sw[0];
        sweeps[1] = sw[1];
        sweeps[2] = sw[2];
    }
    if (st != R3D_OK) return st;
    orc_r3d_update(s);
    if (s->horizontal) {
        /* httrans1, httrans2 of rot3dmghor.f:264-267 */
        const double L = log(s->r0 / s->rmax);
        if (nu) *nu = (double)s->nz / 6.0 * s->r0 * L * trans1 / (s->zmax * 2.0 * s->pi);
        s->nu2 = (double)s->nz / 6.0 * s->rmax * L * trans2 / (s->zmax * 2.0 * s->pi);
    } else if (nu) {
        *nu = -s->r0 * log(s->r0 / s->rmax) * trans1 / (s->zmax * 2.0 * s->pi);
    }
    return R3D_OK;
}
