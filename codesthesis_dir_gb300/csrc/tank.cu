// The horizontal-convection tank of
// monashubuntudir_velvor2dhorconvtankdir/velvor2dhorconvtank.f on the
// device: the periodic layer's scheme closed by side walls in x.  C and v
// live on the faces k = 0..np (walls k = 0, np), T and u on the cells
// k = 1..np with ghost columns k = 0 and np+1, so a tank instance's fields
// carry np+2 columns.  These kernels replace the layer's transport, heat,
// update and right-hand-side kernels; the multigrid is the layer's with its
// x-wall switch (MgEq::xwall).
//
// The differentially heated cavity benchmark of
// monashubuntudir_velvor2ddvdbenchmarkdir/velvor2ddvdbenchmark.f (PrbDev::dvd)
// runs the same kernels with its differences: the wall correction of the
// C-point dT/dr at i = 1 (:382-383), buoyancy -Ra thr (:437, :560), the T
// derivative's wall row 0.5333333333 T0 - 3.6 T1 + 2.9666666667 T2 + 0.1 T4
// (:601, :696), the T Robert filter on i = 1..nr (:763), heat over
// k = 2..np-1 (:780), side-wall vorticities -u(1)/dp and u(np)/dp
// (:819-820), T = 0 and 1 on the bottom and top rows with the insulated
// closure on the side ghosts (:822-830).
//
// Numerics: the reference's expressions in its order with -fmad=false; the
// REAL*4 literals 1./6. and 4./3. of the C-point dT/dr rows (:384-386) are
// the floats they round to.
#include "banded.cuh"
#include "gbcommon.cuh"
#include "prb_internal.cuh"

#define TF16 ((double)(1.0f / 6.0f))
#define TF43 ((double)(4.0f / 3.0f))

// Cvorticity/Cvorticity1 (:334-575): Cr -> A and thr at the C points -> An,
// tdma along r for each column k = 1..np-1 (one thread per column).
__global__ void k_tank_cvort_deriv_r(PrbDev d)
{
    const int k = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (k > d.np - 1 || *d.abort) return;
    const int ld = d.ld, nr = d.nr;
    const double dri = d.dri;
    const double *C = d.f[GB_F_C], *th = d.f[GB_F_th];
    auto rhsC = [&](int j) -> double {
        const int i = j + 1;
        if (i == 1)
            return 3.0 * (C[GIX(2, k, ld)] - C[GIX(0, k, ld)]) * dri -
                   (-1.5 * C[GIX(0, k, ld)] + 2.0 * C[GIX(1, k, ld)] - 0.5 * C[GIX(2, k, ld)]) * dri;
        if (i == nr - 1)
            return 3.0 * (C[GIX(nr, k, ld)] - C[GIX(nr - 2, k, ld)]) * dri -
                   (0.5 * C[GIX(nr - 2, k, ld)] - 2.0 * C[GIX(nr - 1, k, ld)] + 1.5 * C[GIX(nr, k, ld)]) * dri;
        return 3.0 * (C[GIX(i + 1, k, ld)] - C[GIX(i - 1, k, ld)]) * dri;
    };
    apply_tdma_rhs(d.fac_r1, nr - 1, d.f[GB_F_A] + GIX(1, k, ld), 1, rhsC);
    const int ka = k + 1;
    const bool dvd = d.dvd;
    auto rhsT = [&](int j) -> double {
        const int i = j + 1;
        if (i == 1 && dvd)
            return 3.0 * (th[GIX(2, k, ld)] + th[GIX(2, ka, ld)] - th[GIX(1, k, ld)] - th[GIX(1, ka, ld)]) * dri -
                   (-TF43 * (th[GIX(0, k, ld)] + th[GIX(0, ka, ld)]) + 1.5 * (th[GIX(1, k, ld)] + th[GIX(1, ka, ld)]) -
                    TF16 * (th[GIX(2, k, ld)] + th[GIX(2, ka, ld)])) * dri;
        if (i == 1)
            return 3.0 * (th[GIX(2, k, ld)] + th[GIX(2, ka, ld)] - th[GIX(1, k, ld)] - th[GIX(1, ka, ld)]) * dri;
        if (i == nr - 1)
            return 3.0 * (th[GIX(nr, k, ld)] + th[GIX(nr, ka, ld)] - th[GIX(nr - 1, k, ld)] - th[GIX(nr - 1, ka, ld)]) *
                       dri -
                   (TF16 * (th[GIX(nr - 1, k, ld)] + th[GIX(nr - 1, ka, ld)]) -
                    1.5 * (th[GIX(nr, k, ld)] + th[GIX(nr, ka, ld)]) +
                    TF43 * (th[GIX(nr + 1, k, ld)] + th[GIX(nr + 1, ka, ld)])) * dri;
        return 3.0 * (th[GIX(i + 1, k, ld)] + th[GIX(i + 1, ka, ld)] - th[GIX(i, k, ld)] - th[GIX(i, ka, ld)]) * dri;
    };
    apply_tdma_rhs(d.fac_r1, nr - 1, d.f[GB_F_An] + GIX(1, k, ld), 1, rhsT);
}

// Ch -> B and thh at the C points -> Bn: the plain Thomas algorithm along x
// over k = 1..np-1 for each row i = 1..nr-1.
__global__ void k_tank_cvort_deriv_x(PrbDev d)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i > d.nr - 1 || *d.abort) return;
    const int ld = d.ld, np = d.np;
    const double dpi = d.dpi;
    const double *C = d.f[GB_F_C], *th = d.f[GB_F_th];
    auto rhsC = [&](int j) -> double {
        const int k = j + 1;
        return 3.0 * (C[GIX(i, k + 1, ld)] - C[GIX(i, k - 1, ld)]) * dpi;
    };
    apply_tdma_rhs(d.fac_xw1, np - 1, d.f[GB_F_B] + GIX(i, 1, ld), ld, rhsC);
    auto rhsT = [&](int j) -> double {
        const int k = j + 1;
        return 3.0 * (th[GIX(i + 1, k + 1, ld)] + th[GIX(i, k + 1, ld)] - th[GIX(i + 1, k, ld)] - th[GIX(i, k, ld)]) *
               dpi;
    };
    apply_tdma_rhs(d.fac_xw1, np - 1, d.f[GB_F_Bn] + GIX(i, 1, ld), ld, rhsT);
}

// The vorticity update on i = 1..nr-1, k = 1..np-1 (:424-453, :553-575); the
// leapfrog RHS1 takes 0.5 Cp.
__global__ void k_tank_cvort_update(PrbDev d, int first)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nrow = d.nr - 1;
    if (t >= nrow * (d.np - 1) || *d.abort) return;
    const int i = t % nrow + 1, k = t / nrow + 1;
    const int ld = d.ld;
    const double dri = d.dri, dpi = d.dpi, Ptl = d.Pr, dt = d.dt, Ra = d.Ra;
    const double *C = d.f[GB_F_C], *Cp = d.f[GB_F_Cp];
    const double *uel = d.f[GB_F_uel], *vel = d.f[GB_F_vel];
    const int ip = i + 1, km = k - 1, ka = k + 1;
    const double ri = 1.0 / 1.0;
    const double u = (uel[GIX(i, ka, ld)] + uel[GIX(i, k, ld)]) * 0.5;
    const double v = (vel[GIX(i, k, ld)] + vel[GIX(ip, k, ld)]) * 0.5;
    const double Chha = (C[GIX(i, ka, ld)] + C[GIX(i, km, ld)]) * (dpi * dpi);
    const double Ch = d.f[GB_F_B][GIX(i, k, ld)];
    const double Crra = (C[GIX(i - 1, k, ld)] + C[GIX(i + 1, k, ld)]) * (dri * dri);
    const double cnr = -1.0 * (dri * dri);
    const double Cr = d.f[GB_F_A][GIX(i, k, ld)];
    const double thh = d.f[GB_F_Bn][GIX(i, k, ld)];
    const double cnh = (-1.0 * (dpi * dpi)) * (ri * ri);
    double RHS1, cf1;
    if (first) {
        RHS1 = Crra + Chha * (ri * ri) + C[GIX(i, k, ld)] / (Ptl * dt);
        cf1 = 1.0 / (Ptl * dt) - cnr - cnh;
    } else {
        RHS1 = Crra + Chha * (ri * ri) + 0.5 * Cp[GIX(i, k, ld)] / (Ptl * dt);
        cf1 = 0.5 / (Ptl * dt) - cnr - cnh;
    }
    const double ULT = (u * Cr + v * Ch * ri) / Ptl;
    const double RHS2 = d.dvd ? -Ra * d.f[GB_F_An][GIX(i, k, ld)] : -Ra * thh;
    const double cf2 = cnr + cnh;
    const double cn = (cf2 * Cp[GIX(i, k, ld)] - ULT - RHS2 + RHS1) / cf1;
    d.f[GB_F_Cn][GIX(i, k, ld)] = cn;
    if (!first) d.f[GB_F_Ap][GIX(i, k, ld)] = cn;
}

// Robert filter X += 0.02 (Xn - 2X + Xp) on rows i0..i1, columns k0..k1.
__global__ void k_tank_robert(PrbDev d, int fx, int fxn, int fxp, int i0, int i1, int k0, int k1)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int ni = i1 - i0 + 1;
    if (t >= ni * (k1 - k0 + 1) || *d.abort) return;
    const int i = i0 + t % ni, k = k0 + t / ni;
    const size_t c = GIX(i, k, d.ld);
    double *X = d.f[fx];
    X[c] = X[c] + 0.02 * (d.f[fxn][c] - 2.0 * X[c] + d.f[fxp][c]);
}

// temperature/temperature1 (:582-770): thr -> A along r over i = 1..nr for
// each column k = 1..np, with the insulated-wall row at i = 1.
__global__ void k_tank_temp_deriv_r(PrbDev d)
{
    const int k = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (k > d.np || *d.abort) return;
    const int ld = d.ld, nr = d.nr;
    const double dri = d.dri;
    const double *th = d.f[GB_F_th];
    const bool dvd = d.dvd;
    auto rhs = [&](int j) -> double {
        const int i = j + 1;
        if (i == 1 && dvd)
            return dri * (0.5333333333 * th[GIX(0, k, ld)] - 3.6 * th[GIX(1, k, ld)] + 2.9666666667 * th[GIX(2, k, ld)] +
                          0.1 * th[GIX(4, k, ld)]);
        if (i == 1)
            return dri * (-8.0 * th[GIX(0, k, ld)] + 6.0 * th[GIX(1, k, ld)] + 1.9 * th[GIX(2, k, ld)] +
                          0.1 * th[GIX(4, k, ld)]);
        if (i == nr)
            return dri * (-0.1 * th[GIX(nr - 3, k, ld)] - 2.966666667 * th[GIX(nr - 1, k, ld)] +
                          3.6 * th[GIX(nr, k, ld)] - 0.533333333 * th[GIX(nr + 1, k, ld)]);
        return 3.0 * (th[GIX(i + 1, k, ld)] - th[GIX(i - 1, k, ld)]) * dri;
    };
    apply_tdma_rhs(d.fac_rT, nr, d.f[GB_F_A] + GIX(1, k, ld), 1, rhs);
}

// thh -> B: the Thomas algorithm along x over the cells k = 1..np.
__global__ void k_tank_temp_deriv_x(PrbDev d)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i > d.nr || *d.abort) return;
    const int ld = d.ld, np = d.np;
    const double dpi = d.dpi;
    const double *th = d.f[GB_F_th];
    auto rhs = [&](int j) -> double {
        const int k = j + 1;
        return 3.0 * (th[GIX(i, k + 1, ld)] - th[GIX(i, k - 1, ld)]) * dpi;
    };
    apply_tdma_rhs(d.fac_xw2, np, d.f[GB_F_B] + GIX(i, 1, ld), ld, rhs);
}

// The temperature update on i = 1..nr, k = 1..np.
__global__ void k_tank_temp_update(PrbDev d, int first)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nr = d.nr;
    if (t >= nr * d.np || *d.abort) return;
    const int i = t % nr + 1, k = t / nr + 1;
    const int ld = d.ld;
    const double dri = d.dri, dpi = d.dpi, dt = d.dt;
    const double *th = d.f[GB_F_th], *thp = d.f[GB_F_thp];
    const double *uel = d.f[GB_F_uel], *vel = d.f[GB_F_vel];
    const int ip = i + 1, im = i - 1, km = k - 1, ka = k + 1;
    const double ri = 1.0 / 1.0;
    const double u = (uel[GIX(i, k, ld)] + uel[GIX(im, k, ld)]) * 0.5;
    const double v = (vel[GIX(i, k, ld)] + vel[GIX(i, km, ld)]) * 0.5;
    double thrra, cnr;
    if (i == 1) {
        thrra = (3.2 * th[GIX(i - 1, k, ld)] + 2.0 * th[GIX(i + 1, k, ld)] - 0.2 * th[GIX(i + 2, k, ld)]) * (dri * dri);
        cnr = -2.5 * (dri * dri);
    } else if (i == nr) {
        thrra = (3.2 * th[GIX(i + 1, k, ld)] + 2.0 * th[GIX(i - 1, k, ld)] - 0.2 * th[GIX(i - 2, k, ld)]) * (dri * dri);
        cnr = -2.5 * (dri * dri);
    } else {
        thrra = (th[GIX(i - 1, k, ld)] + th[GIX(ip, k, ld)]) * (dri * dri);
        cnr = -1.0 * (dri * dri);
    }
    const double thr = d.f[GB_F_A][GIX(i, k, ld)];
    const double thhha = (th[GIX(i, ka, ld)] + th[GIX(i, km, ld)]) * (dpi * dpi);
    const double thh = d.f[GB_F_B][GIX(i, k, ld)];
    const double cnp = -(1.0 * (dpi * dpi)) * (ri * ri);
    double RHS1, cf1;
    if (first) {
        RHS1 = thrra + thhha * (ri * ri) + th[GIX(i, k, ld)] / dt;
        cf1 = 1.0 / dt - cnr - cnp;
    } else {
        RHS1 = thrra + thhha * (ri * ri) + 0.5 * thp[GIX(i, k, ld)] / dt;
        cf1 = 0.5 / dt - cnr - cnp;
    }
    const double ULT = u * thr + v * thh * ri;
    const double cf2 = cnr + cnp;
    const double tn = (cf2 * thp[GIX(i, k, ld)] - ULT + RHS1) / cf1;
    d.f[GB_F_thn][GIX(i, k, ld)] = tn;
    if (!first) d.f[GB_F_Ap][GIX(i, k, ld)] = tn;
}

// update (:812-845), first half: the wall vorticities on k = 1..np-1, C = 0
// on the side walls, and the new T's boundary values.  Each boundary value
// is formed from interior values only (the bottom closure and the top-wall
// profile are re-derived where a ghost needs them), so the threads need no
// ordering among themselves; the interior T is not written here.
__global__ void k_tank_walls(PrbDev d)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nr = d.nr, np = d.np, ld = d.ld;
    const int ni = nr + 2;
    if (t >= ni * (np + 2) || *d.abort) return;
    const int i = t % ni, k = t / ni;
    const double dr = d.dr;
    const double *vel = d.f[GB_F_vel];
    double *Cn = d.f[GB_F_Cn], *thn = d.f[GB_F_thn];
    if (k >= 1 && k <= np - 1) {
        if (i == 0) Cn[GIX(0, k, ld)] = (3.0 * vel[GIX(1, k, ld)] - vel[GIX(2, k, ld)] / 3.0) / dr;
        else if (i == nr) Cn[GIX(nr, k, ld)] = (vel[GIX(nr - 1, k, ld)] / 3.0 - 3.0 * vel[GIX(nr, k, ld)]) / dr;
    }
    if (i <= nr && (k == 0 || k == np)) {
        const double *uel = d.f[GB_F_uel];
        if (d.dvd) Cn[GIX(i, k, ld)] = k == 0 ? -uel[GIX(i, 1, ld)] / d.dp : uel[GIX(i, np, ld)] / d.dp;
        else Cn[GIX(i, k, ld)] = 0.0;
    }
    if (d.dvd) {
        // T = 0 and 1 on the bottom and top rows (ghost columns included),
        // the insulated closure on the side ghosts of rows 1..nr
        if (i == 0) thn[GIX(0, k, ld)] = 0.0;
        else if (i == nr + 1) thn[GIX(nr + 1, k, ld)] = 1.0;
        else if (k == 0)
            thn[GIX(i, 0, ld)] = -30.0 / 92.0 * (-3.75 * thn[GIX(i, 1, ld)] + 5.0 / 6.0 * thn[GIX(i, 2, ld)] -
                                                 3.0 / 20.0 * thn[GIX(i, 3, ld)]);
        else if (k == np + 1)
            thn[GIX(i, np + 1, ld)] = -30.0 / 92.0 * (-3.75 * thn[GIX(i, np, ld)] + 5.0 / 6.0 * thn[GIX(i, np - 1, ld)] -
                                                      3.0 / 20.0 * thn[GIX(i, np - 2, ld)]);
        return;
    }
    // T on row ii of column kk after the wall rows are set (kk = 0..np)
    auto row = [&](int ii, int kk) -> double {
        if (ii == 0)
            return -30.0 / 92.0 * (-3.75 * thn[GIX(1, kk, ld)] + 5.0 / 6.0 * thn[GIX(2, kk, ld)] -
                                   3.0 / 20.0 * thn[GIX(3, kk, ld)]);
        if (ii == nr + 1) return (double)kk / (double)np * 1.0;
        return thn[GIX(ii, kk, ld)];
    };
    if (k == 0) thn[GIX(i, 0, ld)] = 2.0 / 1.5 * row(i, 1) - 1.0 / 3.0 * row(i, 2);
    else if (k == np + 1) thn[GIX(i, np + 1, ld)] = 2.0 / 1.5 * row(i, np) - 1.0 / 3.0 * row(i, np - 1);
    else if (i == 0 || i == nr + 1) thn[GIX(i, k, ld)] = row(i, k);
}

// update, second half: the time levels move (k = 0..np with the clamp of
// T to (0.01, 0.99); the ghost column np+1 of T without it).
__global__ void k_tank_rotate(PrbDev d)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nr = d.nr, np = d.np, ld = d.ld;
    const int ni = nr + 2;
    if (t >= ni * (np + 2) || *d.abort) return;
    const int i = t % ni, k = t / ni;
    const size_t c = GIX(i, k, ld);
    double *const *f = d.f;
    if (k == np + 1) {
        f[GB_F_thp][c] = f[GB_F_th][c];
        f[GB_F_th][c] = f[GB_F_thn][c];
        return;
    }
    f[GB_F_Cp][c] = f[GB_F_C][c];
    f[GB_F_C][c] = f[GB_F_Cn][c];
    f[GB_F_thp][c] = f[GB_F_th][c];
    double tn = f[GB_F_thn][c];
    unsigned long long clamped = 0;
    if (tn > 1.0) { tn = 0.99; clamped++; }
    if (tn < 0.0) { tn = 0.01; clamped++; }
    f[GB_F_thn][c] = tn;
    f[GB_F_th][c] = tn;
    if (clamped) atomicAdd(d.clamps, clamped);
}

// rhsv on i = 1..nr, k = 1..np-1 and rhsu on i = 1..nr-1, k = 1..np
// (:867-910), r = 1.
__global__ void k_tank_rhs(PrbDev d, int do_v, int do_u)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nr = d.nr, np = d.np, ld = d.ld;
    if (t >= nr * np || *d.abort) return;
    const int i = t % nr + 1, k = t / nr + 1;
    const double *Cn = d.f[GB_F_Cn];
    if (do_v && k <= np - 1) {
        const double Cr = (Cn[GIX(i, k, ld)] - Cn[GIX(i - 1, k, ld)]) / d.dr;
        double v;
        if (i == 1) v = Cn[GIX(1, k, ld)] / d.dr;
        else if (i == nr) v = -Cn[GIX(nr - 1, k, ld)] / d.dr;
        else v = Cr;
        d.f[GB_F_vrh][GIX(i, k, ld)] = v;
    }
    if (do_u && i <= nr - 1) {
        const double Ch = (Cn[GIX(i, k, ld)] - Cn[GIX(i, k - 1, ld)]) / d.dp;
        d.f[GB_F_urh][GIX(i, k, ld)] = -Ch / 1.0;
    }
}

static const int TANK_TPB = 256;

int tank_launch_cvorticity(gb_prb *h, int first, cudaStream_t s)
{
    PrbDev &d = h->dev;
    k_tank_cvort_deriv_r<<<gb_ceil_div(d.np - 1, 64), 64, 0, s>>>(d);
    k_tank_cvort_deriv_x<<<gb_ceil_div(d.nr - 1, 64), 64, 0, s>>>(d);
    k_tank_cvort_update<<<gb_ceil_div((size_t)(d.nr - 1) * (d.np - 1), TANK_TPB), TANK_TPB, 0, s>>>(d, first);
    if (!first)
        k_tank_robert<<<gb_ceil_div((size_t)(d.nr - 1) * (d.np - 1), TANK_TPB), TANK_TPB, 0, s>>>(
            d, GB_F_C, GB_F_Cn, GB_F_Cp, 1, d.nr - 1, 1, d.np - 1);
    h->launches += first ? 3 : 4;
    return GB_OK;
}

int tank_launch_temperature(gb_prb *h, int first, cudaStream_t s)
{
    PrbDev &d = h->dev;
    k_tank_temp_deriv_r<<<gb_ceil_div(d.np, 64), 64, 0, s>>>(d);
    k_tank_temp_deriv_x<<<gb_ceil_div(d.nr, 64), 64, 0, s>>>(d);
    k_tank_temp_update<<<gb_ceil_div((size_t)d.nr * d.np, TANK_TPB), TANK_TPB, 0, s>>>(d, first);
    if (!first)
        k_tank_robert<<<gb_ceil_div((size_t)(d.nr + 1) * d.np, TANK_TPB), TANK_TPB, 0, s>>>(
            d, GB_F_th, GB_F_thn, GB_F_thp, d.dvd ? 1 : 0, d.nr, 1, d.np);
    h->launches += first ? 3 : 4;
    return GB_OK;
}

int tank_launch_rhs(gb_prb *h, int do_v, int do_u, cudaStream_t s)
{
    PrbDev &d = h->dev;
    k_tank_rhs<<<gb_ceil_div((size_t)d.nr * d.np, TANK_TPB), TANK_TPB, 0, s>>>(d, do_v, do_u);
    h->launches += 1;
    return GB_OK;
}

int tank_launch_update(gb_prb *h, cudaStream_t s)
{
    PrbDev &d = h->dev;
    const size_t n = (size_t)(d.nr + 2) * (d.np + 2);
    k_tank_walls<<<gb_ceil_div(n, TANK_TPB), TANK_TPB, 0, s>>>(d);
    k_tank_rotate<<<gb_ceil_div(n, TANK_TPB), TANK_TPB, 0, s>>>(d);
    h->launches += 2;
    return GB_OK;
}
