// Velocity-component multigrid solves of the 2D periodic Rayleigh-Benard
// driver (poisson2/poisson3, relax2/relax3, corser, finer of
// velvor2dperiodicrbconv.f:1724-2859) as one persistent thread block per
// equation: the whole outer sweep loop, every level and every convergence
// test run inside one launch, so a solve costs one kernel launch however many
// sweeps it takes.  The v and u solves of a step are the two blocks of one
// launch (the reference runs them as two OpenMP sections, PRB:370-380).
//
// Two smoother orderings:
//   LEX   - lines k = 1..n3 in order, the reference schedule; one thread
//           marches the lines (the ordering is sequential by definition).
//   ZEBRA - odd lines, then even lines; every line of a colour is solved by
//           its own thread.
// Either way each line is solved with the reference's banded elimination in
// the reference's operation order (-fmad=false), so LEX results are
// bit-identical to the reference algorithm and ZEBRA results to the same
// algorithm under zebra ordering.
//
// The rotating-annulus variant (E.polar; relax2/relax3/corser of
// velvor2dnewsch3.4.f:2071-2716) uses the same kernel: its line matrices
// depend on the radius of row i but not on the line k, so they are still
// factored once per level; the line right-hand sides and residuals gain the
// polar terms, every level visit runs three relaxations (:2134, :2410), and
// the coarse right-hand side of seam line n3c keeps the fine residual stored
// there because that corser does not clear it (:2696-2704).
//
// Storage differs from the reference only in scratch that no output depends
// on: the right-hand sides are read from the packed per-level arrays instead
// of being unpacked into rf, and the prolongation reads the coarse solution
// straight from its packed slot (the reference stages both through psic/rf/
// tempa).  Every value the solution depends on is formed by the same
// arithmetic on the same operands.
#include <string.h>

#include "banded.cuh"
#include "gbcommon.cuh"
#include "prb_internal.cuh"

#define MG_THREADS 512

__device__ __forceinline__ double blk_max(double v, double *s_red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = (lane < nw) ? s_red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
        if (lane == 0) s_red[32] = v;
    }
    __syncthreads();
    const double r = s_red[32];
    __syncthreads();
    return r;
}

// One line k of relax2 (pentadiagonal, rows i = 1..n1, PRB:2113-2191) or
// relax3 (tridiagonal, rows i = 1..n1-1, PRB:2414-2460).
__device__ __forceinline__ void mg_line(const MgEq &E, const MgLevel &L, int k)
{
    const int ld = E.ld, n1 = L.n1, n3 = L.n3;
    double *psif = E.psif;
    const double *f = L.f;
    const double hhpi = L.hhpi;
    const int ka = (k == n3) ? 1 : k + 1, km = k - 1;
    const bool polar = E.polar;
    const double *rvq = L.rvq;
    auto rhs = [&](int j) -> double {
        const int i = j + 1;
        double t = -(psif[GIX(i, ka, ld)] + psif[GIX(i, km, ld)]) * hhpi;
        if (polar) t = t * rvq[i];
        return t + f[(size_t)k * (n1 + 1) + i];
    };
    const int nrow = (E.which == 2) ? n1 : n1 - 1;
    if (E.which == 2) apply_pdma_rhs(L.fac, n1, psif + GIX(1, k, ld), 1, rhs);
    else apply_tdma_rhs(L.fac, n1 - 1, psif + GIX(1, k, ld), 1, rhs);
    if (k == n3)
        for (int i = 1; i <= nrow; ++i) psif[GIX(i, 0, ld)] = psif[GIX(i, k, ld)];
}

// relax2 / relax3: line sweeps (one with nrel = 1; three in the annulus),
// then the residual into rc, its max norm, and psif packed into v.  Only
// the last sweep's residual is formed: the reference recomputes rc and
// resmax after every sweep and keeps the last.  Returns the level's
// residual max norm (NaNs ignored as in the reference's comparison);
// *nan_out (uniform over the block) is set when a NaN residual appears.
__device__ double mg_relax(const MgEq &E, int klev, double *s_red, int *nan_out)
{
    const MgLevel &L = E.lev[klev];
    const int ld = E.ld, n1 = L.n1, n3 = L.n3;
    const double hhri = L.hhri, hhpi = L.hhpi, hri = L.hri;
    const double *rvi = L.rvi, *rvq = L.rvq;
    double *psif = E.psif, *rc = E.rc;
    const double *f = L.f;
    const int nrel = E.polar ? 3 : 1;
    for (int irel = 0; irel < nrel; ++irel) {
        if (E.mode == GB_SMOOTHER_LEX) {
            if (threadIdx.x == 0)
                for (int k = 1; k <= n3; ++k) mg_line(E, L, k);
            __syncthreads();
        } else {
            for (int parity = 1; parity >= 0; --parity) {
                for (int t = threadIdx.x; t < n3 / 2; t += blockDim.x) mg_line(E, L, 2 * t + 2 - parity);
                __syncthreads();
            }
        }
    }
    // residual, PRB:2306-2357 (v) and PRB:2553-2587 (u)
    double m = 0.0;
    int nan = 0;
    const int nrow = (E.which == 2) ? n1 : n1 - 1;
    const int tot = nrow * n3;
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int k = idx / nrow + 1, i = idx - (k - 1) * nrow + 1;
        const int ka = (k == n3) ? 1 : k + 1, km = k - 1;
        double temp;
        if (E.polar && E.which == 2) {
            // velvor2dnewsch3.4.f:2300-2346
            temp = (psif[GIX(i, ka, ld)] - 2.0 * psif[GIX(i, k, ld)] + psif[GIX(i, km, ld)]) * hhpi * rvq[i] +
                   psif[GIX(i, k, ld)] * rvq[i];
            if (i == 1)
                temp = temp + (-2.0 * psif[GIX(i, k, ld)] + 5.0 / 3.0 * psif[GIX(i + 1, k, ld)] -
                               0.2 * psif[GIX(i + 2, k, ld)]) * hhri +
                       4.0 / 3.0 * psif[GIX(i + 1, k, ld)] * hri * rvi[i];
            else if (i == n1)
                temp = temp + (-2.0 * psif[GIX(i, k, ld)] + 5.0 / 3.0 * psif[GIX(i - 1, k, ld)] -
                               0.2 * psif[GIX(i - 2, k, ld)]) * hhri -
                       4.0 / 3.0 * psif[GIX(i - 1, k, ld)] * hri * rvi[i];
            else
                temp = temp + (psif[GIX(i - 1, k, ld)] - 2.0 * psif[GIX(i, k, ld)] + psif[GIX(i + 1, k, ld)]) * hhri +
                       1.5 * (psif[GIX(i + 1, k, ld)] - psif[GIX(i - 1, k, ld)]) * hri * rvi[i];
        } else if (E.polar) {
            // velvor2dnewsch3.4.f:2546-2579
            temp = (psif[GIX(i + 1, k, ld)] + psif[GIX(i - 1, k, ld)]) * hhri +
                   1.5 * (psif[GIX(i + 1, k, ld)] - psif[GIX(i - 1, k, ld)]) * hri * rvi[i] +
                   psif[GIX(i, k, ld)] * rvq[i] +
                   (psif[GIX(i, ka, ld)] + psif[GIX(i, km, ld)]) * hhpi * rvq[i] -
                   psif[GIX(i, k, ld)] * (2.0 * hhri + 2.0 * hhpi * rvq[i]);
        } else if (E.which == 2) {
            temp = (psif[GIX(i, ka, ld)] - 2.0 * psif[GIX(i, k, ld)] + psif[GIX(i, km, ld)]) * hhpi;
            if (i == 1)
                temp = temp + (-2.0 * psif[GIX(i, k, ld)] + 5.0 / 3.0 * psif[GIX(i + 1, k, ld)] -
                               0.2 * psif[GIX(i + 2, k, ld)]) * hhri;
            else if (i == n1)
                temp = temp + (-2.0 * psif[GIX(i, k, ld)] + 5.0 / 3.0 * psif[GIX(i - 1, k, ld)] -
                               0.2 * psif[GIX(i - 2, k, ld)]) * hhri;
            else
                temp = temp + (psif[GIX(i - 1, k, ld)] - 2.0 * psif[GIX(i, k, ld)] + psif[GIX(i + 1, k, ld)]) * hhri;
        } else {
            temp = (psif[GIX(i + 1, k, ld)] + psif[GIX(i - 1, k, ld)]) * hhri +
                   (psif[GIX(i, ka, ld)] + psif[GIX(i, km, ld)]) * hhpi -
                   psif[GIX(i, k, ld)] * (2.0 * hhri + 2.0 * hhpi);
        }
        temp = f[(size_t)k * (n1 + 1) + i] - temp;
        rc[GIX(i, k, ld)] = temp;
        temp = fabs(temp);
        if (temp != temp) nan = 1;
        if (temp > m) m = temp;
    }
    *nan_out = __syncthreads_or(nan);
    m = blk_max(m, s_red);
    // trans1(psif -> v)
    const int tp = (n1 + 1) * (n3 + 1);
    for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
        const int k = idx / (n1 + 1), i = idx - k * (n1 + 1);
        L.v[idx] = psif[GIX(i, k, ld)];
    }
    __syncthreads();
    return m;
}

// corser (PRB:2603-2718): full weighting of rc onto the packed coarse
// right-hand side; psif zeroed over the coarse region.
__device__ void mg_corser(const MgEq &E, int klev)
{
    const int ld = E.ld;
    const int n1c = E.lev[klev + 1].n1, n3c = E.lev[klev + 1].n3;
    const double *rf = E.rc;
    double *psif = E.psif, *fc = E.lev[klev + 1].f;
    const int tot = (n1c + 1) * (n3c + 1);
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int k = idx / (n1c + 1), i = idx - k * (n1c + 1);
        psif[GIX(i, k, ld)] = 0.0;
        double t = 0.0;
        if (i >= 1 && i <= n1c - 1 && k >= 1 && k <= n3c - 1) {
            const int ii = i + i, kk = k + k;
            const int iip = ii + 1, iim = ii - 1, kkp = kk + 1, kkm = kk - 1;
            t = rf[GIX(ii, kk, ld)];
            t = t + t;
            t = t + rf[GIX(iip, kk, ld)];
            t = t + rf[GIX(iim, kk, ld)];
            t = t + rf[GIX(ii, kk, ld)];
            t = t + rf[GIX(ii, kk, ld)];
            t = t + rf[GIX(ii, kkp, ld)];
            t = t + rf[GIX(ii, kkm, ld)];
            t = t + t;
            t = t + rf[GIX(iip, kk, ld)];
            t = t + rf[GIX(iip, kk, ld)];
            t = t + rf[GIX(iim, kk, ld)];
            t = t + rf[GIX(iim, kk, ld)];
            t = t + rf[GIX(iip, kkp, ld)];
            t = t + rf[GIX(iip, kkm, ld)];
            t = t + rf[GIX(iim, kkp, ld)];
            t = t + rf[GIX(iim, kkm, ld)];
            t = t + rf[GIX(ii, kkp, ld)];
            t = t + rf[GIX(ii, kkm, ld)];
            t = t + rf[GIX(ii, kkp, ld)];
            t = t + rf[GIX(ii, kkm, ld)];
            t = t + t;
            t = t + rf[GIX(iip, kkp, ld)];
            t = t + rf[GIX(iip, kkm, ld)];
            t = t + rf[GIX(iip, kkp, ld)];
            t = t + rf[GIX(iip, kkm, ld)];
            t = t + rf[GIX(iim, kkp, ld)];
            t = t + rf[GIX(iim, kkm, ld)];
            t = t + rf[GIX(iim, kkp, ld)];
            t = t + rf[GIX(iim, kkm, ld)];
            t = t * 0.015625;
        } else if (E.polar && i >= 1 && i <= n1c - 1) {
            t = rf[GIX(i, k, ld)];   // seam lines k = 0, n3c keep rc (k = 0 is never written)
        }
        fc[idx] = t;
    }
    __syncthreads();
}

// finer (PRB:2721-2803): bilinear prolongation of the coarse correction plus
// the saved fine solution.
__device__ void mg_finer(const MgEq &E, int klev)
{
    const int ld = E.ld;
    const int n1c = E.lev[klev].n1;
    const int n1f = E.lev[klev - 1].n1, n3f = E.lev[klev - 1].n3;
    const double *vc = E.lev[klev].v, *vf = E.lev[klev - 1].v;
    double *psif = E.psif;
    const int tot = (n1f + 1) * (n3f + 1);
#define PC(ii, kk) vc[(size_t)(kk) * (n1c + 1) + (ii)]
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int k = idx / (n1f + 1), i = idx - k * (n1f + 1);
        const int i1 = i / 2, k1 = k / 2;
        double p;
        if (i1 * 2 == i) {
            if (k1 * 2 == k) p = PC(i1, k1);
            else p = (PC(i1, k1) + PC(i1, k1 + 1)) * 0.5;
        } else {
            if (k1 * 2 == k) p = (PC(i1, k1) + PC(i1 + 1, k1)) * 0.5;
            else p = (PC(i1, k1) + PC(i1 + 1, k1) + PC(i1, k1 + 1) + PC(i1 + 1, k1 + 1)) * 0.25;
        }
        psif[GIX(i, k, ld)] = p + vf[idx];
    }
#undef PC
    __syncthreads();
}

// poisson2 / poisson3 (PRB:1796-1927 / PRB:1930-2059).
__global__ void __launch_bounds__(MG_THREADS) k_mg_solve(const MgEq *eqs, int first_eq)
{
    __shared__ double s_red[33];
    int nan1 = 0, nan_c = 0;
    const MgEq &E = eqs[first_eq + blockIdx.x];
    const int ld = E.ld, np = E.np, nlev = E.nlev;
    const int imax = (E.which == 2) ? E.nr + 1 : E.nr;
    const int n1 = E.lev[1].n1;
    double *psif = E.psif, *psi = E.psi, *psip = E.psip;
    const int rows = imax + 1, tot = rows * (np + 1);
    // initial guess 2 psi - psip; level-1 right-hand side and solution packed
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int k = idx / rows, i = idx - k * rows;
        const size_t c = GIX(i, k, ld);
        const double pf = 2.0 * psi[c] - psip[c];
        psif[c] = pf;
        if (i <= n1) {
            E.lev[1].f[(size_t)k * (n1 + 1) + i] = E.rhs[c];
            E.lev[1].v[(size_t)k * (n1 + 1) + i] = pf;
        }
    }
    __syncthreads();
    int status = GB_MAXSWEEPS, sweeps = 0;
    double res1 = 0.0;
    for (int sweep = 1; sweep <= E.maxsweeps; ++sweep) {
        sweeps = sweep;
        if (sweep != 1) {
            for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
                const int k = idx / rows, i = idx - k * rows;
                const size_t c = GIX(i, k, ld);
                const double pf = psip[c] + E.sor * (psif[c] - psip[c]);
                psif[c] = pf;
                psip[c] = pf;
                if (i <= n1) E.lev[1].v[(size_t)k * (n1 + 1) + i] = pf;
            }
            __syncthreads();
        }
        if (sweep == 1 || nlev == 1) {
            res1 = mg_relax(E, 1, s_red, &nan1);
            for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
                const int k = idx / rows, i = idx - k * rows;
                psip[GIX(i, k, ld)] = psif[GIX(i, k, ld)];
            }
            __syncthreads();
        }
        if (nlev > 1) {
            for (int l = 1; l <= nlev - 1; ++l) {
                mg_corser(E, l);
                mg_relax(E, l + 1, s_red, &nan_c);
            }
            for (int ifmg = 0; ifmg <= nlev - 2; ++ifmg) {
                for (int l = nlev; l >= nlev - ifmg; --l) {
                    mg_finer(E, l);
                    int nn = 0;
                    double r = mg_relax(E, l - 1, s_red, &nn);
                    if (l - 1 == 1) { res1 = r; nan1 = nn; }
                }
                for (int l = nlev - ifmg - 1; l <= nlev - 1; ++l) {
                    mg_corser(E, l);
                    mg_relax(E, l + 1, s_red, &nan_c);
                }
            }
            for (int l = nlev; l >= 2; --l) {
                mg_finer(E, l);
                int nn = 0;
                double r = mg_relax(E, l - 1, s_red, &nn);
                if (l - 1 == 1) { res1 = r; nan1 = nn; }
            }
        }
        // The last relax of a sweep is on level 1; its NaN flag decides.
        if (nan1) {
            status = GB_NAN;
            break;
        }
        if (res1 < E.tolcon) {
            for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
                const int k = idx / rows, i = idx - k * rows;
                const size_t c = GIX(i, k, ld);
                psip[c] = psi[c];
                if (i == 0 || i == imax) psi[c] = 0.0;
                else psi[c] = psif[c];
            }
            status = GB_OK;
            break;
        }
    }
    if (threadIdx.x == 0) {
        E.status[0] = status;
        E.status[1] = sweeps;
        *E.resmax = res1;
        if (status == GB_NAN || (status == GB_MAXSWEEPS && E.stop_on_max)) *E.abort = 1;
    }
}

// Factored line matrices of every level (one thread), the coefficients of
// relax2 (PRB:2128-2156) and relax3 (PRB:2421-2436); for the annulus those
// of velvor2dnewsch3.4.f:2104-2131 and :2401-2408 with the per-row 1/r and
// 1/r^2 they use.
__global__ void k_mg_factors(MgEq eq, double *work)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int l = 1; l <= eq.nlev; ++l) {
        const MgLevel &L = eq.lev[l];
        const int n1 = L.n1;
        const double hhri = L.hhri, hhpi = L.hhpi, hri = L.hri;
        double *a = work, *b = a + n1 + 2, *c = b + n1 + 2, *d = c + n1 + 2, *e = d + n1 + 2, *w = e + n1 + 2;
        double *fac = (double *)L.fac;
        double *rvi = L.rvi, *rvq = L.rvq;
        for (int i = 0; i <= n1 + 1; ++i) { rvi[i] = 1.0; rvq[i] = 1.0; }
        if (eq.which == 2) {
            for (int i = 1; i <= n1; ++i) {
                const int j = i - 1;
                if (eq.polar) {
                    const double rval = eq.r0 + ((double)i - 0.5) * L.hr;
                    rvi[i] = 1.0 / rval;
                    rvq[i] = rvi[i] * rvi[i];
                    if (i == 1) {
                        a[j] = 0.0; b[j] = 0.0;
                        c[j] = -2.0 * hhri - 2.0 * hhpi * rvq[i] + rvq[i];
                        d[j] = 5.0 / 3.0 * hhri + 4.0 / 3.0 * hri * rvi[i];
                        e[j] = -0.2 * hhri;
                    } else if (i == n1) {
                        a[j] = -0.2 * hhri;
                        b[j] = 5.0 / 3.0 * hhri - 4.0 / 3.0 * hri * rvi[i];
                        c[j] = -2.0 * hhri - 2.0 * hhpi * rvq[i] + rvq[i];
                        d[j] = 0.0; e[j] = 0.0;
                    } else {
                        a[j] = 0.0;
                        b[j] = hhri - 1.5 * hri * rvi[i];
                        c[j] = -(2.0 * hhri + 2.0 * hhpi * rvq[i]) + rvq[i];
                        d[j] = hhri + 1.5 * hri * rvi[i];
                        e[j] = 0.0;
                    }
                } else if (i == 1) {
                    a[j] = 0.0; b[j] = 0.0;
                    c[j] = -2.0 * hhri - 2.0 * hhpi;
                    d[j] = 5.0 / 3.0 * hhri;
                    e[j] = -0.2 * hhri;
                } else if (i == n1) {
                    a[j] = -0.2 * hhri;
                    b[j] = 5.0 / 3.0 * hhri;
                    c[j] = -2.0 * hhri - 2.0 * hhpi;
                    d[j] = 0.0; e[j] = 0.0;
                } else {
                    a[j] = 0.0; b[j] = hhri;
                    c[j] = -(2.0 * hhri + 2.0 * hhpi);
                    d[j] = hhri; e[j] = 0.0;
                }
            }
            factor_pdma(a, b, c, d, e, n1, fac, w);
        } else {
            for (int j = 0; j < n1 - 1; ++j) {
                const int i = j + 1;
                if (eq.polar) {
                    const double rval = (double)i * L.hr + eq.r0;
                    rvi[i] = 1.0 / rval;
                    rvq[i] = rvi[i] * rvi[i];
                    a[j] = hhri - 1.5 * hri * rvi[i];
                    b[j] = -(2.0 * hhri - rvq[i] + 2.0 * hhpi * rvq[i]);
                    c[j] = hhri + 1.5 * hri * rvi[i];
                } else {
                    a[j] = hhri;
                    b[j] = -(2.0 * hhri + 2.0 * hhpi);
                    c[j] = hhri;
                }
            }
            factor_tdma(a, b, c, n1 - 1, fac);
        }
    }
}

int prb_mg_create(gb_prb *h)
{
    const gb_prb_params &p = h->p;
    const int nr = p.nr, np = p.np, nlev = h->nlev;
    const int ld = h->dev.ld;
    const double dr = h->dev.dr, dp = h->dev.dp;
    if (np % (1 << nlev) != 0) {
        gb_set_error("np=%d must be divisible by 2^nlev=%d so that every multigrid level has an even number of lines", np, 1 << nlev);
        return GB_ERR_INVALID;
    }
    // pool: per equation psif, rc (full) + per level v, f + factors; plus work
    size_t per_eq = 2 * (size_t)ld * (np + 1);
    for (int l = 1; l <= nlev; ++l) {
        const int n1 = nr * 2 / (1 << l), n3 = np * 2 / (1 << l);
        per_eq += 2 * (size_t)(n1 + 1) * (n3 + 1) + 5 * (size_t)(n1 + 2) + 1 + 2 * (size_t)(n1 + 2);
    }
    const size_t work = 8 * (size_t)(nr + 2);
    cudaError_t e = cudaMalloc(&h->mg_pool, sizeof(double) * (2 * per_eq + work));
    if (e != cudaSuccess) { gb_set_error("multigrid pool: %s", cudaGetErrorString(e)); return GB_ERR_ALLOC; }
    cudaMemset(h->mg_pool, 0, sizeof(double) * (2 * per_eq + work));
    double *wk = h->mg_pool + 2 * per_eq;
    for (int q = 0; q < 2; ++q) {
        MgEq &E = h->eq_host[q];
        memset(&E, 0, sizeof(E));
        E.which = q == 0 ? 2 : 3;
        E.nr = nr; E.np = np; E.ld = ld; E.nlev = nlev;
        E.mode = p.smoother; E.maxsweeps = p.maxsweeps; E.tolcon = p.tolcon; E.sor = p.sor;
        E.polar = p.variant == GB_PRB_ANNULUS;
        E.stop_on_max = !E.polar;
        E.r0 = p.r0;
        double *base = h->mg_pool + q * per_eq;
        E.psif = base; base += (size_t)ld * (np + 1);
        E.rc = base; base += (size_t)ld * (np + 1);
        E.psic = E.rf = E.tempa = nullptr;
        for (int l = 1; l <= nlev; ++l) {
            MgLevel &L = E.lev[l];
            L.n1 = nr * 2 / (1 << l);
            L.n3 = np * 2 / (1 << l);
            const double hr = dr * (double)(1 << l) * 0.5;
            const double hp = dp * (double)(1 << l) * 0.5;
            L.hr = hr;
            L.hhri = 1.0 / (hr * hr);
            L.hhpi = 1.0 / (hp * hp);
            L.hri = 1.0 / hr;
            const size_t sz = (size_t)(L.n1 + 1) * (L.n3 + 1);
            L.v = base; base += sz;
            L.f = base; base += sz;
            L.fac = base; base += 5 * (size_t)(L.n1 + 2) + 1;
            L.rvi = base; base += (size_t)(L.n1 + 2);
            L.rvq = base; base += (size_t)(L.n1 + 2);
        }
        E.psi = h->dev.f[q == 0 ? GB_F_vel : GB_F_uel];
        E.psip = h->dev.f[q == 0 ? GB_F_velp : GB_F_uelp];
        E.rhs = h->dev.f[q == 0 ? GB_F_vrh : GB_F_urh];
        E.status = h->dev.mg_status + 2 * q;
        E.resmax = h->dev.mg_resmax + q;
        E.abort = h->dev.abort;
        k_mg_factors<<<1, 1>>>(E, wk);
    }
    e = cudaMalloc(&h->eq_dev, sizeof(MgEq) * 2);
    if (e != cudaSuccess) { gb_set_error("multigrid descriptors: %s", cudaGetErrorString(e)); return GB_ERR_ALLOC; }
    cudaMemcpy(h->eq_dev, h->eq_host, sizeof(MgEq) * 2, cudaMemcpyHostToDevice);
    return GB_OK;
}

void prb_mg_destroy(gb_prb *h)
{
    cudaFree(h->mg_pool);
    cudaFree(h->eq_dev);
    h->mg_pool = nullptr;
    h->eq_dev = nullptr;
}

// Refreshes the solve parameters that a caller may change between calls
// (tolerance, sweep limit, smoother, SOR factor) and launches the solves.
int prb_launch_mg(gb_prb *h, int do_v, int do_u, cudaStream_t s)
{
    bool changed = false;
    for (int q = 0; q < 2; ++q) {
        MgEq &E = h->eq_host[q];
        if (E.mode != h->p.smoother || E.maxsweeps != h->p.maxsweeps || E.tolcon != h->p.tolcon || E.sor != h->p.sor) {
            E.mode = h->p.smoother; E.maxsweeps = h->p.maxsweeps; E.tolcon = h->p.tolcon; E.sor = h->p.sor;
            changed = true;
        }
    }
    if (changed) cudaMemcpyAsync(h->eq_dev, h->eq_host, sizeof(MgEq) * 2, cudaMemcpyHostToDevice, s);
    const int first = do_v ? 0 : 1;
    const int n = (do_v ? 1 : 0) + (do_u ? 1 : 0);
    if (n == 0) return GB_OK;
    k_mg_solve<<<n, MG_THREADS, 0, s>>>(h->eq_dev, first);
    h->launches += 1;
    return GB_OK;
}
