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
// The rotating-annulus variant (relax2/relax3/corser of
// velvor2dnewsch3.4.f:2071-2716) uses the same kernel: its line matrices
// depend on the radius of row i but not on the line k, so they are still
// factored once per level; the line right-hand sides and residuals gain the
// polar terms (E.polar), every level visit runs three relaxations (E.nrelax,
// :2134, :2410), and the coarse right-hand side of seam line n3c keeps the
// fine residual stored there because that corser does not clear it
// (E.seam_keep, :2696-2704).  The Taylor-Couette driver
// (velvor2dtaycouheat.f) has the polar operator with PRB's single
// relaxation and seam reset.
//
// Storage differs from the reference only in scratch that no output depends
// on: the right-hand sides are read from the packed per-level arrays instead
// of being unpacked into rf, and the prolongation reads the coarse solution
// straight from its packed slot (the reference stages both through psic/rf/
// tempa).  Every value the solution depends on is formed by the same
// arithmetic on the same operands.
#include <stdint.h>
#include <string.h>

#include <cooperative_groups.h>

#include "banded.cuh"
#include "gbcommon.cuh"
#include "prb_internal.cuh"

namespace cg = cooperative_groups;

#define MG_THREADS 512
#define MG_CLUSTER 8   // CTAs sharing one FP64 zebra solve (gb_prb_step's single-instance path)

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

// The threads that share one equation's solve: one CTA (MgBlock), or the
// CTAs of a thread-block cluster (MgCluster), which meet at the hardware
// cluster barrier (arrive with release, wait with acquire at cluster scope:
// what any CTA of the cluster wrote to global memory before it is seen by
// every CTA after it) and reduce through distributed shared memory.  A
// cluster spreads a solve's lines over several SMs' FP64 units; the work of
// each line is unchanged, so both give the same bits.
struct MgBlock {
    static constexpr int C = 1;
    __device__ static int tid() { return threadIdx.x; }
    __device__ static int nthr() { return blockDim.x; }
    __device__ static void sync() { __syncthreads(); }
};
template <int CS> struct MgCluster {
    static constexpr int C = CS;
    __device__ static int tid() { return (int)cg::this_cluster().block_rank() * blockDim.x + threadIdx.x; }
    __device__ static int nthr() { return CS * blockDim.x; }
    __device__ static void sync() { cg::this_cluster().sync(); }
};

// Maximum (NaNs ignored, as blk_max) and logical or over the group.
template <class G> __device__ __forceinline__ double grp_max(double v, double *s_red)
{
    v = blk_max(v, s_red);
    if constexpr (G::C > 1) {
        __shared__ double s_pub;
        if (threadIdx.x == 0) s_pub = v;
        G::sync();
        cg::cluster_group cl = cg::this_cluster();
        double m = 0.0;
        for (int r = 0; r < G::C; ++r) m = fmax(m, *cl.map_shared_rank(&s_pub, r));
        G::sync();   // every CTA has read every slot before the next reduction writes it
        v = m;
    }
    return v;
}
template <class G> __device__ __forceinline__ int grp_or(int x)
{
    x = __syncthreads_or(x);
    if constexpr (G::C > 1) {
        __shared__ int s_or;
        if (threadIdx.x == 0) s_or = x;
        G::sync();
        cg::cluster_group cl = cg::this_cluster();
        int o = 0;
        for (int r = 0; r < G::C; ++r) o |= *cl.map_shared_rank(&s_or, r);
        G::sync();
        x = o;
    }
    return x;
}

// The level operator applied at (i, k) (the part of relax2/relax3's
// residual before it is subtracted from f): PRB:2306-2357 (v),
// PRB:2553-2587 (u), and the annulus forms of velvor2dnewsch3.4.f:2300-2346
// and :2546-2579.  Instantiated for double (bit-identical to the reference)
// and for float (the mixed-precision correction cycle).
template <class T>
__device__ __forceinline__ T mg_apply_op(const T *psif, int ld, int i, int k, int ka, int km, int which, int polar,
                                         int n1, T hhri, T hhpi, T hri, const T *rvi, const T *rvq)
{
    const T two = T(2.0), c53 = T(5.0 / 3.0), c02 = T(0.2), c15 = T(1.5), c43 = T(4.0 / 3.0);
    T temp;
    if (polar && which == 2) {
        temp = (psif[GIX(i, ka, ld)] - two * psif[GIX(i, k, ld)] + psif[GIX(i, km, ld)]) * hhpi * rvq[i] +
               psif[GIX(i, k, ld)] * rvq[i];
        if (i == 1)
            temp = temp + (-two * psif[GIX(i, k, ld)] + c53 * psif[GIX(i + 1, k, ld)] -
                           c02 * psif[GIX(i + 2, k, ld)]) * hhri +
                   c43 * psif[GIX(i + 1, k, ld)] * hri * rvi[i];
        else if (i == n1)
            temp = temp + (-two * psif[GIX(i, k, ld)] + c53 * psif[GIX(i - 1, k, ld)] -
                           c02 * psif[GIX(i - 2, k, ld)]) * hhri -
                   c43 * psif[GIX(i - 1, k, ld)] * hri * rvi[i];
        else
            temp = temp + (psif[GIX(i - 1, k, ld)] - two * psif[GIX(i, k, ld)] + psif[GIX(i + 1, k, ld)]) * hhri +
                   c15 * (psif[GIX(i + 1, k, ld)] - psif[GIX(i - 1, k, ld)]) * hri * rvi[i];
    } else if (polar) {
        temp = (psif[GIX(i + 1, k, ld)] + psif[GIX(i - 1, k, ld)]) * hhri +
               c15 * (psif[GIX(i + 1, k, ld)] - psif[GIX(i - 1, k, ld)]) * hri * rvi[i] +
               psif[GIX(i, k, ld)] * rvq[i] +
               (psif[GIX(i, ka, ld)] + psif[GIX(i, km, ld)]) * hhpi * rvq[i] -
               psif[GIX(i, k, ld)] * (two * hhri + two * hhpi * rvq[i]);
    } else if (which == 2) {
        temp = (psif[GIX(i, ka, ld)] - two * psif[GIX(i, k, ld)] + psif[GIX(i, km, ld)]) * hhpi;
        if (i == 1)
            temp = temp + (-two * psif[GIX(i, k, ld)] + c53 * psif[GIX(i + 1, k, ld)] -
                           c02 * psif[GIX(i + 2, k, ld)]) * hhri;
        else if (i == n1)
            temp = temp + (-two * psif[GIX(i, k, ld)] + c53 * psif[GIX(i - 1, k, ld)] -
                           c02 * psif[GIX(i - 2, k, ld)]) * hhri;
        else
            temp = temp + (psif[GIX(i - 1, k, ld)] - two * psif[GIX(i, k, ld)] + psif[GIX(i + 1, k, ld)]) * hhri;
    } else {
        temp = (psif[GIX(i + 1, k, ld)] + psif[GIX(i - 1, k, ld)]) * hhri +
               (psif[GIX(i, ka, ld)] + psif[GIX(i, km, ld)]) * hhpi -
               psif[GIX(i, k, ld)] * (two * hhri + two * hhpi);
    }
    return temp;
}

// One line k of relax2 (pentadiagonal, rows i = 1..n1, PRB:2113-2191) or
// relax3 (tridiagonal, rows i = 1..n1-1, PRB:2414-2460).
__device__ __forceinline__ void mg_line(const MgEq &E, const MgLevel &L, int k)
{
    const int ld = E.ld, n1 = L.n1, n3 = L.n3;
    double *psif = E.psif;
    const double *f = L.f;
    const double hhpi = L.hhpi;
    // the tank's last u line takes the zero k = 0 as its wall (velvor2dhorconvtank.f:1275)
    const int ka = (k == n3) ? (E.xwall ? 0 : 1) : k + 1, km = k - 1;
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
        for (int i = 1; i <= nrow; ++i) psif[GIX(i, 0, ld)] = E.xwall ? 0.0 : psif[GIX(i, k, ld)];
}

// Shared memory of the FP64 solves: the line buffer of the staged colour
// sweeps (96 KB).
#define MG64_LINE_DOUBLES 12288
#define MG64_SMEM_BYTES (MG64_LINE_DOUBLES * 8)

// One colour (lines k = 2t + 2 - parity, up to klast) of the zebra sweep, in
// batches of lines staged in shared memory: the right-hand sides of mg_line
// go in as [row][line] with an odd pitch (coalesced along rows), one thread
// per line eliminates in place with the level's factors, the solutions go
// back (with mg_line's seam copy).  The lines of a colour read only lines of
// the other colour, so the values are mg_line's.  On a cluster the batches
// go round the CTAs.
template <class G>
__device__ void mg_colour_smem(const MgEq &E, const MgLevel &L, int parity, int klast)
{
    extern __shared__ double s_mg64[];
    const int ld = E.ld, n1 = L.n1, n3 = L.n3;
    const int nrow = (E.which == 2) ? n1 : n1 - 1;
    double *psif = E.psif;
    const double *f = L.f, *rvq = L.rvq;
    const double hhpi = L.hhpi;
    const bool polar = E.polar;
    const int nlines = n3 / 2;
    int B = MG64_LINE_DOUBLES / nrow - 1;
    if (B > nlines) B = nlines;
    int rank = 0;
    if constexpr (G::C > 1) rank = (int)cg::this_cluster().block_rank();
    for (int b0 = rank * B; b0 < nlines; b0 += G::C * B) {
        const int nb = (nlines - b0 < B) ? nlines - b0 : B;
        const int pitch = nb | 1;
        for (int j = threadIdx.x >> 5; j < nb; j += blockDim.x >> 5) {
            const int k = 2 * (b0 + j) + 2 - parity;
            if (k > klast) continue;
            const int ka = (k == n3) ? (E.xwall ? 0 : 1) : k + 1, km = k - 1;
            for (int i = 1 + (threadIdx.x & 31); i <= nrow; i += 32) {
                double t = -(psif[GIX(i, ka, ld)] + psif[GIX(i, km, ld)]) * hhpi;
                if (polar) t = t * rvq[i];
                s_mg64[(i - 1) * pitch + j] = t + f[(size_t)k * (n1 + 1) + i];
            }
        }
        __syncthreads();
        for (int j = threadIdx.x; j < nb; j += blockDim.x) {
            const int k = 2 * (b0 + j) + 2 - parity;
            if (k > klast) continue;
            double *x = s_mg64 + j;
            auto in = [&](int q) -> double { return x[q * pitch]; };
            if (E.which == 2) apply_pdma_rhs(L.fac, n1, x, pitch, in);
            else apply_tdma_rhs(L.fac, n1 - 1, x, pitch, in);
        }
        __syncthreads();
        for (int j = threadIdx.x >> 5; j < nb; j += blockDim.x >> 5) {
            const int k = 2 * (b0 + j) + 2 - parity;
            if (k > klast) continue;
            for (int i = 1 + (threadIdx.x & 31); i <= nrow; i += 32) {
                const double v = s_mg64[(i - 1) * pitch + j];
                psif[GIX(i, k, ld)] = v;
                if (k == n3) psif[GIX(i, 0, ld)] = E.xwall ? 0.0 : v;
            }
        }
        __syncthreads();
    }
    if constexpr (G::C > 1) G::sync();
}

// relax2 / relax3: line sweeps (one with nrel = 1; three in the annulus),
// then the residual into rc, its max norm, and psif packed into v.  Only
// the last sweep's residual is formed: the reference recomputes rc and
// resmax after every sweep and keeps the last.  Returns the level's
// residual max norm (NaNs ignored as in the reference's comparison);
// *nan_out (uniform over the block) is set when a NaN residual appears.
template <class G>
__device__ double mg_relax(const MgEq &E, int klev, double *s_red, int *nan_out)
{
    const MgLevel &L = E.lev[klev];
    const int ld = E.ld, n1 = L.n1, n3 = L.n3;
    const double hhri = L.hhri, hhpi = L.hhpi, hri = L.hri;
    const double *rvi = L.rvi, *rvq = L.rvq;
    double *psif = E.psif, *rc = E.rc;
    const double *f = L.f;
    const int nrel = E.nrelax;
    // the tank's v lines stop short of its wall k = n3 (velvor2dhorconvtank.f:1170, :1216)
    const int klast = (E.xwall && E.which == 2) ? n3 - 1 : n3;
    for (int irel = 0; irel < nrel; ++irel) {
        if (E.mode == GB_SMOOTHER_LEX) {
            if (G::tid() == 0)
                for (int k = 1; k <= klast; ++k) mg_line(E, L, k);
            G::sync();
        } else {
            for (int parity = 1; parity >= 0; --parity) mg_colour_smem<G>(E, L, parity, klast);
        }
    }
    // residual, PRB:2306-2357 (v) and PRB:2553-2587 (u)
    double m = 0.0;
    int nan = 0;
    const int nrow = (E.which == 2) ? n1 : n1 - 1;
    const int tot = nrow * klast;
    for (int idx = G::tid(); idx < tot; idx += G::nthr()) {
        const int k = idx / nrow + 1, i = idx - (k - 1) * nrow + 1;
        const int ka = (k == n3) ? (E.xwall ? 0 : 1) : k + 1, km = k - 1;
        double temp = mg_apply_op<double>(psif, ld, i, k, ka, km, E.which, E.polar, n1, hhri, hhpi, hri, rvi, rvq);
        temp = f[(size_t)k * (n1 + 1) + i] - temp;
        rc[GIX(i, k, ld)] = temp;
        temp = fabs(temp);
        if (temp != temp) nan = 1;
        if (temp > m) m = temp;
    }
    *nan_out = grp_or<G>(nan);
    m = grp_max<G>(m, s_red);
    // trans1(psif -> v)
    const int tp = (n1 + 1) * (n3 + 1);
    for (int idx = G::tid(); idx < tp; idx += G::nthr()) {
        const int k = idx / (n1 + 1), i = idx - k * (n1 + 1);
        L.v[idx] = psif[GIX(i, k, ld)];
    }
    G::sync();
    return m;
}

// corser (PRB:2603-2718): full weighting of rc onto the packed coarse
// right-hand side; psif zeroed over the coarse region.
template <class G>
__device__ void mg_corser(const MgEq &E, int klev)
{
    const int ld = E.ld;
    const int n1c = E.lev[klev + 1].n1, n3c = E.lev[klev + 1].n3;
    const double *rf = E.rc;
    double *psif = E.psif, *fc = E.lev[klev + 1].f;
    const int tot = (n1c + 1) * (n3c + 1);
    for (int idx = G::tid(); idx < tot; idx += G::nthr()) {
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
        } else if (E.seam_keep && i >= 1 && i <= n1c - 1) {
            t = rf[GIX(i, k, ld)];   // seam lines k = 0, n3c keep rc (k = 0 is never written)
        }
        fc[idx] = t;
    }
    G::sync();
}

// finer (PRB:2721-2803): bilinear prolongation of the coarse correction plus
// the saved fine solution.
template <class G>
__device__ void mg_finer(const MgEq &E, int klev)
{
    const int ld = E.ld;
    const int n1c = E.lev[klev].n1;
    const int n1f = E.lev[klev - 1].n1, n3f = E.lev[klev - 1].n3;
    const double *vc = E.lev[klev].v, *vf = E.lev[klev - 1].v;
    double *psif = E.psif;
    const int tot = (n1f + 1) * (n3f + 1);
#define PC(ii, kk) vc[(size_t)(kk) * (n1c + 1) + (ii)]
    for (int idx = G::tid(); idx < tot; idx += G::nthr()) {
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
    G::sync();
}

// poisson2 / poisson3 (PRB:1796-1927 / PRB:1930-2059).
template <class G>
__device__ __forceinline__ void mg_solve(const MgEq *eqs, int first_eq)
{
    __shared__ double s_red[33];
    int nan1 = 0, nan_c = 0;
    const MgEq &E = eqs[first_eq + blockIdx.x / G::C];
    if (*E.abort == GB_RUN_DONE) return;   // a gang member past its last step (uniform over the block)
    const int ld = E.ld, np = E.np, nlev = E.nlev;
    const int imax = (E.which == 2) ? E.nr + 1 : E.nr;
    const int n1 = E.lev[1].n1;
    double *psif = E.psif, *psi = E.psi, *psip = E.psip;
    const int rows = imax + 1, tot = rows * (np + 1);
    // initial guess 2 psi - psip; level-1 right-hand side and solution packed
    for (int idx = G::tid(); idx < tot; idx += G::nthr()) {
        const int k = idx / rows, i = idx - k * rows;
        const size_t c = GIX(i, k, ld);
        const double pf = 2.0 * psi[c] - psip[c];
        psif[c] = pf;
        if (i <= n1) {
            E.lev[1].f[(size_t)k * (n1 + 1) + i] = E.rhs[c];
            E.lev[1].v[(size_t)k * (n1 + 1) + i] = pf;
        }
    }
    G::sync();
    int status = GB_MAXSWEEPS, sweeps = 0;
    double res1 = 0.0;
    for (int sweep = 1; sweep <= E.maxsweeps; ++sweep) {
        sweeps = sweep;
        if (sweep != 1) {
            for (int idx = G::tid(); idx < tot; idx += G::nthr()) {
                const int k = idx / rows, i = idx - k * rows;
                const size_t c = GIX(i, k, ld);
                const double pf = psip[c] + E.sor * (psif[c] - psip[c]);
                psif[c] = pf;
                psip[c] = pf;
                if (i <= n1) E.lev[1].v[(size_t)k * (n1 + 1) + i] = pf;
            }
            G::sync();
        }
        if (sweep == 1 || nlev == 1) {
            res1 = mg_relax<G>(E, 1, s_red, &nan1);
            for (int idx = G::tid(); idx < tot; idx += G::nthr()) {
                const int k = idx / rows, i = idx - k * rows;
                psip[GIX(i, k, ld)] = psif[GIX(i, k, ld)];
            }
            G::sync();
        }
        if (nlev > 1) {
            for (int l = 1; l <= nlev - 1; ++l) {
                mg_corser<G>(E, l);
                mg_relax<G>(E, l + 1, s_red, &nan_c);
            }
            for (int ifmg = 0; ifmg <= nlev - 2; ++ifmg) {
                for (int l = nlev; l >= nlev - ifmg; --l) {
                    mg_finer<G>(E, l);
                    int nn = 0;
                    double r = mg_relax<G>(E, l - 1, s_red, &nn);
                    if (l - 1 == 1) { res1 = r; nan1 = nn; }
                }
                for (int l = nlev - ifmg - 1; l <= nlev - 1; ++l) {
                    mg_corser<G>(E, l);
                    mg_relax<G>(E, l + 1, s_red, &nan_c);
                }
            }
            for (int l = nlev; l >= 2; --l) {
                mg_finer<G>(E, l);
                int nn = 0;
                double r = mg_relax<G>(E, l - 1, s_red, &nn);
                if (l - 1 == 1) { res1 = r; nan1 = nn; }
            }
        }
        // The last relax of a sweep is on level 1; its NaN flag decides.
        if (nan1) {
            status = GB_NAN;
            break;
        }
        if (res1 < E.tolcon) {
            // the tank: v on k = 1..np-1, u on k = 1..np, zero side walls
            // (velvor2dhorconvtank.f:1032-1043, :1129-1140)
            const int kend = (E.which == 2) ? np - 1 : np;
            for (int idx = G::tid(); idx < tot; idx += G::nthr()) {
                const int k = idx / rows, i = idx - k * rows;
                const size_t c = GIX(i, k, ld);
                psip[c] = psi[c];
                if (i == 0 || i == imax || (E.xwall && (k == 0 || k > kend))) psi[c] = 0.0;
                else psi[c] = psif[c];
            }
            if (E.xwall && E.which == 3)
                for (int i = G::tid(); i <= imax; i += G::nthr()) psi[GIX(i, np + 1, ld)] = 0.0;
            status = GB_OK;
            break;
        }
    }
    if (G::tid() == 0) {
        E.status[0] = status;
        E.status[1] = sweeps;
        *E.resmax = res1;
        if (status == GB_NAN || (status == GB_MAXSWEEPS && E.stop_on_max)) *E.abort = 1;
    }
}

// Launched with MG_THREADS (512) threads per block.  With a launch bound of
// 512 threads ptxas held the solve to 64 registers and spilled 604 / 1456
// bytes; allowing 128 (a whole SM's register file per block) removes every
// spill, and the bound that matters, the SM's FP64 pipe, is the same with
// one block per SM as with two.
__global__ void __maxnreg__(128) k_mg_solve(const MgEq *eqs, int first_eq)
{
    mg_solve<MgBlock>(eqs, first_eq);
}

// The same solve with each equation on a cluster of MG_CLUSTER CTAs
// (launch MG_CLUSTER blocks of MG_THREADS per equation).
__global__ void __cluster_dims__(MG_CLUSTER, 1, 1) __maxnreg__(128) k_mg_solve_cluster(const MgEq *eqs, int first_eq)
{
    mg_solve<MgCluster<MG_CLUSTER>>(eqs, first_eq);
}

// ---------------------------------------------------------------------------
// Mixed precision (GB_PRB_MIXED): FP64 defect correction around the
// reference's sweep schedule run in FP32 on the correction equation A e = r.
// A dependent FP32 operation costs a few cycles where an FP64 one costs tens
// (and an FP64 division hundreds) on this part, and the line eliminations
// are dependent chains, so the inner cycle runs an order of magnitude faster.
// The FP32 line solves multiply by stored reciprocal pivots.
// ---------------------------------------------------------------------------
template <class Rhs>
__device__ __forceinline__ void apply_pdma32(const float *fac, int n, float *x, Rhs rhs)
{
    const float *icdiv = fac, *bk1 = fac + n, *aa = fac + 2 * n, *dn = fac + 3 * n, *en = fac + 4 * n;
    const float icN = fac[5 * n];
    float rk = rhs(0), rk1 = rhs(1);
#pragma unroll 4
    for (int k = 0; k <= n - 2; ++k) {
        rk = rk * icdiv[k];
        x[k] = rk;
        rk1 = rk1 - bk1[k] * rk;
        float rk2 = 0.f;
        if (k != n - 2) rk2 = rhs(k + 2) - aa[k + 2] * rk;
        rk = rk1;
        rk1 = rk2;
    }
    float x1 = rk * icN;
    x[n - 1] = x1;
    float x0 = x[n - 2] - dn[n - 2] * x1;
    x[n - 2] = x0;
#pragma unroll 4
    for (int j = n - 3; j >= 0; --j) {
        const float xj = x[j] - dn[j] * x0 - en[j] * x1;
        x[j] = xj;
        x1 = x0;
        x0 = xj;
    }
}

template <class Rhs>
__device__ __forceinline__ void apply_tdma32(const float *fac, int n, float *x, Rhs rhs)
{
    const float *fact = fac, *ibp = fac + n, *c = fac + 2 * n;
    float prev = rhs(0);
    x[0] = prev;
#pragma unroll 4
    for (int j = 1; j < n; ++j) {
        const float rj = rhs(j) - fact[j] * prev;
        x[j] = rj;
        prev = rj;
    }
    float y = prev * ibp[n - 1];
    x[n - 1] = y;
#pragma unroll 4
    for (int j = n - 2; j >= 0; --j) {
        y = (x[j] - c[j] * y) * ibp[j];
        x[j] = y;
    }
}

__device__ __forceinline__ void mg_line32(const MgEq &E, const MgLevel &L, int k)
{
    const int ld = E.ld, n1 = L.n1, n3 = L.n3;
    float *psif = E.psif32;
    const float *f = L.f32, *rvq = L.rvq32;
    const float hhpi = (float)L.hhpi;
    const int ka = (k == n3) ? 1 : k + 1, km = k - 1;
    const int polar = E.polar;
    auto rhs = [&](int j) -> float {
        const int i = j + 1;
        float t = -(psif[GIX(i, ka, ld)] + psif[GIX(i, km, ld)]) * hhpi;
        if (polar) t = t * rvq[i];
        return t + f[(size_t)k * (n1 + 1) + i];
    };
    const int nrow = (E.which == 2) ? n1 : n1 - 1;
    if (E.which == 2) apply_pdma32(L.fac32, n1, psif + GIX(1, k, ld), rhs);
    else apply_tdma32(L.fac32, n1 - 1, psif + GIX(1, k, ld), rhs);
    if (k == n3)
        for (int i = 1; i <= nrow; ++i) psif[GIX(i, 0, ld)] = psif[GIX(i, k, ld)];
}

// Shared memory of the mixed-precision kernel: the level's FP32 factors,
// then a buffer of lines stored [row][line] with an odd pitch, so that
// lanes walking rows (staging) and threads walking their own line
// (elimination) both hit distinct banks.
#define MG32_FAC_FLOATS 8192                  // >= 5 n1 + 1 for n1 <= 1600
#define MG32_LINE_FLOATS 24576                // 96 KB of lines
#define MG32_SMEM_BYTES ((MG32_FAC_FLOATS + MG32_LINE_FLOATS) * 4)

// One colour (lines k = 2t + 2 - parity) of the zebra line sweep of the
// correction cycle, in batches of lines staged in shared memory: right-hand
// sides in (coalesced along rows), one thread per line eliminates, solutions
// out.
template <class G>
__device__ void mg_colour32_smem(const MgEq &E, const MgLevel &L, int parity)
{
    extern __shared__ float s_mg32[];
    float *sfac = s_mg32, *sline = s_mg32 + E.smem_fac;
    const int ld = E.ld, n1 = L.n1, n3 = L.n3;
    const int nrow = (E.which == 2) ? n1 : n1 - 1;
    const int nfac = (E.which == 2) ? 5 * n1 + 1 : 3 * (n1 - 1);
    for (int j = threadIdx.x; j < nfac; j += blockDim.x) sfac[j] = L.fac32[j];
    float *psif = E.psif32;
    const float *f = L.f32, *rvq = L.rvq32;
    const float hhpi = (float)L.hhpi;
    const int nlines = n3 / 2;
    int B = MG32_LINE_FLOATS / nrow - 1;
    if (B > nlines) B = nlines;
    // batches of lines in turn over the group's CTAs; within a batch only
    // this CTA's threads meet
    int rank = 0;
    if constexpr (G::C > 1) rank = (int)cg::this_cluster().block_rank();
    for (int b0 = rank * B; b0 < nlines; b0 += G::C * B) {
        const int nb = (nlines - b0 < B) ? nlines - b0 : B;
        const int pitch = nb | 1;
        for (int j = threadIdx.x >> 5; j < nb; j += blockDim.x >> 5) {
            const int k = 2 * (b0 + j) + 2 - parity;
            const int ka = (k == n3) ? 1 : k + 1, km = k - 1;
            for (int i = 1 + (threadIdx.x & 31); i <= nrow; i += 32) {
                float r = -(psif[GIX(i, ka, ld)] + psif[GIX(i, km, ld)]) * hhpi;
                if (E.polar) r = r * rvq[i];
                sline[(i - 1) * pitch + j] = r + f[(size_t)k * (n1 + 1) + i];
            }
        }
        __syncthreads();
        for (int j = threadIdx.x; j < nb; j += blockDim.x) {
            if (E.which == 2) pdma32_smem(sfac, n1, sline + j, pitch);
            else tdma32_smem(sfac, n1 - 1, sline + j, pitch);
        }
        __syncthreads();
        for (int j = threadIdx.x >> 5; j < nb; j += blockDim.x >> 5) {
            const int k = 2 * (b0 + j) + 2 - parity;
            for (int i = 1 + (threadIdx.x & 31); i <= nrow; i += 32) {
                const float v = sline[(i - 1) * pitch + j];
                psif[GIX(i, k, ld)] = v;
                if (k == n3) psif[GIX(i, 0, ld)] = v;
            }
        }
        __syncthreads();
    }
    if constexpr (G::C > 1) G::sync();
}

// relax2/relax3 of the correction cycle: line sweeps, residual into rc32,
// psif32 packed into v32.
template <class G>
__device__ void mg_relax32(const MgEq &E, int klev)
{
    const MgLevel &L = E.lev[klev];
    const int ld = E.ld, n1 = L.n1, n3 = L.n3;
    const float hhri = (float)L.hhri, hhpi = (float)L.hhpi, hri = (float)L.hri;
    float *psif = E.psif32, *rc = E.rc32;
    const int nrel = E.nrelax;
    for (int irel = 0; irel < nrel; ++irel) {
        if (E.mode == GB_SMOOTHER_LEX) {
            if (G::tid() == 0)
                for (int k = 1; k <= n3; ++k) mg_line32(E, L, k);
            G::sync();
        } else {
            for (int parity = 1; parity >= 0; --parity) mg_colour32_smem<G>(E, L, parity);
        }
    }
    const int nrow = (E.which == 2) ? n1 : n1 - 1;
    const int tot = nrow * n3;
    for (int k = 1 + (G::tid() >> 5); k <= n3; k += (G::nthr() >> 5))
        for (int i = 1 + (threadIdx.x & 31); i <= nrow; i += 32) {
        const int ka = (k == n3) ? 1 : k + 1, km = k - 1;
        const float a = mg_apply_op<float>(psif, ld, i, k, ka, km, E.which, E.polar, n1, hhri, hhpi, hri, L.rvi32,
                                           L.rvq32);
        rc[GIX(i, k, ld)] = L.f32[(size_t)k * (n1 + 1) + i] - a;
    }
    G::sync();
    const int tp = (n1 + 1) * (n3 + 1);
    for (int k = (G::tid() >> 5); k < (tp) / ((n1 + 1)); k += (G::nthr() >> 5))
        for (int i = threadIdx.x & 31; i < (n1 + 1); i += 32) {
            const int idx = k * (n1 + 1) + i;
        L.v32[idx] = psif[GIX(i, k, ld)];
    }
    G::sync();
}

template <class G>
__device__ void mg_corser32(const MgEq &E, int klev)
{
    const int ld = E.ld;
    const int n1c = E.lev[klev + 1].n1, n3c = E.lev[klev + 1].n3;
    const float *rf = E.rc32;
    float *psif = E.psif32, *fc = E.lev[klev + 1].f32;
    const int tot = (n1c + 1) * (n3c + 1);
    for (int k = (G::tid() >> 5); k < (tot) / ((n1c + 1)); k += (G::nthr() >> 5))
        for (int i = threadIdx.x & 31; i < (n1c + 1); i += 32) {
            const int idx = k * (n1c + 1) + i;
        psif[GIX(i, k, ld)] = 0.f;
        float t = 0.f;
        if (i >= 1 && i <= n1c - 1 && k >= 1 && k <= n3c - 1) {
            const int ii = i + i, kk = k + k;
            // full weighting: 1/4 centre, 1/8 edges, 1/16 corners
            t = 0.25f * rf[GIX(ii, kk, ld)] +
                0.125f * (rf[GIX(ii + 1, kk, ld)] + rf[GIX(ii - 1, kk, ld)] + rf[GIX(ii, kk + 1, ld)] +
                          rf[GIX(ii, kk - 1, ld)]) +
                0.0625f * (rf[GIX(ii + 1, kk + 1, ld)] + rf[GIX(ii + 1, kk - 1, ld)] + rf[GIX(ii - 1, kk + 1, ld)] +
                           rf[GIX(ii - 1, kk - 1, ld)]);
        } else if (E.seam_keep && i >= 1 && i <= n1c - 1 && k == n3c) {
            t = rf[GIX(i, k, ld)];
        }
        fc[idx] = t;
    }
    G::sync();
}

template <class G>
__device__ void mg_finer32(const MgEq &E, int klev)
{
    const int ld = E.ld;
    const int n1c = E.lev[klev].n1;
    const int n1f = E.lev[klev - 1].n1, n3f = E.lev[klev - 1].n3;
    const float *vc = E.lev[klev].v32, *vf = E.lev[klev - 1].v32;
    float *psif = E.psif32;
    const int tot = (n1f + 1) * (n3f + 1);
#define PC(ii, kk) vc[(size_t)(kk) * (n1c + 1) + (ii)]
    for (int k = (G::tid() >> 5); k < (tot) / ((n1f + 1)); k += (G::nthr() >> 5))
        for (int i = threadIdx.x & 31; i < (n1f + 1); i += 32) {
            const int idx = k * (n1f + 1) + i;
        const int i1 = i / 2, k1 = k / 2;
        float p;
        if (i1 * 2 == i) {
            if (k1 * 2 == k) p = PC(i1, k1);
            else p = (PC(i1, k1) + PC(i1, k1 + 1)) * 0.5f;
        } else {
            if (k1 * 2 == k) p = (PC(i1, k1) + PC(i1 + 1, k1)) * 0.5f;
            else p = (PC(i1, k1) + PC(i1 + 1, k1) + PC(i1, k1 + 1) + PC(i1 + 1, k1 + 1)) * 0.25f;
        }
        psif[GIX(i, k, ld)] = p + vf[idx];
    }
#undef PC
    G::sync();
}

// One FP32 cycle of the reference's sweep schedule (relax on the finest
// level, the FMG-flavoured down and up legs of PRB:1869-1893) on A e = r
// from e = 0.
template <class G>
__device__ void mg_cycle32(const MgEq &E)
{
    const int nlev = E.nlev;
    mg_relax32<G>(E, 1);
    if (nlev > 1) {
        for (int l = 1; l <= nlev - 1; ++l) {
            mg_corser32<G>(E, l);
            mg_relax32<G>(E, l + 1);
        }
        for (int ifmg = 0; ifmg <= nlev - 2; ++ifmg) {
            for (int l = nlev; l >= nlev - ifmg; --l) {
                mg_finer32<G>(E, l);
                mg_relax32<G>(E, l - 1);
            }
            for (int l = nlev - ifmg - 1; l <= nlev - 1; ++l) {
                mg_corser32<G>(E, l);
                mg_relax32<G>(E, l + 1);
            }
        }
        for (int l = nlev; l >= 2; --l) {
            mg_finer32<G>(E, l);
            mg_relax32<G>(E, l - 1);
        }
    }
}

// poisson2 / poisson3 in mixed precision.  psif holds the FP64 iterate.
template <class G>
__device__ __forceinline__ void mg_solve_mixed(const MgEq *eqs, int first_eq)
{
    __shared__ double s_red[33];
    const MgEq &E = eqs[first_eq + blockIdx.x / G::C];
    if (*E.abort == GB_RUN_DONE) return;   // a gang member past its last step (uniform over the block)
    const MgLevel &L1 = E.lev[1];
    const int ld = E.ld, np = E.np;
    const int imax = (E.which == 2) ? E.nr + 1 : E.nr;
    const int n1 = L1.n1, n3 = L1.n3;
    double *psif = E.psif, *psi = E.psi, *psip = E.psip;
    const int rows = imax + 1, tot = rows * (np + 1);
    for (int k = (G::tid() >> 5); k < (tot) / (rows); k += (G::nthr() >> 5))
        for (int i = threadIdx.x & 31; i < rows; i += 32) {
            const int idx = k * rows + i;
        const size_t c = GIX(i, k, ld);
        psif[c] = 2.0 * psi[c] - psip[c];
        if (i <= n1) L1.f[(size_t)k * (n1 + 1) + i] = E.rhs[c];
    }
    G::sync();
    const int nrow = (E.which == 2) ? n1 : n1 - 1;
    int status = GB_MAXSWEEPS, cycles = 0;
    double res = 0.0;
    for (int it = 0;; ++it) {
        // FP64 residual of the iterate; its FP32 copy is the cycle's right-hand side
        double m = 0.0;
        int nan = 0;
        // packed 1D mapping: partly filled warps cost a full FP64 issue slot
        for (int idx = G::tid(); idx < nrow * n3; idx += G::nthr()) {
            const int k = idx / nrow + 1, i = idx - (k - 1) * nrow + 1;
            const int ka = (k == n3) ? 1 : k + 1, km = k - 1;
            const double a = mg_apply_op<double>(psif, ld, i, k, ka, km, E.which, E.polar, n1, L1.hhri, L1.hhpi,
                                                 L1.hri, L1.rvi, L1.rvq);
            const double r = L1.f[(size_t)k * (n1 + 1) + i] - a;
            L1.f32[(size_t)k * (n1 + 1) + i] = (float)r;
            const double ar = fabs(r);
            if (ar != ar) nan = 1;
            if (ar > m) m = ar;
        }
        nan = grp_or<G>(nan);
        res = grp_max<G>(m, s_red);
        if (nan) { status = GB_NAN; break; }
        if (res < E.tolcon) { status = GB_OK; break; }
        if (it == E.maxsweeps) break;
        // e = 0 on the finest level, then one FP32 cycle
        for (int k = (G::tid() >> 5); k < (n3 + 1); k += (G::nthr() >> 5))
            for (int i = threadIdx.x & 31; i < (n1 + 2); i += 32) {
                const int idx = k * (n1 + 2) + i;
            E.psif32[GIX(i, k, ld)] = 0.f;
        }
        G::sync();
        mg_cycle32<G>(E);
        const double w = (it == 0) ? 1.0 : E.sor;
        for (int idx = G::tid(); idx < nrow * (n3 + 1); idx += G::nthr()) {
            const int k = idx / nrow, i = idx - k * nrow + 1;
            psif[GIX(i, k, ld)] += w * (double)E.psif32[GIX(i, k, ld)];
        }
        G::sync();
        cycles = it + 1;
    }
    if (status == GB_OK) {
        for (int k = (G::tid() >> 5); k < (tot) / (rows); k += (G::nthr() >> 5))
            for (int i = threadIdx.x & 31; i < rows; i += 32) {
                const int idx = k * rows + i;
            const size_t c = GIX(i, k, ld);
            psip[c] = psi[c];
            psi[c] = (i == 0 || i == imax) ? 0.0 : psif[c];
        }
    }
    if (G::tid() == 0) {
        E.status[0] = status;
        E.status[1] = cycles;
        *E.resmax = res;
        if (status == GB_NAN || (status == GB_MAXSWEEPS && E.stop_on_max)) *E.abort = 1;
    }
}

__global__ void __maxnreg__(128) k_mg_solve_mixed(const MgEq *eqs, int first_eq)
{
    mg_solve_mixed<MgBlock>(eqs, first_eq);
}

// The mixed solve with each equation on a cluster of MG_CLUSTER CTAs: the
// FP64 residual passes, the FP32 residual and transfer passes and the
// batches of each colour's lines are spread over the cluster's SMs.
__global__ void __cluster_dims__(MG_CLUSTER, 1, 1) __maxnreg__(128) k_mg_solve_mixed_cluster(const MgEq *eqs,
                                                                                              int first_eq)
{
    mg_solve_mixed<MgCluster<MG_CLUSTER>>(eqs, first_eq);
}

// FP32 copies of the factors (pivots as reciprocals) and radii.
__global__ void k_mg_factors32(MgEq eq)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int l = 1; l <= eq.nlev; ++l) {
        const MgLevel &L = eq.lev[l];
        const int n1 = L.n1;
        float *f32 = L.fac32;
        const double *f = L.fac;
        if (eq.which == 2) {
            const int n = n1;
            for (int j = 0; j < n; ++j) {
                f32[j] = (float)(1.0 / f[j]);                     // cdiv
                f32[n + j] = (float)f[n + j];                     // bk1
                f32[2 * n + j] = (float)f[2 * n + j];             // a
                f32[3 * n + j] = (float)f[3 * n + j];             // d
                f32[4 * n + j] = (float)f[4 * n + j];             // e
            }
            f32[5 * n] = (float)(1.0 / f[5 * n]);
        } else {
            const int n = n1 - 1;
            for (int j = 0; j < n; ++j) {
                f32[j] = (float)f[j];                             // fact
                f32[n + j] = (float)(1.0 / f[n + j]);             // bp
                f32[2 * n + j] = (float)f[2 * n + j];             // c
            }
        }
        for (int i = 0; i <= n1 + 1; ++i) {
            L.rvi32[i] = (float)L.rvi[i];
            L.rvq32[i] = (float)L.rvq[i];
        }
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
    if (5 * nr + 1 > MG32_FAC_FLOATS || 2 * nr > MG32_LINE_FLOATS) {
        gb_set_error("nr=%d exceeds the multigrid kernel's shared-memory line buffers", nr);
        return GB_ERR_INVALID;
    }
    if (np % (1 << nlev) != 0) {
        gb_set_error("np=%d must be divisible by 2^nlev=%d so that every multigrid level has an even number of lines", np, 1 << nlev);
        return GB_ERR_INVALID;
    }
    // pool: per equation psif, rc (full) + per level v, f + factors; plus work
    size_t per_eq = 2 * (size_t)ld * (np + 1) + (size_t)ld * (np + 1) + 8;   // psif, rc; psif32 + rc32
    for (int l = 1; l <= nlev; ++l) {
        const int n1 = nr * 2 / (1 << l), n3 = np * 2 / (1 << l);
        per_eq += 2 * (size_t)(n1 + 1) * (n3 + 1) + pdma_fac_len(n1 + 2) + 2 * (size_t)(n1 + 2);
        // FP32: v32, f32, fac32, rvi32, rvq32 (counted in doubles, rounded up)
        per_eq += ((2 * (size_t)(n1 + 1) * (n3 + 1) + 5 * (size_t)(n1 + 2) + 1 + 2 * (size_t)(n1 + 2)) + 1) / 2 + 4;
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
        E.polar = p.variant == GB_PRB_ANNULUS || p.variant == GB_PRB_TAYCOU;
        E.nrelax = p.variant == GB_PRB_ANNULUS ? 3 : 1;
        E.seam_keep = p.variant == GB_PRB_ANNULUS;
        E.xwall = p.variant == GB_PRB_TANK || p.variant == GB_PRB_DVD;
        if (E.xwall && p.precision != GB_PRB_FP64) return GB_ERR_INVALID;
        E.stop_on_max = p.variant != GB_PRB_ANNULUS;
        E.smem_fac = ((5 * nr + 1 + 31) / 32) * 32;   // the level-1 pentadiagonal factors, rounded to 128 B
        E.r0 = p.r0;
        double *base = h->mg_pool + q * per_eq;
        E.psif = base; base += (size_t)ld * (np + 1);
        E.rc = base; base += (size_t)ld * (np + 1);
        E.psic = E.rf = E.tempa = nullptr;
        float *fbase = (float *)base;
        E.psif32 = fbase; fbase += (size_t)ld * (np + 1);
        E.rc32 = fbase; fbase += (size_t)ld * (np + 1);
        base = (double *)(((uintptr_t)fbase + 15) & ~(uintptr_t)15);
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
            L.fac = base; base += pdma_fac_len(L.n1 + 2);   // >= tdma_fac_len(n1 - 1)
            L.rvi = base; base += (size_t)(L.n1 + 2);
            L.rvq = base; base += (size_t)(L.n1 + 2);
            float *fb = (float *)base;
            L.v32 = fb; fb += sz;
            L.f32 = fb; fb += sz;
            L.fac32 = fb; fb += 5 * (size_t)(L.n1 + 2) + 1;
            L.rvi32 = fb; fb += (size_t)(L.n1 + 2);
            L.rvq32 = fb; fb += (size_t)(L.n1 + 2);
            base = (double *)(((uintptr_t)fb + 15) & ~(uintptr_t)15);
        }
        E.psi = h->dev.f[q == 0 ? GB_F_vel : GB_F_uel];
        E.psip = h->dev.f[q == 0 ? GB_F_velp : GB_F_uelp];
        E.rhs = h->dev.f[q == 0 ? GB_F_vrh : GB_F_urh];
        E.status = h->dev.mg_status + 2 * q;
        E.resmax = h->dev.mg_resmax + q;
        E.abort = h->dev.abort;
        k_mg_factors<<<1, 1>>>(E, wk);
        k_mg_factors32<<<1, 1>>>(E);
    }
    e = cudaFuncSetAttribute(k_mg_solve_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, MG32_SMEM_BYTES);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mg_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, MG64_SMEM_BYTES);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mg_solve_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, MG64_SMEM_BYTES);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mg_solve_mixed_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, MG32_SMEM_BYTES);
    if (e != cudaSuccess) { gb_set_error("multigrid shared memory: %s", cudaGetErrorString(e)); return GB_ERR_CUDA; }
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
// Shared memory of one instance's mixed solve: its factors, then the line
// buffer.
size_t prb_mg_smem(const gb_prb *h)
{
    return sizeof(float) * ((size_t)h->eq_host[0].smem_fac + MG32_LINE_FLOATS);
}

// The solves of neq equation descriptors (any instances') in one launch,
// one block or one cluster of MG_CLUSTER blocks each (the gangs' batched
// multigrid); smem: the largest member's prb_mg_smem.  A gang step waits
// for its slowest solve, so the solves keep the single-instance block of
// MG_THREADS: with half-size blocks, two per SM, the served sweep's mixed
// arm ran 1.5 instead of 2.25 solves/s.
void prb_mg_launch_eqs(const MgEq *d_eqs, int neq, int mixed, int spread, size_t smem, cudaStream_t s)
{
    if (neq <= 0) return;
    if (spread > 1) {
        if (mixed) k_mg_solve_mixed_cluster<<<neq * MG_CLUSTER, MG_THREADS, smem, s>>>(d_eqs, 0);
        else k_mg_solve_cluster<<<neq * MG_CLUSTER, MG_THREADS, MG64_SMEM_BYTES, s>>>(d_eqs, 0);
    } else if (mixed) {
        k_mg_solve_mixed<<<neq, MG_THREADS, smem, s>>>(d_eqs, 0);
    } else {
        k_mg_solve<<<neq, MG_THREADS, MG64_SMEM_BYTES, s>>>(d_eqs, 0);
    }
}

int prb_mg_cluster_ctas() { return MG_CLUSTER; }

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
    const bool spread = h->mg_spread > 1 && h->p.smoother == GB_SMOOTHER_ZEBRA;
    if (h->p.precision == GB_PRB_MIXED) {
        if (spread) k_mg_solve_mixed_cluster<<<n * MG_CLUSTER, MG_THREADS, prb_mg_smem(h), s>>>(h->eq_dev, first);
        else k_mg_solve_mixed<<<n, MG_THREADS, prb_mg_smem(h), s>>>(h->eq_dev, first);
    } else if (spread) {
        k_mg_solve_cluster<<<n * MG_CLUSTER, MG_THREADS, MG64_SMEM_BYTES, s>>>(h->eq_dev, first);
    } else {
        k_mg_solve<<<n, MG_THREADS, MG64_SMEM_BYTES, s>>>(h->eq_dev, first);
    }
    h->launches += 1;
    return GB_OK;
}

extern "C" int gb_prb_set_solve_spread(gb_prb *h, int ctas)
{
    if (!h || (ctas != 1 && ctas != MG_CLUSTER)) {
        gb_set_error("gb_prb_set_solve_spread: ctas must be 1 or %d", MG_CLUSTER);
        return GB_ERR_INVALID;
    }
    if (h->mg_spread != ctas) {
        h->mg_spread = ctas;
        if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; }
        if (h->graph_exec1) { cudaGraphExecDestroy(h->graph_exec1); h->graph_exec1 = nullptr; }
    }
    return GB_OK;
}
