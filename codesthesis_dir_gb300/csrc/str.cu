// Stretched-grid streamfunction multigrid of rcsc.f on sm_103a, FP64,
// bit-identical to the oracle (-fmad=false, IEEE division, the reference's
// order): psi_rr + psi_r / r - psi / r^2 + psi_zz with grid.f's per-level
// finite-difference weights, pentadiagonal r-line and z-line Gauss-Seidel,
// nine-point restriction, bilinear prolongation, plain V-cycle (rcsc.f:
// 1118-1444).
//
// One persistent block per solve (the AXI solver's structure).  Every
// r-line has its own matrix (the z weights of its row shift the diagonal)
// and every z-line its own (the r weights and -1/r^2 of its column), so the
// matrix halves of all line eliminations are done once at creation
// (factor_pdma, one thread per line) and a sweep only carries right-hand
// sides through them.  Line orders: the reference's (r-lines j = 1..n2-1 in
// order, then z-lines i = 1..n1-1, on one thread: each line needs the one
// before it) or four colours (index mod 4 = 1, 2, 3, 0: a line reads the
// lines one and two away, never one of its colour), each colour's lines in
// parallel.
#include "gbcommon.cuh"
#include "banded.cuh"
#include "str_internal.cuh"

#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#define STR_THREADS 512
#define STR_MAXLEV 8

struct StrLevel {
    int n1, n2;
    double *r, *cr, *crr, *czz;
    double *ir, *irr;         // 1/r and 1/(r*r) per row (IEEE, host): the divisors' reciprocals
    double *v, *f;            // packed (n1+1)*(n2+1)
    double *fac_r, *fac_z;    // per r-line j (5(n1-1)+1 each), per z-line i (5(n2-1)+1 each)
    // mixed precision: FP32 copies (pivots of the factors as reciprocals)
    float *r32, *cr32, *crr32, *czz32, *v32, *f32, *fac_r32, *fac_z32;
};

struct StrDev {
    int nlev, ld, nrel, maxsweeps, mode;
    double tolcon;
    double *psif, *rc;        // ld x ld, ld = max(n1, n2) + 1
    float *psif32, *rc32;     // the same for the FP32 correction cycles
    double *io_psi, *io_rhs;  // level-1 (n1+1) x (n2+1) staging of the caller's arrays
    StrLevel lev[STR_MAXLEV];
    int *status;              // [0] status, [1] sweeps
    int *abort;               // optional (a time loop's flag): the solve is skipped while it is set and
                              // sets it to 1 when the residual is a NaN
};

#define PS(i, j) d.psif[(size_t)(i) + (size_t)d.ld * (size_t)(j)]
#define CR(i, k) L.cr[3 * ((i) - 1) + (k) - 1]
#define CRR(i, k) L.crr[4 * ((i) - 1) + (k) - 1]
#define CZZ(j, k) L.czz[4 * ((j) - 1) + (k) - 1]

// Matrix of r-line j (rcsc.f:1228-1252) or z-line i (rcsc.f:1265-1285).
__device__ void str_line_matrix(const StrLevel &L, int dir, int line, double *a, double *b, double *c, double *dd,
                                double *e)
{
    const int n1 = L.n1, n2 = L.n2;
    if (dir == 0) {
        const int j = line;
        for (int i = 1; i <= n1 - 1; ++i) {
            const int q = i - 1;
            const double r = L.r[i];
            if (i <= n1 / 2) {
                a[q] = 0.0;
                b[q] = CRR(i, 1) + CR(i, 1) / r;
                c[q] = CRR(i, 2) + CR(i, 2) / r - 1.0 / (r * r);
                dd[q] = CRR(i, 3) + CR(i, 3) / r;
                e[q] = CRR(i, 4);
            } else {
                a[q] = CRR(i, 1);
                b[q] = CRR(i, 2) + CR(i, 1) / r;
                c[q] = CRR(i, 3) + CR(i, 2) / r - 1.0 / (r * r);
                dd[q] = CRR(i, 4) + CR(i, 3) / r;
                e[q] = 0.0;
            }
            if (j <= n2 / 2) c[q] = c[q] + CZZ(j, 2);
            else c[q] = c[q] + CZZ(j, 3);
        }
    } else {
        const int i = line;
        const double r = L.r[i];
        for (int j = 1; j <= n2 - 1; ++j) {
            const int q = j - 1;
            if (j <= n2 / 2) {
                a[q] = 0.0;
                b[q] = CZZ(j, 1);
                c[q] = CZZ(j, 2) - 1.0 / (r * r);
                dd[q] = CZZ(j, 3);
                e[q] = CZZ(j, 4);
            } else {
                a[q] = CZZ(j, 1);
                b[q] = CZZ(j, 2);
                c[q] = CZZ(j, 3) - 1.0 / (r * r);
                dd[q] = CZZ(j, 4);
                e[q] = 0.0;
            }
            if (i <= n1 / 2) c[q] = c[q] + CRR(i, 2) + CR(i, 2) / r;
            else c[q] = c[q] + CRR(i, 3) + CR(i, 2) / r;
        }
    }
}

struct StrJob {
    int lev, dir, line;
};

__global__ void k_str_factors(const __grid_constant__ StrDev d, const StrJob *jobs, int njobs, double *work, int wstride)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= njobs) return;
    const StrJob J = jobs[q];
    const StrLevel &L = d.lev[J.lev];
    const int n = J.dir == 0 ? L.n1 - 1 : L.n2 - 1;
    double *w = work + (size_t)q * wstride;
    double *a = w, *b = w + n, *c = w + 2 * n, *dd = w + 3 * n, *e = w + 4 * n, *scratch = w + 5 * n;
    str_line_matrix(L, J.dir, J.line, a, b, c, dd, e);
    double *fac = J.dir == 0 ? L.fac_r + (size_t)(J.line - 1) * pdma_fac_len(n) : L.fac_z + (size_t)(J.line - 1) * pdma_fac_len(n);
    factor_pdma(a, b, c, dd, e, n, fac, scratch);
}

// r-line j: right-hand side of row i (rcsc.f:1246-1252)
__device__ __forceinline__ void str_rline(const StrDev &d, const StrLevel &L, int j)
{
    const int n1 = L.n1, n2 = L.n2;
    const double *f = L.f;
    auto rhs = [&](int q) -> double {
        const int i = q + 1;
        if (j <= n2 / 2)
            return -(CZZ(j, 1) * PS(i, j - 1) + CZZ(j, 3) * PS(i, j + 1) + CZZ(j, 4) * PS(i, j + 2)) +
                   f[(size_t)i + (size_t)(n1 + 1) * j];
        return -(CZZ(j, 1) * PS(i, j - 2) + CZZ(j, 2) * PS(i, j - 1) + CZZ(j, 4) * PS(i, j + 1)) +
               f[(size_t)i + (size_t)(n1 + 1) * j];
    };
    const int n = n1 - 1;
    apply_pdma_rhs(L.fac_r + (size_t)(j - 1) * pdma_fac_len(n), n, &PS(1, j), 1, rhs);
}

// z-line i: right-hand side of row j (rcsc.f:1279-1290)
__device__ __forceinline__ void str_zline(const StrDev &d, const StrLevel &L, int i)
{
    const int n1 = L.n1, n2 = L.n2;
    const double *f = L.f;
    const double r = L.r[i];
    auto rhs = [&](int q) -> double {
        const int j = q + 1;
        if (i <= n1 / 2)
            return -(CRR(i, 1) * PS(i - 1, j) + CRR(i, 3) * PS(i + 1, j) + CRR(i, 4) * PS(i + 2, j) +
                     div_by_rcp(CR(i, 1) * PS(i - 1, j) + CR(i, 3) * PS(i + 1, j), r, L.ir[i])) +
                   f[(size_t)i + (size_t)(n1 + 1) * j];
        return -(CRR(i, 1) * PS(i - 2, j) + CRR(i, 2) * PS(i - 1, j) + CRR(i, 4) * PS(i + 1, j) +
                 div_by_rcp(CR(i, 1) * PS(i - 1, j) + CR(i, 3) * PS(i + 1, j), r, L.ir[i])) +
               f[(size_t)i + (size_t)(n1 + 1) * j];
    };
    const int n = n2 - 1;
    apply_pdma_rhs(L.fac_z + (size_t)(i - 1) * pdma_fac_len(n), n, &PS(i, 1), d.ld, rhs);
}

// Shared memory of a solve: the line buffer of the staged two-direction
// sweeps (96 KB: 12288 doubles or 24576 floats).
#define STR_LINE_BYTES (96 * 1024)

// Right-hand sides of r-line j at row i and of z-line i at row j, as
// str_rline and str_zline form them.
__device__ __forceinline__ double str_rhs_r(const StrDev &d, const StrLevel &L, int j, int i)
{
    const int n1 = L.n1, n2 = L.n2;
    const double *f = L.f;
    if (j <= n2 / 2)
        return -(CZZ(j, 1) * PS(i, j - 1) + CZZ(j, 3) * PS(i, j + 1) + CZZ(j, 4) * PS(i, j + 2)) +
               f[(size_t)i + (size_t)(n1 + 1) * j];
    return -(CZZ(j, 1) * PS(i, j - 2) + CZZ(j, 2) * PS(i, j - 1) + CZZ(j, 4) * PS(i, j + 1)) +
           f[(size_t)i + (size_t)(n1 + 1) * j];
}

__device__ __forceinline__ double str_rhs_z(const StrDev &d, const StrLevel &L, int i, int j)
{
    const int n1 = L.n1;
    const double *f = L.f;
    const double r = L.r[i];
    if (i <= n1 / 2)
        return -(CRR(i, 1) * PS(i - 1, j) + CRR(i, 3) * PS(i + 1, j) + CRR(i, 4) * PS(i + 2, j) +
                 div_by_rcp(CR(i, 1) * PS(i - 1, j) + CR(i, 3) * PS(i + 1, j), r, L.ir[i])) +
               f[(size_t)i + (size_t)(n1 + 1) * j];
    return -(CRR(i, 1) * PS(i - 2, j) + CRR(i, 2) * PS(i - 1, j) + CRR(i, 4) * PS(i + 1, j) +
             div_by_rcp(CR(i, 1) * PS(i - 1, j) + CR(i, 3) * PS(i + 1, j), r, L.ir[i])) +
           f[(size_t)i + (size_t)(n1 + 1) * j];
}

// One colour (every fourth line from `first`) of one direction (DIR 0:
// r-lines j, DIR 1: z-lines i) in batches staged in shared memory: the
// right-hand sides go in as [row][line] with an odd pitch (coalesced along
// the grid's rows, conflict-free for the per-line elimination), one thread
// per line eliminates in place, the solutions go back.  The lines of a
// colour read only lines of the other colours, so staging changes no value.
template <int DIR>
__device__ void str_colour_smem(const StrDev &d, const StrLevel &L, int first, double *sline)
{
    const int n1 = L.n1, n2 = L.n2;
    const int lines = DIR == 0 ? n2 - 1 : n1 - 1, n = DIR == 0 ? n1 - 1 : n2 - 1;
    if (first > lines) return;
    const int nl = (lines - first) / 4 + 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int B = (int)(STR_LINE_BYTES / sizeof(double)) / n - 1;
    if (B < 1) {   // lines too long to stage: one thread per line on the level's arrays
        for (int t = threadIdx.x; t < nl; t += blockDim.x) {
            if (DIR == 0) str_rline(d, L, first + 4 * t);
            else str_zline(d, L, first + 4 * t);
        }
        __syncthreads();
        return;
    }
    if (B > nl) B = nl;
    for (int b0 = 0; b0 < nl; b0 += B) {
        const int nb = min(B, nl - b0), pitch = nb | 1;
        if (DIR == 0) {
            for (int t = warp; t < nb; t += nw)
                for (int q = lane; q < n; q += 32) sline[q * pitch + t] = str_rhs_r(d, L, first + 4 * (b0 + t), q + 1);
        } else {
            for (int q = warp; q < n; q += nw)
                for (int t = lane; t < nb; t += 32) sline[q * pitch + t] = str_rhs_z(d, L, first + 4 * (b0 + t), q + 1);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < nb; t += blockDim.x) {
            const int line = first + 4 * (b0 + t);
            double *x = sline + t;
            const double *fac = (DIR == 0 ? L.fac_r : L.fac_z) + (size_t)(line - 1) * pdma_fac_len(n);
            apply_pdma_rhs(fac, n, x, pitch, [&](int q) -> double { return x[q * pitch]; });
        }
        __syncthreads();
        if (DIR == 0) {
            for (int t = warp; t < nb; t += nw)
                for (int q = lane; q < n; q += 32) PS(q + 1, first + 4 * (b0 + t)) = sline[q * pitch + t];
        } else {
            for (int q = warp; q < n; q += nw)
                for (int t = lane; t < nb; t += 32) PS(first + 4 * (b0 + t), q + 1) = sline[q * pitch + t];
        }
        __syncthreads();
    }
}

__device__ __forceinline__ double str_blk_max(double v, double *s_red)
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

// relax (rcsc.f:1197-1341); returns the last residual max norm.
__device__ double str_relax(const StrDev &d, int klev, double *s_red, int *nan_out)
{
    const StrLevel &L = d.lev[klev];
    const int n1 = L.n1, n2 = L.n2;
    const int tp = (n1 + 1) * (n2 + 1);
    for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
        const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
        PS(i, j) = L.v[idx];
    }
    __syncthreads();
    double m = 0.0;
    int nan = 0;
    for (int irel = 0; irel < d.nrel; ++irel) {
        if (d.mode == GB_SMOOTHER_LEX) {
            if (threadIdx.x == 0) {
                for (int j = 1; j <= n2 - 1; ++j) str_rline(d, L, j);
                for (int i = 1; i <= n1 - 1; ++i) str_zline(d, L, i);
            }
            __syncthreads();
        } else {
            extern __shared__ double s_str_line[];
            for (int c = 1; c <= 4; ++c) str_colour_smem<0>(d, L, (c & 3) == 0 ? 4 : (c & 3), s_str_line);
            for (int c = 1; c <= 4; ++c) str_colour_smem<1>(d, L, (c & 3) == 0 ? 4 : (c & 3), s_str_line);
        }
        m = 0.0;
        nan = 0;
        const int ni = n1 - 1, tot = ni * (n2 - 1);
        for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
            const int j = idx / ni + 1, i = idx - (j - 1) * ni + 1;
            const double r = L.r[i];
            double temp;
            if (i <= n1 / 2)
                temp = CRR(i, 1) * PS(i - 1, j) + CRR(i, 2) * PS(i, j) + CRR(i, 3) * PS(i + 1, j) +
                       CRR(i, 4) * PS(i + 2, j) + div_by_rcp(CR(i, 1) * PS(i - 1, j) + CR(i, 2) * PS(i, j) + CR(i, 3) * PS(i + 1, j), r, L.ir[i]) -
                       div_by_rcp(PS(i, j), r * r, L.irr[i]);
            else
                temp = CRR(i, 1) * PS(i - 2, j) + CRR(i, 2) * PS(i - 1, j) + CRR(i, 3) * PS(i, j) +
                       CRR(i, 4) * PS(i + 1, j) + div_by_rcp(CR(i, 1) * PS(i - 1, j) + CR(i, 2) * PS(i, j) + CR(i, 3) * PS(i + 1, j), r, L.ir[i]) -
                       div_by_rcp(PS(i, j), r * r, L.irr[i]);
            if (j <= n2 / 2)
                temp = temp + CZZ(j, 1) * PS(i, j - 1) + CZZ(j, 2) * PS(i, j) + CZZ(j, 3) * PS(i, j + 1) +
                       CZZ(j, 4) * PS(i, j + 2);
            else
                temp = temp + CZZ(j, 1) * PS(i, j - 2) + CZZ(j, 2) * PS(i, j - 1) + CZZ(j, 3) * PS(i, j) +
                       CZZ(j, 4) * PS(i, j + 1);
            temp = L.f[(size_t)i + (size_t)(n1 + 1) * j] - temp;
            d.rc[(size_t)i + (size_t)d.ld * j] = temp;
            temp = fabs(temp);
            if (temp != temp) nan = 1;
            if (temp > m) m = temp;
        }
        nan = __syncthreads_or(nan);
        m = str_blk_max(m, s_red);
    }
    for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
        const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
        L.v[idx] = PS(i, j);
    }
    __syncthreads();
    *nan_out = nan;
    return m;
}

// corser (rcsc.f:1343-1390): restriction of rc into the packed coarse
// right-hand side; rows and columns 0 and n1c of the coarse level (n1 for
// both directions) are zero, as are the boundary rows the restriction does
// not reach (never read by the coarse relax); the coarse correction is zero.
__device__ void str_corser(const StrDev &d, int klev)
{
    const int ld = d.ld;
    const int n1c = d.lev[klev + 1].n1, n2c = d.lev[klev + 1].n2;
    const double *rf = d.rc;
    double *fc = d.lev[klev + 1].f, *vc = d.lev[klev + 1].v;
    const int tot = (n1c + 1) * (n2c + 1);
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int j = idx / (n1c + 1), i = idx - j * (n1c + 1);
        double temp = 0.0;
        if (i >= 1 && i <= n1c - 1 && j >= 1 && j <= n2c - 1 && j != n1c) {
            const int ii = i + i, jj = j + j;
            temp = rf[(size_t)ii + (size_t)ld * jj];
            temp = temp * 2.0 + rf[(size_t)(ii + 1) + (size_t)ld * jj] + rf[(size_t)(ii - 1) + (size_t)ld * jj];
            temp = temp + rf[(size_t)ii + (size_t)ld * (jj + 1)] + rf[(size_t)ii + (size_t)ld * (jj - 1)];
            temp = temp * 2.0 + rf[(size_t)(ii + 1) + (size_t)ld * (jj + 1)] + rf[(size_t)(ii - 1) + (size_t)ld * (jj - 1)];
            temp = temp + rf[(size_t)(ii + 1) + (size_t)ld * (jj - 1)] + rf[(size_t)(ii - 1) + (size_t)ld * (jj + 1)];
            temp = temp / 16.0;
        }
        fc[idx] = temp;
        vc[idx] = 0.0;
    }
    __syncthreads();
}

// finer (rcsc.f:1392-1444)
__device__ void str_finer(const StrDev &d, int klev)
{
    const int n1c = d.lev[klev].n1;
    const int n1f = d.lev[klev - 1].n1, n2f = d.lev[klev - 1].n2;
    const double *vc = d.lev[klev].v;
    double *vf = d.lev[klev - 1].v;
    const int tot = (n1f + 1) * (n2f + 1);
#define PC(ii, jj) vc[(size_t)(jj) * (n1c + 1) + (ii)]
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int j = idx / (n1f + 1), i = idx - j * (n1f + 1);
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
        PS(i, j) = p + vf[idx];
    }
#undef PC
    __syncthreads();
    const int tc = (n1c + 1) * (d.lev[klev].n2 + 1);
    for (int idx = threadIdx.x; idx < tc; idx += blockDim.x) d.lev[klev].v[idx] = 0.0;
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int j = idx / (n1f + 1), i = idx - j * (n1f + 1);
        vf[idx] = PS(i, j);
    }
    __syncthreads();
}

// poisson(psi, rhs, nlev, vel) (rcsc.f:1118-1195) on the staged arrays.
__global__ void __launch_bounds__(STR_THREADS) k_str_solve(const __grid_constant__ StrDev d)
{
    __shared__ double s_red[33];
    if (d.abort && *d.abort) return;   // uniform over the block
    const int nlev = d.nlev;
    const StrLevel &L1 = d.lev[1];
    const int n1 = L1.n1, n2 = L1.n2;
    const int tp = (n1 + 1) * (n2 + 1);
    for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
        L1.f[idx] = d.io_rhs[idx];
        L1.v[idx] = d.io_psi[idx];
    }
    for (int idx = threadIdx.x; idx < d.ld * d.ld; idx += blockDim.x) d.rc[idx] = 0.0;
    __syncthreads();
    int status = GB_MAXSWEEPS, sweeps = d.maxsweeps, nan1 = 0, nn = 0;
    double res1 = 0.0;
    for (int sweep = 1; sweep <= d.maxsweeps; ++sweep) {
        if (sweep == 1 || nlev == 1) res1 = str_relax(d, 1, s_red, &nan1);
        if (nlev > 1) {
            for (int l = 1; l <= nlev - 1; ++l) {
                str_corser(d, l);
                str_relax(d, l + 1, s_red, &nn);
            }
            for (int l = nlev; l >= 2; --l) {
                str_finer(d, l);
                const double r = str_relax(d, l - 1, s_red, &nn);
                if (l - 1 == 1) {
                    res1 = r;
                    nan1 = nn;
                }
            }
        }
        if (nan1) {
            status = GB_NAN;
            sweeps = sweep;
            break;
        }
        if (res1 < d.tolcon) {
            for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
                const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
                d.io_psi[idx] = PS(i, j);
            }
            status = GB_OK;
            sweeps = sweep;
            break;
        }
    }
    if (threadIdx.x == 0) {
        d.status[0] = status;
        d.status[1] = sweeps;
        if (status == GB_NAN && d.abort) *d.abort = 1;
    }
}

// ---------------------------------------------------------------------------
// Mixed precision (FP32 V-cycles inside FP64 defect correction): each outer
// iteration forms the FP64 residual r = f - L psi of the level-1 iterate
// (relax's own residual expression), stops when max |r| < tolcon, else runs
// one FP32 V-cycle of the same schedule on L e = r from e = 0 and updates
// psi += e in FP64 (rcsc.f's solve has no over-relaxation).  The FP32 line
// eliminations multiply by stored reciprocal pivots.
// ---------------------------------------------------------------------------
#define PS32(i, j) d.psif32[(size_t)(i) + (size_t)d.ld * (size_t)(j)]
#define CR32(i, k) L.cr32[3 * ((i) - 1) + (k) - 1]
#define CRR32(i, k) L.crr32[4 * ((i) - 1) + (k) - 1]
#define CZZ32(j, k) L.czz32[4 * ((j) - 1) + (k) - 1]

template <class Rhs>
__device__ inline void apply_pdma_rhs32(const float *fac, int n, float *x, int stride, Rhs rhs)
{
    const float *icdiv = fac, *bk1 = fac + n, *aa = fac + 2 * n, *dn = fac + 3 * n, *en = fac + 4 * n;
    const float icN = fac[5 * n];
    float rk = rhs(0);
    float rk1 = rhs(1);
#pragma unroll 4
    for (int k = 0; k <= n - 2; ++k) {
        rk = rk * icdiv[k];
        x[(size_t)k * stride] = rk;
        rk1 = rk1 - bk1[k] * rk;
        float rk2 = 0.f;
        if (k != n - 2) rk2 = rhs(k + 2) - aa[k + 2] * rk;
        rk = rk1;
        rk1 = rk2;
    }
    float x1 = rk * icN;
    x[(size_t)(n - 1) * stride] = x1;
    float x0 = x[(size_t)(n - 2) * stride] - dn[n - 2] * x1;
    x[(size_t)(n - 2) * stride] = x0;
#pragma unroll 4
    for (int j = n - 3; j >= 0; --j) {
        const float xj = x[(size_t)j * stride] - dn[j] * x0 - en[j] * x1;
        x[(size_t)j * stride] = xj;
        x1 = x0;
        x0 = xj;
    }
}

__device__ __forceinline__ void str_rline32(const StrDev &d, const StrLevel &L, int j)
{
    const int n1 = L.n1, n2 = L.n2;
    const float *f = L.f32;
    auto rhs = [&](int q) -> float {
        const int i = q + 1;
        if (j <= n2 / 2)
            return -(CZZ32(j, 1) * PS32(i, j - 1) + CZZ32(j, 3) * PS32(i, j + 1) + CZZ32(j, 4) * PS32(i, j + 2)) +
                   f[(size_t)i + (size_t)(n1 + 1) * j];
        return -(CZZ32(j, 1) * PS32(i, j - 2) + CZZ32(j, 2) * PS32(i, j - 1) + CZZ32(j, 4) * PS32(i, j + 1)) +
               f[(size_t)i + (size_t)(n1 + 1) * j];
    };
    const int n = n1 - 1;
    apply_pdma_rhs32(L.fac_r32 + (size_t)(j - 1) * (5 * n + 1), n, &PS32(1, j), 1, rhs);
}

__device__ __forceinline__ void str_zline32(const StrDev &d, const StrLevel &L, int i)
{
    const int n1 = L.n1, n2 = L.n2;
    const float *f = L.f32;
    const float ir = 1.0f / L.r32[i];
    auto rhs = [&](int q) -> float {
        const int j = q + 1;
        if (i <= n1 / 2)
            return -(CRR32(i, 1) * PS32(i - 1, j) + CRR32(i, 3) * PS32(i + 1, j) + CRR32(i, 4) * PS32(i + 2, j) +
                     (CR32(i, 1) * PS32(i - 1, j) + CR32(i, 3) * PS32(i + 1, j)) * ir) +
                   f[(size_t)i + (size_t)(n1 + 1) * j];
        return -(CRR32(i, 1) * PS32(i - 2, j) + CRR32(i, 2) * PS32(i - 1, j) + CRR32(i, 4) * PS32(i + 1, j) +
                 (CR32(i, 1) * PS32(i - 1, j) + CR32(i, 3) * PS32(i + 1, j)) * ir) +
               f[(size_t)i + (size_t)(n1 + 1) * j];
    };
    const int n = n2 - 1;
    apply_pdma_rhs32(L.fac_z32 + (size_t)(i - 1) * (5 * n + 1), n, &PS32(i, 1), d.ld, rhs);
}

__device__ __forceinline__ float str_rhs_r32(const StrDev &d, const StrLevel &L, int j, int i)
{
    const int n1 = L.n1, n2 = L.n2;
    const float *f = L.f32;
    if (j <= n2 / 2)
        return -(CZZ32(j, 1) * PS32(i, j - 1) + CZZ32(j, 3) * PS32(i, j + 1) + CZZ32(j, 4) * PS32(i, j + 2)) +
               f[(size_t)i + (size_t)(n1 + 1) * j];
    return -(CZZ32(j, 1) * PS32(i, j - 2) + CZZ32(j, 2) * PS32(i, j - 1) + CZZ32(j, 4) * PS32(i, j + 1)) +
           f[(size_t)i + (size_t)(n1 + 1) * j];
}

__device__ __forceinline__ float str_rhs_z32(const StrDev &d, const StrLevel &L, int i, int j)
{
    const int n1 = L.n1;
    const float *f = L.f32;
    const float ir = 1.0f / L.r32[i];
    if (i <= n1 / 2)
        return -(CRR32(i, 1) * PS32(i - 1, j) + CRR32(i, 3) * PS32(i + 1, j) + CRR32(i, 4) * PS32(i + 2, j) +
                 (CR32(i, 1) * PS32(i - 1, j) + CR32(i, 3) * PS32(i + 1, j)) * ir) +
               f[(size_t)i + (size_t)(n1 + 1) * j];
    return -(CRR32(i, 1) * PS32(i - 2, j) + CRR32(i, 2) * PS32(i - 1, j) + CRR32(i, 4) * PS32(i + 1, j) +
             (CR32(i, 1) * PS32(i - 1, j) + CR32(i, 3) * PS32(i + 1, j)) * ir) +
           f[(size_t)i + (size_t)(n1 + 1) * j];
}

// str_colour_smem in FP32 (the correction cycle).
template <int DIR>
__device__ void str_colour_smem32(const StrDev &d, const StrLevel &L, int first, float *sline)
{
    const int n1 = L.n1, n2 = L.n2;
    const int lines = DIR == 0 ? n2 - 1 : n1 - 1, n = DIR == 0 ? n1 - 1 : n2 - 1;
    if (first > lines) return;
    const int nl = (lines - first) / 4 + 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int B = (int)(STR_LINE_BYTES / sizeof(float)) / n - 1;
    if (B < 1) {
        for (int t = threadIdx.x; t < nl; t += blockDim.x) {
            if (DIR == 0) str_rline32(d, L, first + 4 * t);
            else str_zline32(d, L, first + 4 * t);
        }
        __syncthreads();
        return;
    }
    if (B > nl) B = nl;
    for (int b0 = 0; b0 < nl; b0 += B) {
        const int nb = min(B, nl - b0), pitch = nb | 1;
        if (DIR == 0) {
            for (int t = warp; t < nb; t += nw)
                for (int q = lane; q < n; q += 32) sline[q * pitch + t] = str_rhs_r32(d, L, first + 4 * (b0 + t), q + 1);
        } else {
            for (int q = warp; q < n; q += nw)
                for (int t = lane; t < nb; t += 32) sline[q * pitch + t] = str_rhs_z32(d, L, first + 4 * (b0 + t), q + 1);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < nb; t += blockDim.x) {
            const int line = first + 4 * (b0 + t);
            const float *fac = (DIR == 0 ? L.fac_r32 : L.fac_z32) + (size_t)(line - 1) * (5 * n + 1);
            pdma32_smem(fac, n, sline + t, pitch);
        }
        __syncthreads();
        if (DIR == 0) {
            for (int t = warp; t < nb; t += nw)
                for (int q = lane; q < n; q += 32) PS32(q + 1, first + 4 * (b0 + t)) = sline[q * pitch + t];
        } else {
            for (int q = warp; q < n; q += nw)
                for (int t = lane; t < nb; t += 32) PS32(first + 4 * (b0 + t), q + 1) = sline[q * pitch + t];
        }
        __syncthreads();
    }
}

// nrel sweeps of both line directions on level klev, then the residual of
// the correction into rc32 (for the restriction that follows).
__device__ void str_relax32(const StrDev &d, int klev)
{
    const StrLevel &L = d.lev[klev];
    const int n1 = L.n1, n2 = L.n2;
    const int tp = (n1 + 1) * (n2 + 1);
    for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
        const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
        PS32(i, j) = L.v32[idx];
    }
    __syncthreads();
    for (int irel = 0; irel < d.nrel; ++irel) {
        if (d.mode == GB_SMOOTHER_LEX) {
            if (threadIdx.x == 0) {
                for (int j = 1; j <= n2 - 1; ++j) str_rline32(d, L, j);
                for (int i = 1; i <= n1 - 1; ++i) str_zline32(d, L, i);
            }
            __syncthreads();
        } else {
            extern __shared__ float s_str_line32[];
            for (int c = 1; c <= 4; ++c) str_colour_smem32<0>(d, L, (c & 3) == 0 ? 4 : (c & 3), s_str_line32);
            for (int c = 1; c <= 4; ++c) str_colour_smem32<1>(d, L, (c & 3) == 0 ? 4 : (c & 3), s_str_line32);
        }
    }
    const int ni = n1 - 1, tot = ni * (n2 - 1);
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int j = idx / ni + 1, i = idx - (j - 1) * ni + 1;
        const float ir = 1.0f / L.r32[i];
        float temp;
        if (i <= n1 / 2)
            temp = CRR32(i, 1) * PS32(i - 1, j) + CRR32(i, 2) * PS32(i, j) + CRR32(i, 3) * PS32(i + 1, j) +
                   CRR32(i, 4) * PS32(i + 2, j) +
                   (CR32(i, 1) * PS32(i - 1, j) + CR32(i, 2) * PS32(i, j) + CR32(i, 3) * PS32(i + 1, j)) * ir -
                   PS32(i, j) * (ir * ir);
        else
            temp = CRR32(i, 1) * PS32(i - 2, j) + CRR32(i, 2) * PS32(i - 1, j) + CRR32(i, 3) * PS32(i, j) +
                   CRR32(i, 4) * PS32(i + 1, j) +
                   (CR32(i, 1) * PS32(i - 1, j) + CR32(i, 2) * PS32(i, j) + CR32(i, 3) * PS32(i + 1, j)) * ir -
                   PS32(i, j) * (ir * ir);
        if (j <= n2 / 2)
            temp = temp + CZZ32(j, 1) * PS32(i, j - 1) + CZZ32(j, 2) * PS32(i, j) + CZZ32(j, 3) * PS32(i, j + 1) +
                   CZZ32(j, 4) * PS32(i, j + 2);
        else
            temp = temp + CZZ32(j, 1) * PS32(i, j - 2) + CZZ32(j, 2) * PS32(i, j - 1) + CZZ32(j, 3) * PS32(i, j) +
                   CZZ32(j, 4) * PS32(i, j + 1);
        d.rc32[(size_t)i + (size_t)d.ld * j] = L.f32[(size_t)i + (size_t)(n1 + 1) * j] - temp;
    }
    for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
        const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
        L.v32[idx] = PS32(i, j);
    }
    __syncthreads();
}

// corser (rcsc.f:1343-1390) in FP32, with its clearing of rows and columns 0
// and n1c in both directions
__device__ void str_corser32(const StrDev &d, int klev)
{
    const int ld = d.ld;
    const int n1c = d.lev[klev + 1].n1, n2c = d.lev[klev + 1].n2;
    const float *rf = d.rc32;
    float *fc = d.lev[klev + 1].f32, *vc = d.lev[klev + 1].v32;
    const int tot = (n1c + 1) * (n2c + 1);
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int j = idx / (n1c + 1), i = idx - j * (n1c + 1);
        float temp = 0.f;
        if (i >= 1 && i <= n1c - 1 && j >= 1 && j <= n2c - 1 && j != n1c) {
            const int ii = i + i, jj = j + j;
            temp = rf[(size_t)ii + (size_t)ld * jj];
            temp = temp * 2.f + rf[(size_t)(ii + 1) + (size_t)ld * jj] + rf[(size_t)(ii - 1) + (size_t)ld * jj];
            temp = temp + rf[(size_t)ii + (size_t)ld * (jj + 1)] + rf[(size_t)ii + (size_t)ld * (jj - 1)];
            temp = temp * 2.f + rf[(size_t)(ii + 1) + (size_t)ld * (jj + 1)] + rf[(size_t)(ii - 1) + (size_t)ld * (jj - 1)];
            temp = temp + rf[(size_t)(ii + 1) + (size_t)ld * (jj - 1)] + rf[(size_t)(ii - 1) + (size_t)ld * (jj + 1)];
            temp = temp * 0.0625f;
        }
        fc[idx] = temp;
        vc[idx] = 0.f;
    }
    __syncthreads();
}

// finer (rcsc.f:1392-1444) in FP32
__device__ void str_finer32(const StrDev &d, int klev)
{
    const int n1c = d.lev[klev].n1;
    const int n1f = d.lev[klev - 1].n1, n2f = d.lev[klev - 1].n2;
    const float *vc = d.lev[klev].v32;
    float *vf = d.lev[klev - 1].v32;
    const int tot = (n1f + 1) * (n2f + 1);
#define PC32(ii, jj) vc[(size_t)(jj) * (n1c + 1) + (ii)]
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int j = idx / (n1f + 1), i = idx - j * (n1f + 1);
        const int i1 = i / 2, j1 = j / 2;
        float p;
        if (i1 * 2 == i) p = (j1 * 2 == j) ? PC32(i1, j1) : (PC32(i1, j1) + PC32(i1, j1 + 1)) * 0.5f;
        else if (j1 * 2 == j) p = (PC32(i1, j1) + PC32(i1 + 1, j1)) * 0.5f;
        else p = (PC32(i1, j1) + PC32(i1 + 1, j1 + 1) + PC32(i1, j1 + 1) + PC32(i1 + 1, j1)) * 0.25f;
        PS32(i, j) = p + vf[idx];
    }
#undef PC32
    __syncthreads();
    const int tc = (n1c + 1) * (d.lev[klev].n2 + 1);
    for (int idx = threadIdx.x; idx < tc; idx += blockDim.x) d.lev[klev].v32[idx] = 0.f;
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int j = idx / (n1f + 1), i = idx - j * (n1f + 1);
        vf[idx] = PS32(i, j);
    }
    __syncthreads();
}

// FP64 residual of level 1 (relax's expression, rcsc.f:1300-1330)
__device__ __forceinline__ double str_resid64(const StrDev &d, const StrLevel &L, int i, int j)
{
    const int n1 = L.n1, n2 = L.n2;
    const double r = L.r[i];
    double temp;
    if (i <= n1 / 2)
        temp = CRR(i, 1) * PS(i - 1, j) + CRR(i, 2) * PS(i, j) + CRR(i, 3) * PS(i + 1, j) + CRR(i, 4) * PS(i + 2, j) +
               div_by_rcp(CR(i, 1) * PS(i - 1, j) + CR(i, 2) * PS(i, j) + CR(i, 3) * PS(i + 1, j), r, L.ir[i]) - div_by_rcp(PS(i, j), r * r, L.irr[i]);
    else
        temp = CRR(i, 1) * PS(i - 2, j) + CRR(i, 2) * PS(i - 1, j) + CRR(i, 3) * PS(i, j) + CRR(i, 4) * PS(i + 1, j) +
               div_by_rcp(CR(i, 1) * PS(i - 1, j) + CR(i, 2) * PS(i, j) + CR(i, 3) * PS(i + 1, j), r, L.ir[i]) - div_by_rcp(PS(i, j), r * r, L.irr[i]);
    if (j <= n2 / 2)
        temp = temp + CZZ(j, 1) * PS(i, j - 1) + CZZ(j, 2) * PS(i, j) + CZZ(j, 3) * PS(i, j + 1) + CZZ(j, 4) * PS(i, j + 2);
    else
        temp = temp + CZZ(j, 1) * PS(i, j - 2) + CZZ(j, 2) * PS(i, j - 1) + CZZ(j, 3) * PS(i, j) + CZZ(j, 4) * PS(i, j + 1);
    return L.f[(size_t)i + (size_t)(n1 + 1) * j] - temp;
}

__global__ void __launch_bounds__(STR_THREADS) k_str_solve_mixed(const __grid_constant__ StrDev d)
{
    __shared__ double s_red[33];
    if (d.abort && *d.abort) return;
    const int nlev = d.nlev;
    const StrLevel &L1 = d.lev[1];
    const int n1 = L1.n1, n2 = L1.n2;
    const int tp = (n1 + 1) * (n2 + 1);
    for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
        const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
        L1.f[idx] = d.io_rhs[idx];
        PS(i, j) = d.io_psi[idx];
        L1.f32[idx] = 0.f;
    }
    for (int idx = threadIdx.x; idx < d.ld * d.ld; idx += blockDim.x) d.rc32[idx] = 0.f;
    __syncthreads();
    const int ni = n1 - 1, tot = ni * (n2 - 1);
    int status = GB_MAXSWEEPS, cycles = 0;
    for (int it = 0;; ++it) {
        double m = 0.0;
        int nan = 0;
        for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
            const int j = idx / ni + 1, i = idx - (j - 1) * ni + 1;
            const double rr = str_resid64(d, L1, i, j);
            L1.f32[(size_t)i + (size_t)(n1 + 1) * j] = (float)rr;
            const double a = fabs(rr);
            if (a != a) nan = 1;
            if (a > m) m = a;
        }
        nan = __syncthreads_or(nan);
        const double res = str_blk_max(m, s_red);
        if (nan) { status = GB_NAN; break; }
        if (res < d.tolcon) { status = GB_OK; break; }
        if (it == d.maxsweeps) break;
        for (int q = threadIdx.x; q < tp; q += blockDim.x) L1.v32[q] = 0.f;
        __syncthreads();
        str_relax32(d, 1);
        if (nlev > 1) {
            for (int l = 1; l <= nlev - 1; ++l) {
                str_corser32(d, l);
                str_relax32(d, l + 1);
            }
            for (int l = nlev; l >= 2; --l) {
                str_finer32(d, l);
                str_relax32(d, l - 1);
            }
        }
        for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
            const int j = idx / ni + 1, i = idx - (j - 1) * ni + 1;
            PS(i, j) += (double)L1.v32[(size_t)i + (size_t)(n1 + 1) * j];
        }
        __syncthreads();
        cycles = it + 1;
    }
    if (status == GB_OK)
        for (int idx = threadIdx.x; idx < tp; idx += blockDim.x) {
            const int j = idx / (n1 + 1), i = idx - j * (n1 + 1);
            d.io_psi[idx] = PS(i, j);
        }
    if (threadIdx.x == 0) {
        d.status[0] = status;
        d.status[1] = cycles;
        if (status == GB_NAN && d.abort) *d.abort = 1;
    }
}

// FP32 copies of a level's tables and factors (pivots as reciprocals), one
// thread per level.
__global__ void k_str_factors32(const __grid_constant__ StrDev d)
{
    const int l = 1 + blockIdx.x;
    if (threadIdx.x != 0 || l > d.nlev) return;
    const StrLevel &L = d.lev[l];
    const int a = L.n1, b = L.n2;
    for (int i = 0; i <= a; ++i) L.r32[i] = (float)L.r[i];
    for (int q = 0; q < 3 * (a - 1); ++q) L.cr32[q] = (float)L.cr[q];
    for (int q = 0; q < 4 * (a - 1); ++q) L.crr32[q] = (float)L.crr[q];
    for (int q = 0; q < 4 * (b - 1); ++q) L.czz32[q] = (float)L.czz[q];
    auto conv = [](const double *fac, float *g, int n) {
        for (int k = 0; k < n; ++k) g[k] = (float)(1.0 / fac[k]);   // cdiv as reciprocals
        for (int k = n; k < 5 * n; ++k) g[k] = (float)fac[k];
        g[5 * n] = (float)(1.0 / fac[5 * n]);
    };
    const int nr = a - 1, nz = b - 1;
    for (int j = 1; j <= b - 1; ++j)
        conv(L.fac_r + (size_t)(j - 1) * pdma_fac_len(nr), L.fac_r32 + (size_t)(j - 1) * (5 * nr + 1), nr);
    for (int i = 1; i <= a - 1; ++i)
        conv(L.fac_z + (size_t)(i - 1) * pdma_fac_len(nz), L.fac_z32 + (size_t)(i - 1) * (5 * nz + 1), nz);
}

#undef PS32
#undef CR32
#undef CRR32
#undef CZZ32
#undef PS
#undef CR
#undef CRR
#undef CZZ

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct gb_str {
    StrDev dev;
    double *pool = nullptr;
    int *status = nullptr;
    cudaStream_t stream = nullptr;
};

extern "C" int gb_str_destroy(gb_str *h)
{
    if (!h) return GB_OK;
    cudaFree(h->pool);
    cudaFree(h->status);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return GB_OK;
}

extern "C" int gb_str_create(int nlev, const gb_str_level *lv, double tolcon, int maxsweeps, int nrel, int smoother,
                             gb_str **out)
{
    if (!out || !lv || nlev < 1 || nlev >= STR_MAXLEV || maxsweeps < 1 || nrel < 1 ||
        (smoother != GB_SMOOTHER_LEX && smoother != GB_SMOOTHER_ZEBRA)) {
        gb_set_error("gb_str_create: invalid argument");
        return GB_ERR_INVALID;
    }
    *out = nullptr;
    const int n1 = lv[0].n1, n2 = lv[0].n2;
    if (n1 < 4 || n2 < 4 || n1 > 8192 || n2 > 8192) {
        gb_set_error("gb_str_create: level-1 grid %d x %d unsupported", n1, n2);
        return GB_ERR_INVALID;
    }
    for (int l = 0; l < nlev; ++l) {
        if (lv[l].n1 != (n1 >> l) || lv[l].n2 != (n2 >> l) || (l && (lv[l - 1].n1 & 1 || lv[l - 1].n2 & 1)) ||
            lv[l].n1 < 4 || lv[l].n2 < 4 || !lv[l].r || !lv[l].cr || !lv[l].crr || !lv[l].czz) {
            gb_set_error("gb_str_create: level %d must be %d x %d (halvings of level 1, >= 4) with all tables", l + 1,
                         n1 >> l, n2 >> l);
            return GB_ERR_INVALID;
        }
    }
    gb_str *h = new gb_str();
    StrDev &d = h->dev;
    memset(&d, 0, sizeof(d));
    d.nlev = nlev;
    d.ld = std::max(n1, n2) + 1;
    d.nrel = nrel;
    d.maxsweeps = maxsweeps;
    d.mode = smoother;
    d.tolcon = tolcon;
    size_t need = 2 * (size_t)d.ld * d.ld + 2 * (size_t)(n1 + 1) * (n2 + 1);
    for (int l = 0; l < nlev; ++l) {
        const size_t a = lv[l].n1, b = lv[l].n2;
        need += 3 * (a + 1) + 3 * (a - 1) + 4 * (a - 1) + 4 * (b - 1) + 2 * (a + 1) * (b + 1);
        need += (b - 1) * pdma_fac_len((int)a - 1) + (a - 1) * pdma_fac_len((int)b - 1);
    }
    // FP32 copies: psif32, rc32 and every level's tables (half a double each, rounded up per array)
    size_t need32 = 2 * (size_t)d.ld * d.ld + 16;
    for (int l = 0; l < nlev; ++l) {
        const size_t a = lv[l].n1, b = lv[l].n2;
        need32 += (a + 1) + 3 * (a - 1) + 4 * (a - 1) + 4 * (b - 1) + 2 * (a + 1) * (b + 1);
        need32 += (b - 1) * (5 * (a - 1) + 1) + (a - 1) * (5 * (b - 1) + 1) + 16;
    }
    const size_t need64 = need;
    need += (need32 + 1) / 2;
    cudaError_t e = cudaMalloc(&h->pool, sizeof(double) * need);
    if (e != cudaSuccess) { delete h; gb_set_error("gb_str_create: %s", cudaGetErrorString(e)); return GB_ERR_ALLOC; }
    cudaMemset(h->pool, 0, sizeof(double) * need);
    double *b = h->pool;
    d.psif = b; b += (size_t)d.ld * d.ld;
    d.rc = b; b += (size_t)d.ld * d.ld;
    d.io_psi = b; b += (size_t)(n1 + 1) * (n2 + 1);
    d.io_rhs = b; b += (size_t)(n1 + 1) * (n2 + 1);
    std::vector<StrJob> jobs;
    int wmax = 0;
    for (int l = 0; l < nlev; ++l) {
        StrLevel &L = d.lev[l + 1];
        const int a = lv[l].n1, bb = lv[l].n2;
        L.n1 = a;
        L.n2 = bb;
        L.r = b; b += a + 1;
        L.ir = b; b += a + 1;
        L.irr = b; b += a + 1;
        L.cr = b; b += 3 * (size_t)(a - 1);
        L.crr = b; b += 4 * (size_t)(a - 1);
        L.czz = b; b += 4 * (size_t)(bb - 1);
        L.v = b; b += (size_t)(a + 1) * (bb + 1);
        L.f = b; b += (size_t)(a + 1) * (bb + 1);
        L.fac_r = b; b += (size_t)(bb - 1) * pdma_fac_len((int)a - 1);
        L.fac_z = b; b += (size_t)(a - 1) * pdma_fac_len((int)bb - 1);
        cudaMemcpy(L.r, lv[l].r, sizeof(double) * (a + 1), cudaMemcpyHostToDevice);
        {
            std::vector<double> inv(2 * (size_t)(a + 1));
            for (int i = 0; i <= a; ++i) {
                const double r = lv[l].r[i];
                inv[i] = 1.0 / r;
                inv[a + 1 + i] = 1.0 / (r * r);
            }
            cudaMemcpy(L.ir, inv.data(), sizeof(double) * inv.size(), cudaMemcpyHostToDevice);
        }
        cudaMemcpy(L.cr, lv[l].cr, sizeof(double) * 3 * (a - 1), cudaMemcpyHostToDevice);
        cudaMemcpy(L.crr, lv[l].crr, sizeof(double) * 4 * (a - 1), cudaMemcpyHostToDevice);
        cudaMemcpy(L.czz, lv[l].czz, sizeof(double) * 4 * (bb - 1), cudaMemcpyHostToDevice);
        for (int j = 1; j <= bb - 1; ++j) jobs.push_back({l + 1, 0, j});
        for (int i = 1; i <= a - 1; ++i) jobs.push_back({l + 1, 1, i});
        wmax = std::max(wmax, std::max(a, bb));
    }
    if ((size_t)(b - h->pool) != need64) {
        gb_str_destroy(h);
        gb_set_error("gb_str_create: pool layout mismatch");
        return GB_ERR_CUDA;
    }
    {
        float *fb = (float *)b;
        float *fend = (float *)(h->pool + need);
        d.psif32 = fb; fb += (size_t)d.ld * d.ld;
        d.rc32 = fb; fb += (size_t)d.ld * d.ld;
        for (int l = 1; l <= nlev; ++l) {
            StrLevel &L = d.lev[l];
            const size_t a = L.n1, bb = L.n2;
            L.r32 = fb; fb += a + 1;
            L.cr32 = fb; fb += 3 * (a - 1);
            L.crr32 = fb; fb += 4 * (a - 1);
            L.czz32 = fb; fb += 4 * (bb - 1);
            L.v32 = fb; fb += (a + 1) * (bb + 1);
            L.f32 = fb; fb += (a + 1) * (bb + 1);
            L.fac_r32 = fb; fb += (bb - 1) * (5 * (a - 1) + 1);
            L.fac_z32 = fb; fb += (a - 1) * (5 * (bb - 1) + 1);
        }
        if (fb > fend) {
            gb_str_destroy(h);
            gb_set_error("gb_str_create: FP32 pool layout overflow");
            return GB_ERR_CUDA;
        }
    }
    const int wstride = 7 * wmax;
    StrJob *djobs = nullptr;
    double *work = nullptr;
    e = cudaMalloc(&djobs, sizeof(StrJob) * jobs.size());
    if (e == cudaSuccess) e = cudaMalloc(&work, sizeof(double) * (size_t)wstride * jobs.size());
    if (e != cudaSuccess) {
        cudaFree(djobs);
        gb_str_destroy(h);
        gb_set_error("gb_str_create: factor scratch");
        return GB_ERR_ALLOC;
    }
    cudaMemcpy(djobs, jobs.data(), sizeof(StrJob) * jobs.size(), cudaMemcpyHostToDevice);
    k_str_factors<<<gb_ceil_div(jobs.size(), 64), 64>>>(d, djobs, (int)jobs.size(), work, wstride);
    e = cudaDeviceSynchronize();
    cudaFree(djobs);
    cudaFree(work);
    if (e == cudaSuccess) {
        k_str_factors32<<<nlev, 32>>>(d);
        e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) { gb_set_error("gb_str_create: factors: %s", cudaGetErrorString(e)); gb_str_destroy(h); return GB_ERR_CUDA; }
    e = cudaMalloc(&h->status, 64);
    if (e != cudaSuccess) { gb_str_destroy(h); gb_set_error("gb_str_create: status"); return GB_ERR_ALLOC; }
    d.status = h->status;
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { gb_str_destroy(h); gb_set_error("gb_str_create: stream"); return GB_ERR_CUDA; }
    e = cudaFuncSetAttribute(k_str_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, STR_LINE_BYTES);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_str_solve_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, STR_LINE_BYTES);
    if (e != cudaSuccess) { gb_str_destroy(h); gb_set_error("gb_str_create: shared memory: %s", cudaGetErrorString(e)); return GB_ERR_CUDA; }
    *out = h;
    return GB_OK;
}

// The solve on device arrays (0:n1, 0:n2) with leading dimension n1 + 1,
// queued on stream s with the given tolerance, sweep limit, relaxation count
// and line order: psi is read and, on convergence, written in place; the
// status and sweep (mixed: outer iteration) count go to status[0..1]; abort
// as in StrDev.  mixed != 0 runs the FP32-inner / FP64-outer solve.
cudaError_t gb_str_launch_device(const gb_str *h, double *psi, const double *rhs, int *status, int *abort, int mixed,
                                 double tolcon, int maxsweeps, int nrel, int mode, cudaStream_t s)
{
    StrDev d = h->dev;
    d.tolcon = tolcon;
    d.maxsweeps = maxsweeps;
    d.nrel = nrel;
    d.mode = mode;
    d.io_psi = psi;
    d.io_rhs = const_cast<double *>(rhs);
    d.status = status;
    d.abort = abort;
    if (mixed) k_str_solve_mixed<<<1, STR_THREADS, STR_LINE_BYTES, s>>>(d);
    else k_str_solve<<<1, STR_THREADS, STR_LINE_BYTES, s>>>(d);
    return cudaGetLastError();
}

extern "C" int gb_str_poisson(gb_str *h, double *psi, const double *rhs, int ld, int *sweeps)
{
    if (!h || !psi || !rhs) { gb_set_error("gb_str_poisson: null argument"); return GB_ERR_INVALID; }
    const StrDev &d = h->dev;
    const int n1 = d.lev[1].n1, n2 = d.lev[1].n2;
    if (ld < n1 + 1) { gb_set_error("gb_str_poisson: ld %d < n1+1", ld); return GB_ERR_INVALID; }
    const size_t row = sizeof(double) * (size_t)(n1 + 1);
    GB_CUDA_TRY(cudaMemcpy2DAsync(d.io_psi, row, psi, sizeof(double) * (size_t)ld, row, n2 + 1, cudaMemcpyHostToDevice,
                                  h->stream));
    GB_CUDA_TRY(cudaMemcpy2DAsync(d.io_rhs, row, rhs, sizeof(double) * (size_t)ld, row, n2 + 1, cudaMemcpyHostToDevice,
                                  h->stream));
    k_str_solve<<<1, STR_THREADS, STR_LINE_BYTES, h->stream>>>(d);
    GB_CUDA_TRY(cudaGetLastError());
    int st[2] = {0, 0};
    GB_CUDA_TRY(cudaMemcpyAsync(st, d.status, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    GB_CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (st[0] == GB_OK)
        GB_CUDA_TRY(cudaMemcpy2D(psi, sizeof(double) * (size_t)ld, d.io_psi, row, row, n2 + 1, cudaMemcpyDeviceToHost));
    if (sweeps) *sweeps = st[1];
    return st[0];
}
