// Batched Dirichlet Poisson solver: many independent n x n vertex-grid
// problems of uneven size, V(nu1,nu2) red-black Gauss-Seidel cycles with
// full-weighting restriction and bilinear prolongation (the transfer
// operators of rotann2.f:755-854), in plain FP64 or as an FP32 inner
// V-cycle inside FP64 defect correction.
//
// Execution: every level of every problem larger than LOCAL_N is processed
// by level-synchronous kernels whose blocks are drawn from one table over
// all problems (a block never spans two problems); the remaining coarse
// levels of each problem (n <= LOCAL_N) are solved by one thread block per
// problem entirely in shared memory.  Converged problems drop out: every
// block of an inactive problem returns at once.
//
// Numerics: explicit __fma_rn/__fmaf_rn where the oracle calls fma/fmaf and
// no other contraction (-fmad=false).  The multiplications by h^2, 1/h^2,
// 0.25 and 0.0625 are by powers of two, so each stencil rounds exactly as
// its unfused form; results match the CPU oracle bit for bit except for the
// order of the norm reductions.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "gbcommon.cuh"

#define BP_MAXL 16
#define LOCAL_N 65
#define BP_THREADS 256

template <class T> __device__ __forceinline__ T fmaT(T a, T b, T c);
template <> __device__ __forceinline__ double fmaT<double>(double a, double b, double c) { return __fma_rn(a, b, c); }
template <> __device__ __forceinline__ float fmaT<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }

struct TileEntry {
    int p;            // problem
    short tx, ty;     // tile index (origin tx*TX, ty*TY in grid points)
};

struct BatchDev {
    int nprob;
    const int *n_of;          // [p*BP_MAXL + l] level sizes (0 past the last level)
    const int *nlev;          // [p]
    const int *dloc;          // [p] first level solved locally
    void *const *x;           // [(slot*nprob + p)*BP_MAXL + l] the two buffers of level l's solution (T*)
    void *const *f;           // right-hand side of level l (T*)
    void *const *r;           // unused
    int *active;              // [p]
    int *cycles;              // [p]
    int *failed;              // [p]
    double *fnorm, *relres;   // [p]
    double *partial;          // per level-0 block
    const int *p_blk0, *p_nblk0;  // level-0 table range of each problem
    double *const *psi;       // [p] the caller's FP64 solution of level 0
    int *num_active;
    int max_cycles;
    int inner;                // V-cycles per outer iteration (defect correction)
    double rtol;
};

template <class T> __device__ __forceinline__ T *XS(const BatchDev &B, int p, int l, int slot)
{
    return (T *)B.x[((size_t)slot * B.nprob + p) * BP_MAXL + l];
}
template <class T> __device__ __forceinline__ T *FP(const BatchDev &B, int p, int l) { return (T *)B.f[p * BP_MAXL + l]; }
template <class T> __device__ __forceinline__ T *RP(const BatchDev &B, int p, int l) { return (T *)B.r[p * BP_MAXL + l]; }

// ---------------------------------------------------------------------------
// Level-synchronous tile kernels (one table entry per block)
//
// A fine tile is TX x TY grid points with origin (tx*TX, ty*TY); a block
// stages the tile plus a halo of H = 2*NU points in shared memory and runs
// NU red-black sweeps there: sweep s updates red on ring H-1-2s and black
// on ring H-2-2s, so after NU sweeps the tile itself is exact.  Points on
// the Dirichlet boundary or outside the grid are never updated.
// ---------------------------------------------------------------------------
#define TX 128
#define TY 32
#define CX 64    // coarse tile of the restriction kernel (fine 128 x 32)
#define CY 16
#define TILE_THREADS 256

// One red (color 0) or black (color 1) phase on ring rho around the tile.
// The smem array has origin (ox, oy) in grid coordinates and row stride SX.
template <class T>
__device__ __forceinline__ void tile_phase(T *sx, const T *sf, int SX, int ox, int oy, int x0, int y0, int n,
                                           T h2, int rho, int color)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int gxa = max(x0 - rho, 1), gxb = min(x0 + TX + rho, n - 1);
    const int gya = max(y0 - rho, 1), gyb = min(y0 + TY + rho, n - 1);
    for (int gy = gya + warp; gy < gyb; gy += nw) {
        const int base = (gy - oy) * SX - ox;
        const int first = gxa + ((gxa + gy + color) & 1);
        for (int gx = first + 2 * lane; gx < gxb; gx += 64) {
            const int c = base + gx;
            const T s = (sx[c - 1] + sx[c + 1]) + (sx[c - SX] + sx[c + SX]);
            sx[c] = fmaT<T>(-h2, sf[c], s) * (T)0.25;
        }
    }
    __syncthreads();
}

template <class T>
__device__ __forceinline__ void tile_sweeps(T *sx, const T *sf, int SX, int ox, int oy, int x0, int y0, int n,
                                            int nu, int H)
{
    const T h = (T)1 / (T)(n - 1), h2 = h * h;
    for (int s = 0; s < nu; ++s) {
        tile_phase<T>(sx, sf, SX, ox, oy, x0, y0, n, h2, H - 1 - 2 * s, 0);
        tile_phase<T>(sx, sf, SX, ox, oy, x0, y0, n, h2, H - 2 - 2 * s, 1);
    }
}

// Stores the tile's interior points into x, or (psi != nullptr) adds them to
// the FP64 solution instead: the last level-0 kernel of an inner cycle
// applies the defect correction psi += e point by point.
template <class T, bool CORRECT>
__device__ __forceinline__ void tile_store(const T *sx, int SX, int ox, int oy, int x0, int y0, int n, T *x,
                                           double *psi)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int gxa = max(x0, 1), gxb = min(x0 + TX, n - 1);
    const int gya = max(y0, 1), gyb = min(y0 + TY, n - 1);
    for (int gy = gya + warp; gy < gyb; gy += nw)
        for (int gx = gxa + lane; gx < gxb; gx += 32) {
            const size_t g = (size_t)gy * n + gx;
            const T v = sx[(gy - oy) * SX + gx - ox];
            if (CORRECT) psi[g] = psi[g] + (double)v;
            else x[g] = v;
        }
}

// NU smoothing sweeps of level l from buffer src into buffer dst (never the
// same buffer: blocks read their neighbours' tiles as halo).  zero_init: the
// level's current solution is zero (the correction of a coarse level, or the
// FP32 correction of the defect-correction loop) and is not read.  correct:
// add the result to the FP64 solution instead of storing it (level 0).
template <class T, int NU, bool CORR>
__global__ void __launch_bounds__(TILE_THREADS) k_smooth(BatchDev B, const TileEntry *tiles, int l, int zero_init,
                                                         int src, int dst)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int H = 2 * NU, SX = TX + 2 * H, SY = TY + 2 * H;
    T *sx = (T *)smem_raw, *sf = sx + SX * SY;
    const TileEntry e = tiles[blockIdx.x];
    if (!B.active[e.p]) return;
    const int n = B.n_of[e.p * BP_MAXL + l];
    const int x0 = e.tx * TX, y0 = e.ty * TY, ox = x0 - H, oy = y0 - H;
    const T *x = XS<T>(B, e.p, l, src);
    const T *f = FP<T>(B, e.p, l);
#pragma unroll 4
    for (int i = threadIdx.x; i < SX * SY; i += TILE_THREADS) {
        const int r = i / SX, c = i - r * SX;
        const int gy = oy + r, gx = ox + c;
        T v = (T)0, fv = (T)0;
        if (gy >= 0 && gy < n && gx >= 0 && gx < n) {
            const size_t g = (size_t)gy * n + gx;
            fv = f[g];
            if (!zero_init) v = x[g];
        }
        sx[i] = v;
        sf[i] = fv;
    }
    __syncthreads();
    tile_sweeps<T>(sx, sf, SX, ox, oy, x0, y0, n, NU, H);
    tile_store<T, CORR>(sx, SX, ox, oy, x0, y0, n, XS<T>(B, e.p, l, dst), CORR ? B.psi[e.p] : nullptr);
}

// Bilinear prolongation of level l+1 (buffer csrc) added into level l
// (buffer src) over the tile and its halo (rotann2.f:821-858), then NU
// post-smoothing sweeps, stored into buffer dst (or added to psi: correct).
template <class T, int NU, bool CORR>
__global__ void __launch_bounds__(TILE_THREADS) k_prolong_smooth(BatchDev B, const TileEntry *tiles, int l, int src,
                                                                 int csrc, int dst)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int H = 2 * NU, SX = TX + 2 * H, SY = TY + 2 * H;
    T *sx = (T *)smem_raw, *sf = sx + SX * SY;
    const TileEntry e = tiles[blockIdx.x];
    if (!B.active[e.p]) return;
    const int n = B.n_of[e.p * BP_MAXL + l], nc = B.n_of[e.p * BP_MAXL + l + 1];
    const int x0 = e.tx * TX, y0 = e.ty * TY, ox = x0 - H, oy = y0 - H;
    const T *x = XS<T>(B, e.p, l, src);
    const T *f = FP<T>(B, e.p, l);
    const T *ec = XS<T>(B, e.p, l + 1, csrc);
#pragma unroll 4
    for (int i = threadIdx.x; i < SX * SY; i += TILE_THREADS) {
        const int r = i / SX, c = i - r * SX;
        const int gy = oy + r, gx = ox + c;
        {
            T v = (T)0, fv = (T)0;
            if (gy >= 0 && gy < n && gx >= 0 && gx < n) {
                const size_t g = (size_t)gy * n + gx;
                v = x[g];
                if (NU > 0) fv = f[g];
                if (gx >= 1 && gx <= n - 2 && gy >= 1 && gy <= n - 2) {
                    const T *ep = ec + (size_t)(gy / 2) * nc + (gx / 2);
                    T p;
                    if ((gx & 1) == 0) {
                        if ((gy & 1) == 0) p = ep[0];
                        else p = (ep[0] + ep[nc]) * (T)0.5;
                    } else {
                        if ((gy & 1) == 0) p = (ep[0] + ep[1]) * (T)0.5;
                        else {
                            T t = ep[0] + ep[nc + 1];
                            t = t + ep[nc] + ep[1];
                            p = t * (T)0.25;
                        }
                    }
                    v = v + p;
                }
            }
            sx[i] = v;
            if (NU > 0) sf[i] = fv;
        }
    }
    __syncthreads();
    if (NU > 0) tile_sweeps<T>(sx, sf, SX, ox, oy, x0, y0, n, NU, H);
    tile_store<T, CORR>(sx, SX, ox, oy, x0, y0, n, XS<T>(B, e.p, l, dst), CORR ? B.psi[e.p] : nullptr);
}

// Residual of level l and its full weighting onto level l+1 (rotann2.f:
// 773-785 summation order) for one CX x CY tile of coarse points.
template <class T>
__global__ void __launch_bounds__(TILE_THREADS) k_resid_restrict(BatchDev B, const TileEntry *ctiles, int l, int src)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int FW = 2 * CX + 1, FH = 2 * CY + 1, XW = FW + 2, XH = FH + 2;
    T *sx = (T *)smem_raw, *sr = sx + XW * XH;
    const TileEntry e = ctiles[blockIdx.x];
    if (!B.active[e.p]) return;
    const int n = B.n_of[e.p * BP_MAXL + l], nc = B.n_of[e.p * BP_MAXL + l + 1];
    const int X0 = e.tx * CX, Y0 = e.ty * CY;
    const int rx = 2 * X0 - 1, ry = 2 * Y0 - 1;     // residual region origin
    const T *x = XS<T>(B, e.p, l, src);
    const T *f = FP<T>(B, e.p, l);
    T *fc = FP<T>(B, e.p, l + 1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll 4
    for (int i = threadIdx.x; i < XW * XH; i += TILE_THREADS) {
        const int r = i / XW, c = i - r * XW;
        const int gy = ry - 1 + r, gx = rx - 1 + c;
        sx[i] = (gy >= 0 && gy < n && gx >= 0 && gx < n) ? x[(size_t)gy * n + gx] : (T)0;
    }
    __syncthreads();
    const T h = (T)1 / (T)(n - 1), ih2 = (T)1 / (h * h);
    for (int r = warp; r < FH; r += nw) {
        const int gy = ry + r;
        for (int c = lane; c < FW; c += 32) {
            const int gx = rx + c;
            T rv = (T)0;
            if (gx >= 1 && gx <= n - 2 && gy >= 1 && gy <= n - 2) {
                const int q = (r + 1) * XW + (c + 1);
                const T s = (sx[q - 1] + sx[q + 1]) + (sx[q - XW] + sx[q + XW]);
                const T lap = fmaT<T>((T)-4, sx[q], s);
                rv = fmaT<T>(-ih2, lap, f[(size_t)gy * n + gx]);
            }
            sr[r * FW + c] = rv;
        }
    }
    __syncthreads();
    const int Ia = max(X0, 1), Ib = min(X0 + CX, nc - 1);
    const int Ja = max(Y0, 1), Jb = min(Y0 + CY, nc - 1);
    for (int J = Ja + warp; J < Jb; J += nw) {
        for (int I = Ia + lane; I < Ib; I += 32) {
            const int q = (2 * (J - Y0) + 1) * FW + (2 * (I - X0) + 1);
            T t = sr[q];
            t = t * (T)2 + sr[q + 1] + sr[q - 1];
            t = t + sr[q + FW] + sr[q - FW];
            t = t * (T)2 + sr[q + 1 + FW] + sr[q - 1 - FW];
            t = t + sr[q + 1 - FW] + sr[q - 1 + FW];
            fc[(size_t)J * nc + I] = t * (T)0.0625;
        }
    }
}

// ---------------------------------------------------------------------------
// Coarse levels of one problem in shared memory (one block per problem).
// ---------------------------------------------------------------------------
template <class T>
__device__ void loc_rb_half(T *x, const T *f, int n, T h2, int color)
{
    const int m = n - 2;
    for (int q = threadIdx.x; q < m * m; q += blockDim.x) {
        const int j = q / m + 1, i = q - (j - 1) * m + 1;
        if (((i + j) & 1) != color) continue;
        const int c = j * n + i;
        const T s = (x[c - 1] + x[c + 1]) + (x[c - n] + x[c + n]);
        x[c] = fmaT<T>(-h2, f[c], s) * (T)0.25;
    }
    __syncthreads();
}

template <class T>
__global__ void __launch_bounds__(BP_THREADS) k_local_vcycle(BatchDev B, int nu1, int nu2, int zero_level0,
                                                               int correct_level0)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = (T *)smem_raw;
    const int p = blockIdx.x;
    if (!B.active[p]) return;
    const int L = B.nlev[p], d0 = B.dloc[p];
    int off[BP_MAXL];
    int tot = 0;
    for (int l = d0; l < L; ++l) {
        off[l] = tot;
        const int n = B.n_of[p * BP_MAXL + l];
        tot += n * n;
    }
    T *X = sm, *F = sm + tot, *R = sm + 2 * tot;
    // load level d0 (x and f), zero everything else
    for (int q = threadIdx.x; q < tot; q += blockDim.x) { X[q] = (T)0; F[q] = (T)0; R[q] = (T)0; }
    __syncthreads();
    {
        // the level's solution is a correction that starts at zero unless this
        // is the finest level of a plain FP64 solve
        const bool zero = d0 > 0 || zero_level0;
        const int n = B.n_of[p * BP_MAXL + d0];
        const T *gx = XS<T>(B, p, d0, 0), *gf = FP<T>(B, p, d0);
        for (int q = threadIdx.x; q < n * n; q += blockDim.x) {
            if (!zero) X[q] = gx[q];
            F[q] = gf[q];
        }
    }
    __syncthreads();
    // descent
    for (int l = d0; l < L - 1; ++l) {
        const int n = B.n_of[p * BP_MAXL + l], nc = B.n_of[p * BP_MAXL + l + 1];
        T *x = X + off[l], *f = F + off[l], *r = R + off[l];
        const T h = (T)1 / (T)(n - 1), h2 = h * h, ih2 = (T)1 / h2;
        for (int s = 0; s < nu1; ++s) { loc_rb_half(x, f, n, h2, 0); loc_rb_half(x, f, n, h2, 1); }
        const int m = n - 2;
        for (int q = threadIdx.x; q < m * m; q += blockDim.x) {
            const int j = q / m + 1, i = q - (j - 1) * m + 1;
            const int c = j * n + i;
            const T s = (x[c - 1] + x[c + 1]) + (x[c - n] + x[c + n]);
            const T lap = fmaT<T>((T)-4, x[c], s);
            r[c] = fmaT<T>(-ih2, lap, f[c]);
        }
        __syncthreads();
        T *fc = F + off[l + 1], *xc = X + off[l + 1];
        const int mc = nc - 2;
        for (int q = threadIdx.x; q < mc * mc; q += blockDim.x) {
            const int j = q / mc + 1, i = q - (j - 1) * mc + 1;
            const int c = (2 * j) * n + 2 * i;
            T t = r[c];
            t = t * (T)2 + r[c + 1] + r[c - 1];
            t = t + r[c + n] + r[c - n];
            t = t * (T)2 + r[c + 1 + n] + r[c - 1 - n];
            t = t + r[c + 1 - n] + r[c - 1 + n];
            fc[j * nc + i] = t * (T)0.0625;
            xc[j * nc + i] = (T)0;
        }
        __syncthreads();
    }
    // coarsest: one red update solves the single interior point
    {
        const int n = B.n_of[p * BP_MAXL + L - 1];
        const T h = (T)1 / (T)(n - 1);
        loc_rb_half(X + off[L - 1], F + off[L - 1], n, h * h, 0);
    }
    // ascent
    for (int l = L - 2; l >= d0; --l) {
        const int n = B.n_of[p * BP_MAXL + l], nc = B.n_of[p * BP_MAXL + l + 1], m = n - 2;
        T *x = X + off[l], *f = F + off[l];
        const T *ec = X + off[l + 1];
        for (int q = threadIdx.x; q < m * m; q += blockDim.x) {
            const int j = q / m + 1, i = q - (j - 1) * m + 1;
            const T *ep = ec + (j / 2) * nc + (i / 2);
            T v;
            if ((i & 1) == 0) {
                if ((j & 1) == 0) v = ep[0];
                else v = (ep[0] + ep[nc]) * (T)0.5;
            } else {
                if ((j & 1) == 0) v = (ep[0] + ep[1]) * (T)0.5;
                else {
                    T t = ep[0] + ep[nc + 1];
                    t = t + ep[nc] + ep[1];
                    v = t * (T)0.25;
                }
            }
            const int c = j * n + i;
            x[c] = x[c] + v;
        }
        __syncthreads();
        const T h = (T)1 / (T)(n - 1), h2 = h * h;
        for (int s = 0; s < nu2; ++s) { loc_rb_half(x, f, n, h2, 0); loc_rb_half(x, f, n, h2, 1); }
    }
    {
        // the local levels end in buffer 0; a mixed solve local from level 0
        // applies its correction to the FP64 solution directly
        const int n = B.n_of[p * BP_MAXL + d0];
        if (d0 == 0 && correct_level0) {
            double *psi = B.psi[p];
            for (int q = threadIdx.x; q < n * n; q += blockDim.x) psi[q] = psi[q] + (double)X[q];
        } else {
            T *gx = XS<T>(B, p, d0, 0);
            for (int q = threadIdx.x; q < n * n; q += blockDim.x) gx[q] = X[q];
        }
    }
}

// ---------------------------------------------------------------------------
// Norms, defect correction and convergence bookkeeping
// ---------------------------------------------------------------------------
__device__ __forceinline__ double blk_sum(double v, double *s_red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < nw; ++w) r += s_red[w];
    return r;
}

// FP64 outer pass over one TX x TY tile of level 0 (psi, f: the caller's
// arrays): the residual r = f - A psi, its squared norm (block partial) and,
// when store_r, r rounded to FP32 as the inner cycle's right-hand side.
// psi is only read here, so neighbouring tiles may overlap freely.
__global__ void __launch_bounds__(TILE_THREADS) k_outer(BatchDev B, const TileEntry *tiles, const double *const *f_p,
                                                        int store_r)
{
    __shared__ double sp[(TY + 2) * (TX + 2)];
    __shared__ double s_red[32];
    constexpr int SX = TX + 2, SY = TY + 2;
    const TileEntry e = tiles[blockIdx.x];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (!B.active[e.p]) {
        if (threadIdx.x == 0) B.partial[blockIdx.x] = 0.0;
        return;
    }
    const int n = B.n_of[e.p * BP_MAXL];
    const int x0 = e.tx * TX, y0 = e.ty * TY, ox = x0 - 1, oy = y0 - 1;
    const double *psi = B.psi[e.p];
    const double *f = f_p[e.p];
    for (int r = warp; r < SY; r += nw) {
        const int gy = oy + r;
        const bool rowin = gy >= 0 && gy < n;
        for (int c = lane; c < SX; c += 32) {
            const int gx = ox + c;
            sp[r * SX + c] = (rowin && gx >= 0 && gx < n) ? psi[(size_t)gy * n + gx] : 0.0;
        }
    }
    __syncthreads();
    const double h = 1.0 / (double)(n - 1), ih2 = 1.0 / (h * h);
    float *f32 = store_r ? FP<float>(B, e.p, 0) : nullptr;
    double acc = 0.0;
    const int gxa = max(x0, 1), gxb = min(x0 + TX, n - 1);
    const int gya = max(y0, 1), gyb = min(y0 + TY, n - 1);
    for (int gy = gya + warp; gy < gyb; gy += nw) {
        for (int gx = gxa + lane; gx < gxb; gx += 32) {
            const int q = (gy - oy) * SX + gx - ox;
            const size_t g = (size_t)gy * n + gx;
            const double s = (sp[q - 1] + sp[q + 1]) + (sp[q - SX] + sp[q + SX]);
            const double lap = __fma_rn(-4.0, sp[q], s);
            const double r = __fma_rn(-ih2, lap, f[g]);
            acc = __fma_rn(r, r, acc);
            if (store_r) f32[g] = (float)r;
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) s_red[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; ++w) t += s_red[w];
        B.partial[blockIdx.x] = t;
    }
}

// Copies buffer 1 of level 0 into the caller's psi (plain FP64 cycles whose
// level-0 kernels leave the result in the internal buffer).
__global__ void __launch_bounds__(TILE_THREADS) k_copy_back(BatchDev B, const TileEntry *tiles)
{
    const TileEntry e = tiles[blockIdx.x];
    if (!B.active[e.p]) return;
    const int n = B.n_of[e.p * BP_MAXL];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const double *src = XS<double>(B, e.p, 0, 1);
    double *dst = B.psi[e.p];
    const int x0 = e.tx * TX, y0 = e.ty * TY;
    const int gxa = max(x0, 1), gxb = min(x0 + TX, n - 1);
    const int gya = max(y0, 1), gyb = min(y0 + TY, n - 1);
    for (int gy = gya + warp; gy < gyb; gy += nw)
        for (int gx = gxa + lane; gx < gxb; gx += 32) dst[(size_t)gy * n + gx] = src[(size_t)gy * n + gx];
}

// One warp per problem: sums the problem's tile partials in a fixed order
// and decides whether it keeps cycling.  first != 0 records ||f|| (psi = 0).
__global__ void k_finalize(BatchDev B, int first)
{
    const int lane = threadIdx.x & 31;
    const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (p >= B.nprob) return;
    if (!B.active[p]) return;
    double s = 0.0;
    const int b0 = B.p_blk0[p], nb = B.p_nblk0[p];
    for (int b = lane; b < nb; b += 32) s += B.partial[b0 + b];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane != 0) return;
    const double rn = sqrt(s);
    if (first) B.fnorm[p] = rn;
    const double fn = B.fnorm[p];
    B.relres[p] = fn > 0.0 ? rn / fn : 0.0;
    if (rn <= B.rtol * fn) {
        B.active[p] = 0;
    } else if (B.cycles[p] >= B.max_cycles) {
        B.active[p] = 0;
        B.failed[p] = 1;
    } else {
        B.cycles[p] += B.inner;
        atomicAdd(B.num_active, 1);
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct gb_batch {
    int nprob = 0, precision = 0, nu1 = 2, nu2 = 2, max_cycles = 100;
    int inner = 1;                      // V-cycles per outer iteration (mixed)
    int cur0 = 0;                       // level-0 buffer holding the correction between inner cycles
    double rtol = 1e-10;
    std::vector<int> n, L, dloc;
    long long total = 0;
    std::vector<long long> off0;        // level-0 offsets in the packed user arrays
    int maxdepth_global = 0;            // levels 0..maxdepth_global-1 have tile work
    void *pool = nullptr;               // per-level x, f (T = double or float)
    size_t pool_bytes = 0;
    int *d_int = nullptr;
    double *d_dbl = nullptr;
    void **d_ptrs = nullptr;
    TileEntry *d_tiles = nullptr;
    std::vector<int> ft_off, ft_cnt;    // per level: fine tiles (problems with l < dloc)
    std::vector<int> ct_off, ct_cnt;    // per level l >= 1: coarse tiles of l (problems with l <= dloc)
    int ot_off = 0, ot_cnt = 0;         // level-0 tiles of every problem (outer pass)
    BatchDev dev;
    double **d_psi_tab = nullptr, **d_f_tab = nullptr;
    std::vector<void *> hx, hf;
    size_t local_smem = 0;
    int *h_pinned = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t cycle_graph = nullptr;
    long long launches = 0, launches_per_cycle = 0;
    // optional per-launch timing of the finest-level pre-smoothing kernel
    int profile = 0, graph_profile = -1, graph_ev = 0;
    std::vector<cudaEvent_t> ev;
    int ev_used = 0;
    double prof_ms = 0.0, prof_bytes = 0.0;
    long long prof_launches = 0;
    std::vector<int> h_active;
};

static int levels_of(int n, int *nl)
{
    int L = 0;
    while (true) {
        nl[L++] = n;
        if (n <= 3) break;
        n = (n - 1) / 2 + 1;
    }
    return L;
}

template <class T, int NU> static size_t smem_smooth() { return 2 * sizeof(T) * (TX + 4 * NU) * (TY + 4 * NU); }
template <class T> static size_t smem_restrict() { return sizeof(T) * ((2 * CX + 3) * (2 * CY + 3) + (2 * CX + 1) * (2 * CY + 1)); }

template <class T> static cudaError_t set_smem_attrs(size_t local)
{
    cudaError_t e;
#define SA(k, sz) if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sz))) != cudaSuccess) return e
    SA((k_smooth<T, 1, false>), (smem_smooth<T, 1>()));
    SA((k_smooth<T, 2, false>), (smem_smooth<T, 2>()));
    SA((k_smooth<T, 1, true>), (smem_smooth<T, 1>()));
    SA((k_smooth<T, 2, true>), (smem_smooth<T, 2>()));
    SA((k_prolong_smooth<T, 0, false>), (smem_smooth<T, 0>()));
    SA((k_prolong_smooth<T, 1, false>), (smem_smooth<T, 1>()));
    SA((k_prolong_smooth<T, 2, false>), (smem_smooth<T, 2>()));
    SA((k_prolong_smooth<T, 0, true>), (smem_smooth<T, 0>()));
    SA((k_prolong_smooth<T, 1, true>), (smem_smooth<T, 1>()));
    SA((k_prolong_smooth<T, 2, true>), (smem_smooth<T, 2>()));
    SA((k_resid_restrict<T>), (smem_restrict<T>()));
    SA((k_local_vcycle<T>), (local));
#undef SA
    return cudaSuccess;
}

extern "C" int gb_batch_create(int nprob, const int *n, int precision, int nu1, int nu2, double rtol,
                               int max_cycles, gb_batch **out)
{
    if (!out || !n || nprob <= 0 || (precision != GB_BATCH_FP64 && precision != GB_BATCH_MIXED) || nu1 < 1 ||
        nu1 > 8 || nu2 < 0 || nu2 > 8 || max_cycles < 0 || !(rtol >= 0.0)) {
        gb_set_error("gb_batch_create: invalid argument (need nprob > 0, 1 <= nu1 <= 8, 0 <= nu2 <= 8)");
        return GB_ERR_INVALID;
    }
    *out = nullptr;
    gb_batch *b = new gb_batch();
    b->nprob = nprob;
    b->precision = precision;
    b->nu1 = nu1;
    b->nu2 = nu2;
    b->rtol = rtol;
    b->max_cycles = max_cycles;
    b->n.assign(n, n + nprob);
    b->L.resize(nprob);
    b->dloc.resize(nprob);
    b->off0.resize(nprob);
    std::vector<int> nof((size_t)nprob * BP_MAXL, 0);
    const size_t esz = precision == GB_BATCH_FP64 ? sizeof(double) : sizeof(float);
    size_t pool_elems = 0;
    long long tot = 0;
    int maxd = 0;
    for (int p = 0; p < nprob; ++p) {
        const int np_ = n[p];
        if (np_ < 3 || np_ > 8193 || ((np_ - 1) & (np_ - 2)) != 0) {
            gb_set_error("gb_batch_create: problem %d has n=%d (need n = 2^m + 1, 3 <= n <= 8193)", p, np_);
            delete b;
            return GB_ERR_INVALID;
        }
        int nl[BP_MAXL];
        const int L = levels_of(np_, nl);
        b->L[p] = L;
        int d = 0;
        while (nl[d] > LOCAL_N) ++d;
        b->dloc[p] = d;
        maxd = std::max(maxd, d);
        for (int l = 0; l < L; ++l) {
            nof[(size_t)p * BP_MAXL + l] = nl[l];
            // x buffers 0 and 1 plus f; the plain solve's level 0 uses the
            // caller's psi and f, with one internal FP64 buffer beside psi
            const size_t sz = (size_t)nl[l] * nl[l];
            if (precision == GB_BATCH_FP64 && l == 0) pool_elems += sz;
            else pool_elems += 3 * sz;
        }
        b->off0[p] = tot;
        tot += (long long)np_ * np_;
    }
    b->total = tot;
    b->maxdepth_global = maxd;
    size_t smax = 0;
    for (int p = 0; p < nprob; ++p) {
        size_t sz = 0;
        for (int l = b->dloc[p]; l < b->L[p]; ++l) sz += (size_t)nof[(size_t)p * BP_MAXL + l] * nof[(size_t)p * BP_MAXL + l];
        smax = std::max(smax, 3 * sz * esz);
    }
    b->local_smem = smax;
    // tile tables
    std::vector<TileEntry> tiles;
    b->ft_off.assign(BP_MAXL + 1, 0);
    b->ft_cnt.assign(BP_MAXL + 1, 0);
    b->ct_off.assign(BP_MAXL + 1, 0);
    b->ct_cnt.assign(BP_MAXL + 1, 0);
    std::vector<int> pb0(nprob), pnb0(nprob);
    auto add_tiles = [&](int p, int nn, int tw, int th) {
        for (int ty = 0; ty * th < nn - 1; ++ty)
            for (int tx = 0; tx * tw < nn - 1; ++tx) tiles.push_back({p, (short)tx, (short)ty});
    };
    for (int l = 0; l < BP_MAXL; ++l) {
        b->ft_off[l] = (int)tiles.size();
        for (int p = 0; p < nprob; ++p)
            if (l < b->dloc[p]) add_tiles(p, nof[(size_t)p * BP_MAXL + l], TX, TY);
        b->ft_cnt[l] = (int)tiles.size() - b->ft_off[l];
        b->ct_off[l] = (int)tiles.size();
        for (int p = 0; p < nprob; ++p)
            if (l >= 1 && l <= b->dloc[p]) add_tiles(p, nof[(size_t)p * BP_MAXL + l], CX, CY);
        b->ct_cnt[l] = (int)tiles.size() - b->ct_off[l];
    }
    b->ot_off = (int)tiles.size();
    for (int p = 0; p < nprob; ++p) {
        pb0[p] = (int)tiles.size() - b->ot_off;
        add_tiles(p, n[p], TX, TY);
        pnb0[p] = (int)tiles.size() - b->ot_off - pb0[p];
    }
    b->ot_cnt = (int)tiles.size() - b->ot_off;

#define BTRY(x)                                                                 \
    do {                                                                        \
        cudaError_t _e = (x);                                                   \
        if (_e != cudaSuccess) {                                                \
            gb_set_error("gb_batch_create: %s: %s", #x, cudaGetErrorString(_e)); \
            gb_batch_destroy(b);                                                \
            return GB_ERR_ALLOC;                                                \
        }                                                                       \
    } while (0)
    b->pool_bytes = std::max<size_t>(pool_elems * esz, 16);
    BTRY(cudaMalloc(&b->pool, b->pool_bytes));
    BTRY(cudaMemset(b->pool, 0, b->pool_bytes));
    const size_t nint = (size_t)nprob * BP_MAXL + 7 * (size_t)nprob + 1;
    BTRY(cudaMalloc(&b->d_int, sizeof(int) * nint));
    BTRY(cudaMemset(b->d_int, 0, sizeof(int) * nint));
    BTRY(cudaMalloc(&b->d_dbl, sizeof(double) * (2 * (size_t)nprob + (size_t)b->ot_cnt)));
    // pointer tables: x (two buffers per level), f (one per level), psi and f of level 0
    const size_t nptr = 2 * (size_t)nprob * BP_MAXL + (size_t)nprob * BP_MAXL + 2 * (size_t)nprob;
    BTRY(cudaMalloc(&b->d_ptrs, sizeof(void *) * nptr));
    BTRY(cudaMalloc(&b->d_tiles, sizeof(TileEntry) * tiles.size()));
    BTRY(cudaMallocHost(&b->h_pinned, sizeof(int) * 16));
    BTRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    b->hx.assign(2 * (size_t)nprob * BP_MAXL, nullptr);
    b->hf.assign((size_t)nprob * BP_MAXL, nullptr);
    char *base = (char *)b->pool;
    for (int p = 0; p < nprob; ++p) {
        for (int l = 0; l < b->L[p]; ++l) {
            const size_t sz = (size_t)nof[(size_t)p * BP_MAXL + l] * nof[(size_t)p * BP_MAXL + l] * esz;
            const size_t k = (size_t)p * BP_MAXL + l;
            const size_t k1 = ((size_t)nprob + p) * BP_MAXL + l;
            if (precision == GB_BATCH_FP64 && l == 0) {
                b->hx[k1] = base; base += sz;
                continue;
            }
            b->hx[k] = base; base += sz;
            b->hx[k1] = base; base += sz;
            b->hf[k] = base; base += sz;
        }
    }
    int *di = b->d_int;
    int *d_nof = di; di += (size_t)nprob * BP_MAXL;
    int *d_nlev = di; di += nprob;
    int *d_dloc = di; di += nprob;
    int *d_active = di; di += nprob;
    int *d_cycles = di; di += nprob;
    int *d_failed = di; di += nprob;
    int *d_pb0 = di; di += nprob;
    int *d_pnb0 = di; di += nprob;
    int *d_numact = di;
    BTRY(cudaMemcpy(d_nof, nof.data(), sizeof(int) * nof.size(), cudaMemcpyHostToDevice));
    BTRY(cudaMemcpy(d_nlev, b->L.data(), sizeof(int) * nprob, cudaMemcpyHostToDevice));
    BTRY(cudaMemcpy(d_dloc, b->dloc.data(), sizeof(int) * nprob, cudaMemcpyHostToDevice));
    BTRY(cudaMemcpy(d_pb0, pb0.data(), sizeof(int) * nprob, cudaMemcpyHostToDevice));
    BTRY(cudaMemcpy(d_pnb0, pnb0.data(), sizeof(int) * nprob, cudaMemcpyHostToDevice));
    BTRY(cudaMemcpy(b->d_tiles, tiles.data(), sizeof(TileEntry) * tiles.size(), cudaMemcpyHostToDevice));
    void **dp = b->d_ptrs;
    BTRY(cudaMemcpy(dp, b->hx.data(), sizeof(void *) * b->hx.size(), cudaMemcpyHostToDevice));
    BTRY(cudaMemcpy(dp + b->hx.size(), b->hf.data(), sizeof(void *) * b->hf.size(), cudaMemcpyHostToDevice));
    // table layout: x (2 buffers), f, then the caller's psi and f per problem
    b->d_psi_tab = (double **)(dp + b->hx.size() + b->hf.size());
    b->d_f_tab = (double **)(dp + b->hx.size() + b->hf.size() + nprob);
    if (b->hx.size() + b->hf.size() + 2 * (size_t)nprob != nptr) {
        gb_set_error("gb_batch_create: pointer table layout mismatch");
        gb_batch_destroy(b);
        return GB_ERR_INVALID;
    }
    BatchDev &D = b->dev;
    D.nprob = nprob;
    D.n_of = d_nof;
    D.nlev = d_nlev;
    D.dloc = d_dloc;
    D.x = dp;
    D.f = dp + b->hx.size();
    D.r = nullptr;
    D.psi = b->d_psi_tab;
    D.active = d_active;
    D.cycles = d_cycles;
    D.failed = d_failed;
    D.fnorm = b->d_dbl;
    D.relres = b->d_dbl + nprob;
    D.partial = b->d_dbl + 2 * nprob;
    D.p_blk0 = d_pb0;
    D.p_nblk0 = d_pnb0;
    D.num_active = d_numact;
    D.max_cycles = max_cycles;
    D.inner = 1;
    D.rtol = rtol;
    if (precision == GB_BATCH_FP64) BTRY(set_smem_attrs<double>(b->local_smem));
    else BTRY(set_smem_attrs<float>(b->local_smem));
#undef BTRY
    *out = b;
    return GB_OK;
}

extern "C" int gb_batch_destroy(gb_batch *b)
{
    if (!b) return GB_OK;
    if (b->cycle_graph) cudaGraphExecDestroy(b->cycle_graph);
    for (auto &e : b->ev) cudaEventDestroy(e);
    cudaFree(b->pool);
    cudaFree(b->d_int);
    cudaFree(b->d_dbl);
    cudaFree(b->d_ptrs);
    cudaFree(b->d_tiles);
    if (b->h_pinned) cudaFreeHost(b->h_pinned);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return GB_OK;
}

extern "C" long long gb_batch_total_points(const gb_batch *b) { return b ? b->total : 0; }

extern "C" int gb_batch_set_inner_cycles(gb_batch *b, int inner)
{
    if (!b || inner < 1 || inner > 16 || (b->precision == GB_BATCH_FP64 && inner != 1)) {
        gb_set_error("gb_batch_set_inner_cycles: need 1 <= inner <= 16 (and 1 for the plain FP64 solve)");
        return GB_ERR_INVALID;
    }
    if (inner != b->inner && b->cycle_graph) {
        cudaGraphExecDestroy(b->cycle_graph);
        b->cycle_graph = nullptr;
    }
    b->inner = inner;
    b->dev.inner = inner;
    return GB_OK;
}
extern "C" long long gb_batch_last_launches(const gb_batch *b) { return b ? b->launches : 0; }

// Records a timing event: as an event node of the graph while the stream is
// being captured, as a plain record otherwise.
static void prof_record(cudaEvent_t e, cudaStream_t s)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cs);
    if (cs == cudaStreamCaptureStatusActive) cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    else cudaEventRecord(e, s);
}

// Launch plan of one level: how many sweeps each smoothing launch does
// (two per launch in FP32, one in FP64, whose pipe is the bottleneck and
// would pay for the wider halo's redundant updates).
template <class T> static int sweeps_per_launch(int nu) { return (sizeof(T) == 4 && nu >= 2) ? 2 : 1; }
template <class T> static int launches_for(int nu)
{
    int k = 0;
    while (nu > 0) { nu -= sweeps_per_launch<T>(nu); ++k; }
    return k;
}

template <class T>
static void launch_smooth(gb_batch *b, int l, int k, int zero_init, int src, int dst, int correct, cudaStream_t s,
                          bool timed)
{
    const int cnt = b->ft_cnt[l];
    const TileEntry *t = b->d_tiles + b->ft_off[l];
    const bool ev = timed && b->profile && b->ev_used + 2 <= (int)b->ev.size();
    const size_t sm = k == 2 ? smem_smooth<T, 2>() : smem_smooth<T, 1>();
    if (ev) prof_record(b->ev[b->ev_used], s);
    if (k == 2 && correct) k_smooth<T, 2, true><<<cnt, TILE_THREADS, sm, s>>>(b->dev, t, l, zero_init, src, dst);
    else if (k == 2) k_smooth<T, 2, false><<<cnt, TILE_THREADS, sm, s>>>(b->dev, t, l, zero_init, src, dst);
    else if (correct) k_smooth<T, 1, true><<<cnt, TILE_THREADS, sm, s>>>(b->dev, t, l, zero_init, src, dst);
    else k_smooth<T, 1, false><<<cnt, TILE_THREADS, sm, s>>>(b->dev, t, l, zero_init, src, dst);
    if (ev) { prof_record(b->ev[b->ev_used + 1], s); b->ev_used += 2; }
    b->launches += 1;
}

template <class T>
static void launch_prolong(gb_batch *b, int l, int nu, int src, int dst, int correct, cudaStream_t s)
{
    const int cnt = b->ft_cnt[l];
    const TileEntry *t = b->d_tiles + b->ft_off[l];
#define PL(NU, C) k_prolong_smooth<T, NU, C><<<cnt, TILE_THREADS, smem_smooth<T, NU>(), s>>>(b->dev, t, l, src, 0, dst)
    if (nu == 2) { if (correct) PL(2, true); else PL(2, false); }
    else if (nu == 1) { if (correct) PL(1, true); else PL(1, false); }
    else { if (correct) PL(0, true); else PL(0, false); }
#undef PL
    b->launches += 1;
}

// The kernels of one V-cycle: pre-smoothing, residual + restriction on each
// tile level, the local coarse cycles, then prolongation + post-smoothing.
// Tile kernels read one buffer of a level and write the other; the plan
// picks the buffers so that every coarse level ends in buffer 0 (where the
// local kernel also leaves its levels) and the plain solve's level 0 ends in
// the caller's psi (buffer 0).  Mixed: zero0 = the level-0 correction starts
// at zero (first inner cycle of an outer iteration), corr0 = the last
// level-0 kernel adds the correction to psi (last inner cycle); between
// inner cycles the correction waits in level-0 buffer b->cur0.
template <class T>
static void enqueue_vcycle(gb_batch *b, cudaStream_t s, bool zero0, bool corr0)
{
    const bool mixed = b->precision == GB_BATCH_MIXED;
    int cur[BP_MAXL] = {0};
    const int k1 = launches_for<T>(b->nu1);
    const int pro = std::min(b->nu2, sizeof(T) == 4 ? 2 : 1);  // sweeps fused into the prolongation
    const int k2 = launches_for<T>(b->nu2 - pro);
    for (int l = 0; l < b->maxdepth_global; ++l) {
        if (b->ft_cnt[l] == 0) continue;
        const bool zero = l > 0 || (mixed && zero0);
        const int writes = k1 + 1 + k2;
        int src, dst;
        if (zero) { dst = (writes - 1) & 1; src = 1 - dst; }
        else if (mixed) { src = b->cur0; dst = 1 - src; }   // level 0, later inner cycle
        else { src = 0; dst = 1; }                          // level 0 of the plain solve: psi
        int nu = b->nu1;
        for (int i = 0; i < k1; ++i) {
            const int k = sweeps_per_launch<T>(nu);
            launch_smooth<T>(b, l, k, (zero && i == 0) ? 1 : 0, src, dst, 0, s, l == 0);
            nu -= k;
            src = dst;
            dst = 1 - dst;
        }
        cur[l] = src;
        k_resid_restrict<T><<<b->ct_cnt[l + 1], TILE_THREADS, smem_restrict<T>(), s>>>(
            b->dev, b->d_tiles + b->ct_off[l + 1], l, cur[l]);
        b->launches += 1;
    }
    k_local_vcycle<T><<<b->nprob, BP_THREADS, b->local_smem, s>>>(b->dev, b->nu1, b->nu2, (mixed && zero0) ? 1 : 0,
                                                                 (mixed && corr0) ? 1 : 0);
    b->launches += 1;
    for (int l = b->maxdepth_global - 1; l >= 0; --l) {
        if (b->ft_cnt[l] == 0) continue;
        const int correct_last = (mixed && l == 0 && corr0) ? 1 : 0;
        int src = cur[l], dst = 1 - cur[l];
        launch_prolong<T>(b, l, pro, src, dst, k2 == 0 ? correct_last : 0, s);
        src = dst;
        dst = 1 - dst;
        int nu = b->nu2 - pro;
        for (int i = 0; i < k2; ++i) {
            const int k = sweeps_per_launch<T>(nu);
            launch_smooth<T>(b, l, k, 0, src, dst, (i == k2 - 1) ? correct_last : 0, s, false);
            nu -= k;
            src = dst;
            dst = 1 - dst;
        }
        cur[l] = src;
        if (!mixed && l == 0 && cur[0] != 0) {
            k_copy_back<<<b->ft_cnt[0], TILE_THREADS, 0, s>>>(b->dev, b->d_tiles + b->ft_off[0]);
            b->launches += 1;
        }
    }
    if (mixed) b->cur0 = cur[0];
}

// One outer iteration: the FP64 residual norm of level 0 (mixed: also its
// FP32 copy as the inner right-hand side), convergence bookkeeping, then
// b->inner V-cycles (mixed: the last one's final level-0 kernel adds the
// correction to psi).
static void enqueue_iteration(gb_batch *b, int first, cudaStream_t s)
{
    BatchDev &D = b->dev;
    const TileEntry *t0 = b->d_tiles + b->ot_off;
    cudaMemsetAsync(D.num_active, 0, sizeof(int), s);
    const bool mixed = b->precision == GB_BATCH_MIXED;
    k_outer<<<b->ot_cnt, TILE_THREADS, 0, s>>>(D, t0, (const double *const *)b->d_f_tab, mixed ? 1 : 0);
    k_finalize<<<gb_ceil_div(b->nprob, 4), 128, 0, s>>>(D, first);
    b->launches += 2;
    if (mixed) {
        b->cur0 = 0;
        for (int k = 0; k < b->inner; ++k) enqueue_vcycle<float>(b, s, k == 0, k == b->inner - 1);
    } else {
        enqueue_vcycle<double>(b, s, false, false);
    }
    cudaMemcpyAsync(b->h_pinned, D.num_active, sizeof(int), cudaMemcpyDeviceToHost, s);
}

// After an iteration has completed: adds the recorded pre-smoothing launch
// times and the algorithmic bytes of the problems that took part (per sweep
// and interior point: psi read, f read, psi written, one word each).
static void batch_profile_collect(gb_batch *b, cudaStream_t s)
{
    if (!b->profile || b->ev_used == 0) return;
    b->h_active.resize(b->nprob);
    cudaMemcpyAsync(b->h_active.data(), b->dev.active, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    double pts = 0.0;
    for (int p = 0; p < b->nprob; ++p)
        if (b->h_active[p] && b->dloc[p] > 0) pts += (double)(b->n[p] - 2) * (double)(b->n[p] - 2);
    const double esz = b->precision == GB_BATCH_FP64 ? 8.0 : 4.0;
    const int per_launch_sweeps = (b->precision == GB_BATCH_MIXED && b->nu1 >= 2) ? 2 : 1;  // first pre-smoothing launch
    for (int i = 0; i + 1 < b->ev_used; i += 2) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, b->ev[i], b->ev[i + 1]) == cudaSuccess) {
            b->prof_ms += ms;
            b->prof_launches += 1;
            b->prof_bytes += 3.0 * esz * per_launch_sweeps * pts;
        } else {
            cudaGetLastError();  // timing is advisory: never let it fail a solve
        }
    }
}

extern "C" int gb_batch_profile(gb_batch *b, int enable)
{
    if (!b) return GB_ERR_INVALID;
    if (enable && b->ev.empty()) {
        b->ev.resize(2 * (b->nu1 + 1));
        for (auto &e : b->ev) GB_CUDA_TRY(cudaEventCreate(&e));
    }
    b->profile = enable ? 1 : 0;
    return GB_OK;
}

extern "C" int gb_batch_profile_read(gb_batch *b, double *ms, long long *launches, double *alg_bytes, int reset)
{
    if (!b) return GB_ERR_INVALID;
    if (ms) *ms = b->prof_ms;
    if (launches) *launches = b->prof_launches;
    if (alg_bytes) *alg_bytes = b->prof_bytes;
    if (reset) {
        b->prof_ms = 0.0;
        b->prof_bytes = 0.0;
        b->prof_launches = 0;
    }
    return GB_OK;
}

static int batch_bind_io(gb_batch *b, const double *d_f, double *d_psi, cudaStream_t s)
{
    std::vector<const void *> pf(b->nprob), pp(b->nprob);
    for (int p = 0; p < b->nprob; ++p) {
        pf[p] = d_f + b->off0[p];
        pp[p] = d_psi + b->off0[p];
    }
    GB_CUDA_TRY(cudaMemcpyAsync(b->d_f_tab, pf.data(), sizeof(void *) * b->nprob, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemcpyAsync(b->d_psi_tab, pp.data(), sizeof(void *) * b->nprob, cudaMemcpyHostToDevice, s));
    if (b->precision == GB_BATCH_FP64) {
        // level-0 x and f of the plain cycle are the caller's arrays
        for (int p = 0; p < b->nprob; ++p) {
            b->hx[(size_t)p * BP_MAXL] = d_psi + b->off0[p];            // buffer 0 of level 0
            b->hf[(size_t)p * BP_MAXL] = (void *)(d_f + b->off0[p]);
        }
        GB_CUDA_TRY(cudaMemcpyAsync(b->d_ptrs, b->hx.data(), sizeof(void *) * b->hx.size(), cudaMemcpyHostToDevice, s));
        GB_CUDA_TRY(cudaMemcpyAsync(b->d_ptrs + b->hx.size(), b->hf.data(), sizeof(void *) * b->hf.size(),
                                    cudaMemcpyHostToDevice, s));
    }
    // the pointer tables live in pageable host vectors: complete the copies
    // before those vectors can change
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return GB_OK;
}

extern "C" int gb_batch_solve_device(gb_batch *b, const double *d_f, double *d_psi, int *cycles, double *relres,
                                     void *stream)
{
    if (!b || !d_f || !d_psi) { gb_set_error("gb_batch_solve_device: null argument"); return GB_ERR_INVALID; }
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    BatchDev &D = b->dev;
    b->launches = 0;
    int st = batch_bind_io(b, d_f, d_psi, s);
    if (st != GB_OK) return st;
    GB_CUDA_TRY(cudaMemsetAsync(d_psi, 0, sizeof(double) * (size_t)b->total, s));
    std::vector<int> ones(b->nprob, 1);
    GB_CUDA_TRY(cudaMemcpyAsync(D.active, ones.data(), sizeof(int) * b->nprob, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemsetAsync(D.cycles, 0, sizeof(int) * b->nprob, s));
    GB_CUDA_TRY(cudaMemsetAsync(D.failed, 0, sizeof(int) * b->nprob, s));
    // first iteration eagerly (records ||f||); later ones from a CUDA graph
    b->ev_used = 0;
    enqueue_iteration(b, 1, s);
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    batch_profile_collect(b, s);
    if (!b->cycle_graph || b->graph_profile != b->profile) {
        if (b->cycle_graph) cudaGraphExecDestroy(b->cycle_graph);
        b->cycle_graph = nullptr;
        cudaStream_t cs = b->stream;
        cudaGraph_t g;
        const long long l0 = b->launches;
        b->ev_used = 0;
        GB_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        enqueue_iteration(b, 0, cs);
        GB_CUDA_TRY(cudaStreamEndCapture(cs, &g));
        b->launches_per_cycle = b->launches - l0;
        b->launches = l0;
        GB_CUDA_TRY(cudaGraphInstantiate(&b->cycle_graph, g, 0));
        cudaGraphDestroy(g);
        b->graph_profile = b->profile;
        b->graph_ev = b->ev_used;
    }
    for (int it = 0; it <= b->max_cycles + 1 && *b->h_pinned > 0; ++it) {
        GB_CUDA_TRY(cudaGraphLaunch(b->cycle_graph, s));
        b->launches += b->launches_per_cycle;
        GB_CUDA_TRY(cudaStreamSynchronize(s));
        b->ev_used = b->graph_ev;
        batch_profile_collect(b, s);
    }
    std::vector<int> fl(b->nprob);
    GB_CUDA_TRY(cudaMemcpyAsync(fl.data(), D.failed, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost, s));
    if (cycles) GB_CUDA_TRY(cudaMemcpyAsync(cycles, D.cycles, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost, s));
    if (relres) GB_CUDA_TRY(cudaMemcpyAsync(relres, D.relres, sizeof(double) * b->nprob, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    GB_CUDA_TRY(cudaGetLastError());
    for (int p = 0; p < b->nprob; ++p)
        if (fl[p]) return GB_MAXSWEEPS;
    return GB_OK;
}

extern "C" int gb_batch_solve_host(gb_batch *b, const double *h_f, double *h_psi, int *cycles, double *relres)
{
    if (!b || !h_f || !h_psi) { gb_set_error("gb_batch_solve_host: null argument"); return GB_ERR_INVALID; }
    double *d = nullptr;
    GB_CUDA_TRY(cudaMallocAsync((void **)&d, sizeof(double) * 2 * (size_t)b->total, b->stream));
    GB_CUDA_TRY(cudaMemcpyAsync(d, h_f, sizeof(double) * (size_t)b->total, cudaMemcpyHostToDevice, b->stream));
    int st = gb_batch_solve_device(b, d, d + b->total, cycles, relres, b->stream);
    cudaMemcpyAsync(h_psi, d + b->total, sizeof(double) * (size_t)b->total, cudaMemcpyDeviceToHost, b->stream);
    cudaFreeAsync(d, b->stream);
    GB_CUDA_TRY(cudaStreamSynchronize(b->stream));
    return st;
}
