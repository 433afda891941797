// Batched Dirichlet Poisson solver: many independent n x n vertex-grid
// problems of uneven size, V(nu1,nu2) red-black Gauss-Seidel cycles with
// full-weighting restriction and bilinear prolongation (the transfer
// operators of rotann2.f:755-854), in plain FP64 or as FP32 inner V-cycles
// inside defect correction.  The defect correction's outer residual, its
// norm and the update of psi run either in FP64 (GB_BATCH_MIXED_F64OUTER)
// or in float-pair arithmetic (about 48 significand bits) on the FP32 pipe
// (GB_BATCH_MIXED); the solution is returned in FP64 either way.
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
#include <type_traits>
#include <vector>

#include "gbcommon.cuh"
#include "gridsync.cuh"

#define BP_MAXL 16
#define LOCAL_N 65        // default: levels with n <= 65 run in one block per problem
#define BP_THREADS 256

template <class T> __device__ __forceinline__ T fmaT(T a, T b, T c);
template <> __device__ __forceinline__ double fmaT<double>(double a, double b, double c) { return __fma_rn(a, b, c); }
template <> __device__ __forceinline__ float fmaT<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// Conversions between float and double on the integer pipe.  GB300 issues
// FP64 instructions (conversions included) at about 1/64 of the FP32 rate,
// and the defect-correction loop converts every point twice per outer
// iteration.  Both functions round as IEEE 754 binary conversion does
// (round to nearest, ties to even; float -> double is exact) over the whole
// range, denormals, infinities and overflow included, with integer
// operations only, so that no FP64 instruction is issued even on a
// predicated path.  A NaN converts to a quiet NaN of the same sign.
// gb_check_conversions compares both with the hardware conversions.
__device__ __forceinline__ float d2f_rn(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ffu);
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    unsigned int r;
    if (e >= 897 && e <= 1150) {
        // normal float range: keep the top 23 fraction bits, round on the
        // 29 dropped (a carry into the exponent rounds up to the next
        // binade, or to infinity past the largest float)
        r = ((unsigned int)(e - 896) << 23) | (unsigned int)(m >> 29);
        const unsigned int rem = (unsigned int)(m & 0x1FFFFFFFull);
        r += (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) ? 1u : 0u;
    } else if (e == 0x7ff) {
        r = m ? 0x7fc00000u : 0x7f800000u;
    } else if (e > 1150) {
        r = 0x7f800000u;   // at or above 2^128: overflows to infinity
    } else if (e == 0) {
        r = 0u;            // double denormals are far below the float range
    } else {
        // float denormal range: the result counts units of 2^-149, the
        // significand (with its hidden bit) shifted right by 926 - e >= 30
        const int sh = 926 - e;
        if (sh > 53) {
            r = 0u;        // below half the smallest denormal
        } else {
            const unsigned long long full = m | (1ull << 52);
            r = (unsigned int)(full >> sh);
            const unsigned long long rem = full & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
            r += (rem > half || (rem == half && (r & 1u))) ? 1u : 0u;
        }
    }
    return __uint_as_float(sign | r);
}

__device__ __forceinline__ double f2d(float v)
{
    const unsigned int u = __float_as_uint(v);
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    const unsigned int e = (u >> 23) & 0xffu, m = u & 0x7FFFFFu;
    unsigned long long r;
    if (e != 0u && e != 255u) {
        r = ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    } else if (e == 255u) {
        r = m ? 0x7ff8000000000000ull | ((unsigned long long)m << 29) : 0x7ff0000000000000ull;
    } else if (m == 0u) {
        r = 0ull;
    } else {
        // float denormal m * 2^-149: normalise so that the leading bit of m
        // becomes the hidden bit
        const int lz = __clz(m) - 8;   // m < 2^23: 9 or more leading zeros
        r = ((unsigned long long)(897 - lz) << 52) | ((unsigned long long)((m << lz) & 0x7FFFFFu) << 29);
    }
    return __longlong_as_double((long long)(sign | r));
}

__device__ __forceinline__ double to_double(float v) { return f2d(v); }

// Float pairs (hi, lo), |lo| <= ulp(hi)/2: about 48 significand bits with
// FP32 arithmetic only.  two_sum finds the rounding error of a float sum
// exactly (Knuth, TAOCP vol. 2, 4.2.2); df_add is the accurate pair sum of
// Dekker (1971) as the QD library's ieee_add arranges it.  The mixed solve
// keeps psi and f as pairs so that its outer residual runs on the FP32
// pipe; every multiplication in it is by a power of two (exact).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e)   // |a| >= |b| or a = 0
{
    s = a + b;
    e = b - (s - a);
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b)
{
    float s, e, t, f;
    two_sum(a.x, b.x, s, e);
    two_sum(a.y, b.y, t, f);
    e = e + t;
    fast_two_sum(s, e, s, e);
    e = e + f;
    fast_two_sum(s, e, s, e);
    return make_float2(s, e);
}
__device__ __forceinline__ float2 df_add_f(float2 a, float b)
{
    float s, e;
    two_sum(a.x, b, s, e);
    e = e + a.y;
    fast_two_sum(s, e, s, e);
    return make_float2(s, e);
}
__device__ __forceinline__ float2 df_scale(float2 a, float p) { return make_float2(a.x * p, a.y * p); }
__device__ __forceinline__ double to_double(double v) { return v; }

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
    double *const *psi;       // [p] the caller's solution of level 0 (FP64, or float pairs in place)
    // [p*BP_MAXL + l] h^2 and 1/h^2 of level l, h = 1/(n-1), rounded in the
    // precision of use; formed once on the host (IEEE division there as
    // here) so that no thread spends FP64 divisions on them
    const double *h2d, *ih2d;
    const float *h2f, *ih2f;
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
template <class T> __device__ __forceinline__ T H2(const BatchDev &B, int p, int l);
template <> __device__ __forceinline__ double H2<double>(const BatchDev &B, int p, int l) { return B.h2d[p * BP_MAXL + l]; }
template <> __device__ __forceinline__ float H2<float>(const BatchDev &B, int p, int l) { return B.h2f[p * BP_MAXL + l]; }
template <class T> __device__ __forceinline__ T IH2(const BatchDev &B, int p, int l);
template <> __device__ __forceinline__ double IH2<double>(const BatchDev &B, int p, int l) { return B.ih2d[p * BP_MAXL + l]; }
template <> __device__ __forceinline__ float IH2<float>(const BatchDev &B, int p, int l) { return B.ih2f[p * BP_MAXL + l]; }

// ---------------------------------------------------------------------------
// Tile operations
//
// A fine tile is TX x TY grid points with origin (tx*TX, ty*TY); the block
// stages the tile plus a halo of H points in shared memory and runs NU
// red-black sweeps there: sweep s updates red on ring H-1-2s and black on
// ring H-2-2s, so after NU sweeps the tile plus ring H-2*NU is exact.
// Points on the Dirichlet boundary or outside the grid are never updated.
// Every operation reads one buffer of a level and writes another (or a
// different array), because neighbouring tiles read each other's points as
// halo while they run.  Each operation ends with a block barrier so that a
// block may run the next operation in the same shared memory.
// ---------------------------------------------------------------------------
// 128 x 32 tiles of 256 threads.  128 x 64 tiles of 512 threads (halo
// rings adding 17% instead of 29% to a down operation's sweeps, the same
// warps per SM) measured 5% slower per solve of the 256-problem workload
// (5.96 against 5.67 ms); updating two points per lane with paired shared
// loads measured no faster (5.63 ms either way).
#define TX 128
#define TY 32
#define TILE_THREADS (8 * TY)   // 256
#define ST_R (TY / (TILE_THREADS / 32))   // rows a thread stores: the block's warps step through TY rows
#define ST_C (TX / 32)                    // columns a thread stores

// Colour-split shared layout of a tile staged with halo H: the points of
// one parity of (row + column) in one half, those of the other in the other
// half, each half row-major with SX/2 points per row.  A red-black phase then
// walks consecutive words of one half (its neighbours are consecutive words
// of the other), where the plain layout would walk every other word and
// serialise half of each warp's accesses into a second wavefront.  The halves
// are 16 banks apart, so accesses that alternate colour (loads, stores,
// residual) stay conflict-free too.  The tile origin is even in both
// directions (tiles are TX x TY apart and H is even), so the layout parity
// is the grid parity (gx + gy) & 1.
template <class T, int H> struct TileLayout {
    static constexpr int SX = TX + 2 * H, SY = TY + 2 * H, SXH = SX / 2;
    static constexpr int W = 128 / (int)sizeof(T);                     // words in 32 banks
    static constexpr int HALF = ((SY * SXH + W - 1) / W) * W + W / 2;  // plus 16 banks
    __device__ static __forceinline__ int at(int r, int c) { return ((r + c) & 1) * HALF + r * SXH + (c >> 1); }
};

// One row of a red-black phase: the points of one colour between the
// bounds, as consecutive words of one half (c = 2k + odd; the row neighbours
// c -+ 1 are k - 1 + odd and k + odd of the other half).
template <class T> struct PhaseRow {
    T *X;
    const T *F, *N;
    int odd, k0, kend;
};

template <class T, int H>
__device__ __forceinline__ PhaseRow<T> phase_row(T *sx, const T *sf, int gy, int oy, int ox, int gxa, int gxb,
                                                 int color)
{
    using LY = TileLayout<T, H>;
    const int row = (gy - oy) * LY::SXH;
    const int first = gxa + ((gxa + gy + color) & 1);
    const int c0 = first - ox, odd = c0 & 1;
    PhaseRow<T> R;
    R.X = sx + color * LY::HALF + row;
    R.F = sf + color * LY::HALF + row;
    R.N = sx + (color ^ 1) * LY::HALF + row;
    R.odd = odd;
    R.k0 = c0 >> 1;
    R.kend = (gxb - ox - odd + 1) >> 1;
    return R;
}

template <class T, int H>
__device__ __forceinline__ void phase_point(const PhaseRow<T> &R, int k, T h2)
{
    using LY = TileLayout<T, H>;
    const T s = (R.N[k - 1 + R.odd] + R.N[k + R.odd]) + (R.N[k - LY::SXH] + R.N[k + LY::SXH]);
    R.X[k] = fmaT<T>(-h2, R.F[k], s) * (T)0.25;
}

// One red (color 0) or black (color 1) phase on ring rho around the tile.
// The smem tile has origin (ox, oy) in grid coordinates, colour-split.  A
// row holds at most SXH = 64 + H points of a colour, so a warp covers the
// first 64 of each of two rows in two passes per row and the rest of both
// (at most H each) in one shared pass: half the lanes per row.
template <class T, int H>
__device__ __forceinline__ void tile_phase(T *sx, const T *sf, int ox, int oy, int x0, int y0, int n, T h2,
                                           int rho, int color)
{
    static_assert(TileLayout<T, H>::SXH <= 64 + 16, "row remainder must fit in half a warp");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int gxa = max(x0 - rho, 1), gxb = min(x0 + TX + rho, n - 1);
    const int gya = max(y0 - rho, 1), gyb = min(y0 + TY + rho, n - 1);
    for (int gy = gya + warp; gy < gyb; gy += 2 * nw) {
        const PhaseRow<T> A = phase_row<T, H>(sx, sf, gy, oy, ox, gxa, gxb, color);
        const bool two = gy + nw < gyb;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int k = A.k0 + lane + 32 * j;
            if (k < A.kend) phase_point<T, H>(A, k, h2);
        }
        if (two) {
            const PhaseRow<T> B = phase_row<T, H>(sx, sf, gy + nw, oy, ox, gxa, gxb, color);
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int k = B.k0 + lane + 32 * j;
                if (k < B.kend) phase_point<T, H>(B, k, h2);
            }
            const PhaseRow<T> &R = lane < 16 ? A : B;
            const int k = R.k0 + 64 + (lane & 15);
            if (k < R.kend) phase_point<T, H>(R, k, h2);
        } else if (lane < 16) {
            const int k = A.k0 + 64 + lane;
            if (k < A.kend) phase_point<T, H>(A, k, h2);
        }
    }
    __syncthreads();
}

template <class T, int H>
__device__ __forceinline__ void tile_sweeps(T *sx, const T *sf, int ox, int oy, int x0, int y0, int n, T h2, int nu)
{
    for (int s = 0; s < nu; ++s) {
        tile_phase<T, H>(sx, sf, ox, oy, x0, y0, n, h2, H - 1 - 2 * s, 0);
        tile_phase<T, H>(sx, sf, ox, oy, x0, y0, n, h2, H - 2 - 2 * s, 1);
    }
}

// Correction modes of the last level-0 operation of an inner cycle:
// CM_NONE stores the tile into x; CM_PAIR adds it to psi held as float
// pairs (GB_BATCH_MIXED); CM_F64 adds it, widened exactly, to the FP64 psi
// (GB_BATCH_MIXED_F64OUTER).
#define CM_NONE 0
#define CM_PAIR 1
#define CM_F64 2

// psi values of the points this thread stores (fixed assignment: row
// warp + 8*rr, column lane + 32*cc of the tile), fetched together after the
// sweeps so that the defect correction's reads of psi overlap one another.
// Both correction modes hold 8 bytes per point (a float pair or a double).
template <class V>
__device__ __forceinline__ void psi_prefetch(const V *psi, int x0, int y0, int n, V (&pv)[ST_R * ST_C])
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int rr = 0; rr < ST_R; ++rr)
#pragma unroll
        for (int cc = 0; cc < ST_C; ++cc) {
            const int gy = y0 + warp + (TILE_THREADS / 32) * rr, gx = x0 + lane + 32 * cc;
            const bool in = gx >= 1 && gx <= n - 2 && gy >= 1 && gy <= n - 2;
            V z;
            if constexpr (std::is_same<V, float2>::value) z = make_float2(0.f, 0.f);
            else z = (V)0;
            pv[rr * ST_C + cc] = in ? psi[(size_t)gy * n + gx] : z;
        }
}

template <int CM> struct CorrVal { typedef float2 type; };
template <> struct CorrVal<CM_F64> { typedef double type; };

// Stores the tile's interior points into x, or (CM != CM_NONE) adds them to
// the solution: the last level-0 operation of an inner cycle applies the
// defect correction psi += e point by point.
template <class T, int H, int CM>
__device__ __forceinline__ void tile_store(const T *sx, int ox, int oy, int x0, int y0, int n, T *x, void *psi,
                                           const typename CorrVal<CM>::type (&pv)[ST_R * ST_C])
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int rr = 0; rr < ST_R; ++rr)
#pragma unroll
        for (int cc = 0; cc < ST_C; ++cc) {
            const int gy = y0 + warp + (TILE_THREADS / 32) * rr, gx = x0 + lane + 32 * cc;
            if (gx < 1 || gx > n - 2 || gy < 1 || gy > n - 2) continue;
            const size_t g = (size_t)gy * n + gx;
            const T v = sx[TileLayout<T, H>::at(gy - oy, gx - ox)];
            if constexpr (CM == CM_PAIR) ((float2 *)psi)[g] = df_add_f(pv[rr * ST_C + cc], (float)v);
            else if constexpr (CM == CM_F64) ((double *)psi)[g] = pv[rr * ST_C + cc] + f2d((float)v);
            else x[g] = v;
        }
}

// Loads x (or zeros) and f over the tile plus an H halo: warps step
// through the rows, each lane through pairs of columns (2P, 2P + 1: even
// and odd, the tile origin being even), whose points go to the same word
// of the two colour halves (coalesced in global memory, conflict-free in
// shared memory; no division and one row base per row).
template <class T, int H>
__device__ __forceinline__ void tile_load(T *sx, T *sf, const T *x, const T *f, int ox, int oy, int n,
                                          bool zero_x, bool load_f)
{
    using LY = TileLayout<T, H>;
    constexpr int SX = LY::SX, SY = LY::SY, NP = SX / 2;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int r = warp; r < SY; r += TILE_THREADS / 32) {
        const int gy = oy + r;
        const bool rin = gy >= 0 && gy < n;
        const size_t base = rin ? (size_t)gy * n : 0;
        const T *xr = x + base, *fr = f + base;
        T *xs = sx + r * LY::SXH, *fs = sf + r * LY::SXH;
        const int he = (r & 1) * LY::HALF, ho = ((r + 1) & 1) * LY::HALF;
        constexpr int NJ = (NP + 31) / 32;
        T ve[NJ], vo[NJ], fe[NJ], fo[NJ];
        // all loads of the row first, then the shared stores
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const int P = lane + 32 * j, gx = ox + 2 * P;
            ve[j] = vo[j] = fe[j] = fo[j] = (T)0;
            if (P < NP && rin) {
                if (gx >= 0 && gx < n) {
                    if (load_f) fe[j] = fr[gx];
                    if (!zero_x) ve[j] = xr[gx];
                }
                if (gx + 1 >= 0 && gx + 1 < n) {
                    if (load_f) fo[j] = fr[gx + 1];
                    if (!zero_x) vo[j] = xr[gx + 1];
                }
            }
        }
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const int P = lane + 32 * j;
            if (P < NP) {
                xs[he + P] = ve[j];
                xs[ho + P] = vo[j];
                if (load_f) {
                    fs[he + P] = fe[j];
                    fs[ho + P] = fo[j];
                }
            }
        }
    }
}

// NU smoothing sweeps of level l from buffer src into buffer dst.
// zero_init: the level's current solution is zero (a coarse-level
// correction, or the FP32 correction of the defect-correction loop) and is
// not read.  RESTRICT: also form the residual on the tile plus one ring and
// its full weighting (rotann2.f:773-785 summation order) onto the coarse
// points of the tile, which the halo of 2*NU + 2 makes exact.
template <class T, int NU, int CM, bool RESTRICT>
__device__ void op_smooth(const BatchDev &B, TileEntry e, int l, int zero_init, int src, int dst,
                          unsigned char *smem)
{
    constexpr int H = 2 * NU + (RESTRICT ? 2 : 0);
    using LY = TileLayout<T, H>;
    T *sx = (T *)smem, *sf = sx + 2 * LY::HALF;
    const int n = B.n_of[e.p * BP_MAXL + l];
    const int x0 = e.tx * TX, y0 = e.ty * TY, ox = x0 - H, oy = y0 - H;
    tile_load<T, H>(sx, sf, XS<T>(B, e.p, l, src), FP<T>(B, e.p, l), ox, oy, n, zero_init != 0, true);
    __syncthreads();
    tile_sweeps<T, H>(sx, sf, ox, oy, x0, y0, n, H2<T>(B, e.p, l), NU);
    typename CorrVal<CM>::type pv[ST_R * ST_C];
    if (CM != CM_NONE) psi_prefetch((const typename CorrVal<CM>::type *)B.psi[e.p], x0, y0, n, pv);
    tile_store<T, H, CM>(sx, ox, oy, x0, y0, n, XS<T>(B, e.p, l, dst), CM != CM_NONE ? (void *)B.psi[e.p] : nullptr, pv);
    if (RESTRICT) {
        // residual on the tile plus one ring, in place of f (each point
        // reads f only at itself and x, which stays put, so both colours of
        // a row go in one pass: 65 points each, two full passes per colour
        // and one shared pass for the last point of each)
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        const T ih2 = IH2<T>(B, e.p, l);
        const int gxa = x0 - 1, gxb = x0 + TX + 1;
        for (int gy = y0 - 1 + warp; gy <= y0 + TY; gy += nw) {
            const bool rin = gy >= 1 && gy <= n - 2;
            const PhaseRow<T> R0 = phase_row<T, H>(sx, sf, gy, oy, ox, gxa, gxb, 0);
            const PhaseRow<T> R1 = phase_row<T, H>(sx, sf, gy, oy, ox, gxa, gxb, 1);
            auto res_point = [&](const PhaseRow<T> &R, int k) {
                const int gx = 2 * k + R.odd + ox;
                T rv = (T)0;
                if (rin && gx >= 1 && gx <= n - 2) {
                    const T s = (R.N[k - 1 + R.odd] + R.N[k + R.odd]) + (R.N[k - LY::SXH] + R.N[k + LY::SXH]);
                    const T lap = fmaT<T>((T)-4, R.X[k], s);
                    rv = fmaT<T>(-ih2, lap, R.F[k]);
                }
                const_cast<T *>(R.F)[k] = rv;
            };
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int k = R0.k0 + lane + 32 * j;
                if (k < R0.kend) res_point(R0, k);
            }
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int k = R1.k0 + lane + 32 * j;
                if (k < R1.kend) res_point(R1, k);
            }
            const PhaseRow<T> &R = lane < 16 ? R0 : R1;
            const int k = R.k0 + 64 + (lane & 15);
            if (k < R.kend) res_point(R, k);
        }
        __syncthreads();
        const int nc = B.n_of[e.p * BP_MAXL + l + 1];
        T *fc = FP<T>(B, e.p, l + 1);
        const int Ia = max(x0 / 2, 1), Ib = min(x0 / 2 + TX / 2, nc - 1);
        const int Ja = max(y0 / 2, 1), Jb = min(y0 / 2 + TY / 2, nc - 1);
        for (int J = Ja + warp; J < Jb; J += nw) {
            // the fine point (2J, 2I) has even row and column (the tile origin
            // is even): colour 0 at k = I - ox/2; its row and column neighbours
            // are colour 1 at k and k - 1, its diagonals colour 0 at k, k - 1
            const int row = (2 * J - oy) * LY::SXH;
            const T *F0 = sf + row, *F1 = sf + LY::HALF + row;
            const T *F0u = F0 - LY::SXH, *F0d = F0 + LY::SXH, *F1u = F1 - LY::SXH, *F1d = F1 + LY::SXH;
            for (int I = Ia + lane; I < Ib; I += 32) {
                const int k = I - ox / 2;
                T t = F0[k];
                t = t * (T)2 + F1[k] + F1[k - 1];
                t = t + F1d[k] + F1u[k];
                t = t * (T)2 + F0d[k] + F0u[k - 1];
                t = t + F0u[k] + F0d[k - 1];
                fc[(size_t)J * nc + I] = t * (T)0.0625;
            }
        }
    }
    __syncthreads();
}

// Bilinear prolongation of level l+1 (buffer 0) added into level l (buffer
// src) over the tile and its halo (rotann2.f:821-858), then NU
// post-smoothing sweeps, stored into buffer dst (or added to psi: CM).
template <class T, int NU, int CM>
__device__ void op_prolong(const BatchDev &B, TileEntry e, int l, int src, int dst, unsigned char *smem)
{
    constexpr int H = 2 * NU, SX = TX + 2 * H, SY = TY + 2 * H;
    using LY = TileLayout<T, H>;
    T *sx = (T *)smem, *sf = sx + 2 * LY::HALF;
    const int n = B.n_of[e.p * BP_MAXL + l], nc = B.n_of[e.p * BP_MAXL + l + 1];
    const int x0 = e.tx * TX, y0 = e.ty * TY, ox = x0 - H, oy = y0 - H;
    const T *x = XS<T>(B, e.p, l, src);
    const T *f = FP<T>(B, e.p, l);
    const T *ec = XS<T>(B, e.p, l + 1, 0);
    // rows by warp; each lane takes one coarse column and the two fine
    // columns it feeds (the tile origin ox is even, so fine column 2P is
    // even and 2P + 1 odd): one coarse load serves both on an even row, two
    // on an odd row, and the interpolation forms need no parity select.
    // The sums are those of rotann2.f:821-850 in its order.
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int NP = SX / 2;   // coarse columns over the tile and its halo
    for (int r = warp; r < SY; r += TILE_THREADS / 32) {
        const int gy = oy + r;
        const bool rin = gy >= 0 && gy < n, rint = gy >= 1 && gy <= n - 2, yodd = (gy & 1) != 0;
        const size_t base = rin ? (size_t)gy * n : 0;
        const T *xr = x + base, *fr = f + base;
        const T *er = ec + (rint ? (size_t)(gy / 2) * nc : 0);
        T *xs = sx + r * LY::SXH, *fs = sf + r * LY::SXH;
        const int he = (r & 1) * LY::HALF, ho = ((r + 1) & 1) * LY::HALF;   // colour halves of columns 2P, 2P+1
#pragma unroll
        for (int j = 0; j < (NP + 31) / 32; ++j) {
            const int P = lane + 32 * j;
            if (P >= NP) continue;
            const int gx = ox + 2 * P;   // even
            const bool ge = rin && gx >= 0 && gx < n, go = rin && gx + 1 >= 0 && gx + 1 < n;
            const bool ie = ge && rint && gx >= 1 && gx <= n - 2, io = go && rint && gx + 1 >= 1 && gx + 1 <= n - 2;
            T ve = ge ? xr[gx] : (T)0, vo = go ? xr[gx + 1] : (T)0;
            const T fe = (NU > 0 && ge) ? fr[gx] : (T)0, fo = (NU > 0 && go) ? fr[gx + 1] : (T)0;
            if (ie || io) {
                const T *ep = er + (gx / 2);
                const T e00 = ep[0];
                const T e01 = io ? ep[1] : (T)0;
                if (!yodd) {
                    if (ie) ve = ve + e00;
                    if (io) vo = vo + (e00 + e01) * (T)0.5;
                } else {
                    const T e10 = ep[nc];
                    const T e11 = io ? ep[nc + 1] : (T)0;
                    if (ie) ve = ve + (e00 + e10) * (T)0.5;
                    if (io) {
                        T t = e00 + e11;
                        t = t + e10 + e01;
                        vo = vo + t * (T)0.25;
                    }
                }
            }
            xs[he + P] = ve;
            xs[ho + P] = vo;
            if (NU > 0) {
                fs[he + P] = fe;
                fs[ho + P] = fo;
            }
        }
    }
    __syncthreads();
    if (NU > 0) tile_sweeps<T, H>(sx, sf, ox, oy, x0, y0, n, H2<T>(B, e.p, l), NU);
    typename CorrVal<CM>::type pv[ST_R * ST_C];
    if (CM != CM_NONE) psi_prefetch((const typename CorrVal<CM>::type *)B.psi[e.p], x0, y0, n, pv);
    tile_store<T, H, CM>(sx, ox, oy, x0, y0, n, XS<T>(B, e.p, l, dst), CM != CM_NONE ? (void *)B.psi[e.p] : nullptr, pv);
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Coarse levels of one problem in shared memory (one block per problem):
// the V-cycle below level dloc, solution and right-hand side of every level
// resident, residuals formed inside the restriction.
// ---------------------------------------------------------------------------
// One colour of a red-black sweep over the interior: the points of that
// colour only, (m + 1) / 2 slots per row (row j starts at i = 1 or 2).
template <class T>
__device__ void loc_rb_half(T *x, const T *f, int n, T h2, int color)
{
    const int m = n - 2, w = (m + 1) >> 1;
    for (int q = threadIdx.x; q < m * w; q += blockDim.x) {
        const int jj = q / w, j = jj + 1;
        const int i = 1 + ((1 + j + color) & 1) + 2 * (q - jj * w);
        if (i > m) continue;
        const int c = j * n + i;
        const T s = (x[c - 1] + x[c + 1]) + (x[c - n] + x[c + n]);
        x[c] = fmaT<T>(-h2, f[c], s) * (T)0.25;
    }
    __syncthreads();
}

template <class T>
__device__ __forceinline__ T loc_residual(const T *x, const T *f, int n, int c, T ih2)
{
    const T s = (x[c - 1] + x[c + 1]) + (x[c - n] + x[c + n]);
    const T lap = fmaT<T>((T)-4, x[c], s);
    return fmaT<T>(-ih2, lap, f[c]);
}

// zero0: the level-dloc solution starts at zero (a coarse correction, or the
// first inner cycle of a mixed solve); corr0 (dloc == 0 only): add the
// result to the solution instead of storing it, as float pairs or (f64) to
// the FP64 solution.
template <class T>
__device__ void op_local(const BatchDev &B, int p, int nu1, int nu2, int zero_level0, int correct_level0,
                         int f64, unsigned char *smem)
{
    T *sm = (T *)smem;
    const int L = B.nlev[p], d0 = B.dloc[p];
    int off[BP_MAXL];
    int tot = 0;
    for (int l = d0; l < L; ++l) {
        off[l] = tot;
        const int n = B.n_of[p * BP_MAXL + l];
        tot += n * n;
    }
    T *X = sm, *F = sm + tot;
    for (int q = threadIdx.x; q < tot; q += blockDim.x) { X[q] = (T)0; F[q] = (T)0; }
    __syncthreads();
    {
        const bool zero = d0 > 0 || zero_level0;
        const int n = B.n_of[p * BP_MAXL + d0];
        const T *gx = XS<T>(B, p, d0, 0), *gf = FP<T>(B, p, d0);
        for (int q = threadIdx.x; q < n * n; q += blockDim.x) {
            if (!zero) X[q] = gx[q];
            F[q] = gf[q];
        }
    }
    __syncthreads();
    for (int l = d0; l < L - 1; ++l) {
        const int n = B.n_of[p * BP_MAXL + l], nc = B.n_of[p * BP_MAXL + l + 1];
        T *x = X + off[l], *f = F + off[l];
        const T h2 = H2<T>(B, p, l), ih2 = IH2<T>(B, p, l);
        for (int s = 0; s < nu1; ++s) { loc_rb_half(x, f, n, h2, 0); loc_rb_half(x, f, n, h2, 1); }
        T *fc = F + off[l + 1];
        const int mc = nc - 2;
        for (int q = threadIdx.x; q < mc * mc; q += blockDim.x) {
            const int j = q / mc + 1, i = q - (j - 1) * mc + 1;
            const int c = (2 * j) * n + 2 * i;
            T t = loc_residual(x, f, n, c, ih2);
            t = t * (T)2 + loc_residual(x, f, n, c + 1, ih2) + loc_residual(x, f, n, c - 1, ih2);
            t = t + loc_residual(x, f, n, c + n, ih2) + loc_residual(x, f, n, c - n, ih2);
            t = t * (T)2 + loc_residual(x, f, n, c + 1 + n, ih2) + loc_residual(x, f, n, c - 1 - n, ih2);
            t = t + loc_residual(x, f, n, c + 1 - n, ih2) + loc_residual(x, f, n, c - 1 + n, ih2);
            fc[j * nc + i] = t * (T)0.0625;
        }
        __syncthreads();
    }
    {
        const int n = B.n_of[p * BP_MAXL + L - 1];
        loc_rb_half(X + off[L - 1], F + off[L - 1], n, H2<T>(B, p, L - 1), 0);
    }
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
        const T h2 = H2<T>(B, p, l);
        for (int s = 0; s < nu2; ++s) { loc_rb_half(x, f, n, h2, 0); loc_rb_half(x, f, n, h2, 1); }
    }
    {
        const int n = B.n_of[p * BP_MAXL + d0];
        if (d0 == 0 && correct_level0 && f64) {
            double *psi = (double *)B.psi[p];
            for (int q = threadIdx.x; q < n * n; q += blockDim.x) psi[q] = psi[q] + f2d((float)X[q]);
        } else if (d0 == 0 && correct_level0) {
            float2 *psi = (float2 *)B.psi[p];
            for (int q = threadIdx.x; q < n * n; q += blockDim.x) psi[q] = df_add_f(psi[q], (float)X[q]);
        } else {
            T *gx = XS<T>(B, p, d0, 0);
            for (int q = threadIdx.x; q < n * n; q += blockDim.x) gx[q] = X[q];
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Outer pass (residual and norm), convergence bookkeeping
// ---------------------------------------------------------------------------
// One TX x TY tile of level 0 (psi, f: the caller's arrays): the FP64
// residual r = f - A psi, its squared norm (the tile's partial sum) and,
// when store_r, r rounded to FP32 as the inner cycle's right-hand side.
// psi is only read here, so neighbouring tiles may overlap freely.
// OM = CM_NONE (plain FP64 cycles): psi and f are the caller's FP64 arrays
// and the pass forms only the norm.  OM = CM_F64 (FP32 inner cycles, FP64
// defect correction): the same FP64 residual, also stored rounded to FP32
// as the inner cycles' right-hand side.  OM = CM_PAIR: psi is held as float
// pairs in the caller's array and f as float pairs split at the start of
// the solve; the residual is formed in pair arithmetic (rounding error
// about 2^-48 of the terms) and its high part is both the FP32 right-hand
// side and, widened exactly, the term of the FP64 norm.
// FIRST: the first pass of a solve, where psi is zero: the pass reads f
// alone and skips the stencil, with the same bits.  In FP64 the stencil of
// zeros gives lap = +0 and r = fma(-ih2, +0, f) = f exactly.  In pairs it
// gives lap = (+0, +0) and r = f + (-0, -0), which is not always f itself
// (when the low half is exactly half an ulp of the high half the pair sum
// may round the tie the other way), so that sum is still formed.
template <class T, int OM, bool FIRST>
__device__ void op_outer(const BatchDev &B, TileEntry e, int item, const void *const *f_p, int store_r,
                         unsigned char *smem)
{
    constexpr bool PAIR = OM == CM_PAIR;
    using V = typename std::conditional<PAIR, float2, double>::type;
    constexpr int SX = TX + 2, SY = TY + 2;
    V *sp = (V *)smem;
    double *s_red = (double *)(sp + SX * SY);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (!B.active[e.p]) {
        if (threadIdx.x == 0) B.partial[item] = 0.0;
        return;
    }
    const int n = B.n_of[e.p * BP_MAXL];
    const int x0 = e.tx * TX, y0 = e.ty * TY, ox = x0 - 1, oy = y0 - 1;
    const V *psi = (const V *)B.psi[e.p];
    const V *f = (const V *)f_p[e.p];
    V zero;
    if constexpr (PAIR) zero = make_float2(0.f, 0.f);
    else zero = 0.0;
    // rows by warp, a row's loads issued before its shared stores
    if (!FIRST) {
        for (int r = warp; r < SY; r += TILE_THREADS / 32) {
            const int gy = oy + r;
            const bool rin = gy >= 0 && gy < n;
            const V *pr = psi + (rin ? (size_t)gy * n : 0);
            constexpr int NJ = (SX + 31) / 32;
            V v[NJ];
#pragma unroll
            for (int j = 0; j < NJ; ++j) {
                const int c = lane + 32 * j, gx = ox + c;
                v[j] = (c < SX && rin && gx >= 0 && gx < n) ? pr[gx] : zero;
            }
#pragma unroll
            for (int j = 0; j < NJ; ++j) {
                const int c = lane + 32 * j;
                if (c < SX) sp[r * SX + c] = v[j];
            }
        }
        __syncthreads();
    }
    float *f32 = store_r ? FP<float>(B, e.p, 0) : nullptr;
    // one accumulator per column group: the sum of squares is a dependent
    // FP64 chain, and TX / 32 independent chains let the points overlap
    double accs[TX / 32];
#pragma unroll
    for (int a = 0; a < TX / 32; ++a) accs[a] = 0.0;
    const int gxa = max(x0, 1), gxb = min(x0 + TX, n - 1);
    const int gya = max(y0, 1), gyb = min(y0 + TY, n - 1);
    for (int gy0 = gya + warp; gy0 < gyb; gy0 += 2 * nw) {
        // two rows per pass: both rows' f loads are in flight together
        V fr[2][TX / 32];
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int a = 0; a < TX / 32; ++a) {
                const int gy = gy0 + h * nw, gx = x0 + lane + 32 * a;
                fr[h][a] = (gy < gyb && gx >= gxa && gx < gxb) ? f[(size_t)gy * n + gx] : zero;
            }
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int a = 0; a < TX / 32; ++a) {
            const int gy = gy0 + h * nw, gx = x0 + lane + 32 * a;
            if (gy >= gyb || gx < gxa || gx >= gxb) continue;
            const int q = (gy - oy) * SX + gx - ox;
            const size_t g = (size_t)gy * n + gx;
            double rw;
            if constexpr (FIRST) {
                if constexpr (PAIR) {
                    const float2 r = df_add(fr[h][a], make_float2(-0.0f, -0.0f));
                    rw = f2d(r.x);
                    if (store_r) f32[g] = r.x;
                } else {
                    rw = fr[h][a];
                    if (store_r) f32[g] = d2f_rn(rw);
                }
            } else if constexpr (PAIR) {
                // ih2 = 4^m exactly (n = 2^m + 1): every scaling is exact
                const float2 sum = df_add(df_add(sp[q - 1], sp[q + 1]), df_add(sp[q - SX], sp[q + SX]));
                const float2 lap = df_add(sum, df_scale(sp[q], -4.0f));
                const float2 r = df_add(fr[h][a], df_scale(lap, -B.ih2f[e.p * BP_MAXL]));
                rw = f2d(r.x);
                if (store_r) f32[g] = r.x;
            } else {
                const double sum = (sp[q - 1] + sp[q + 1]) + (sp[q - SX] + sp[q + SX]);
                const double lap = __fma_rn(-4.0, sp[q], sum);
                rw = __fma_rn(-B.ih2d[e.p * BP_MAXL], lap, fr[h][a]);
                if (store_r) f32[g] = d2f_rn(rw);
            }
            accs[a] = __fma_rn(rw, rw, accs[a]);
        }
    }
    double acc = 0.0;
#pragma unroll
    for (int a = 0; a < TX / 32; ++a) acc += accs[a];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) s_red[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; ++w) t += s_red[w];
        B.partial[item] = t;
    }
    __syncthreads();
}

// The right-hand side as float pairs (hi = f rounded to FP32, lo = the
// remainder rounded), once per mixed solve; and the solution back from
// pairs to FP64 (hi + lo, exact: the pair spans at most 48 bits) at its end,
// in place.
__global__ void k_split_pairs(const double *f, float2 *out, long long total)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const double v = f[q];
        const float hi = d2f_rn(v);
        out[q] = make_float2(hi, d2f_rn(v - f2d(hi)));
    }
}

__global__ void k_join_pairs(double *psi, long long total)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const float2 v = ((const float2 *)psi)[q];
        psi[q] = f2d(v.x) + f2d(v.y);
    }
}

// Copies buffer 1 of level 0 into the caller's psi (plain FP64 cycles whose
// level-0 operations leave the result in the internal buffer).
__device__ void op_copyback(const BatchDev &B, TileEntry e)
{
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
// A residual norm that is not finite stops the problem as failed (2).
__device__ void op_finalize(const BatchDev &B, int p, int first)
{
    const int lane = threadIdx.x & 31;
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
    if (!(rn <= 1.79769313486231570815e308)) {
        // a NaN or an infinity in the residual (or in f): the problem stops
        B.active[p] = 0;
        B.failed[p] = 2;
    } else if (rn <= B.rtol * fn) {
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
// Operation list.  One outer iteration is a fixed sequence of operations;
// the host builds it once and either launches one kernel per operation
// (captured in a CUDA graph) or hands the whole list to the persistent
// kernel, which runs every operation of every iteration in one launch with
// grid-wide barriers between them.
// ---------------------------------------------------------------------------
enum OpKind { OP_SMOOTH = 0, OP_SMOOTH_R = 1, OP_PROLONG = 2, OP_LOCAL = 3, OP_OUTER = 4, OP_FINALIZE = 5,
              OP_COPYBACK = 6 };
// profile slot of the first outer pass of a solve (reads f alone, no residual
// arithmetic), kept apart from the later passes filed under OP_OUTER
constexpr int OP_PROFILE_OUTER_FIRST = 7;

struct Op {
    int kind, l, nu, zero, src, dst, corr;
    int off, cnt;     // work items: tiles [off, off+cnt) of the tile table, or problems / warps
    int aux;          // OP_LOCAL: zero0 | corr0 << 1; OP_OUTER: store_r; OP_FINALIZE: first
};

// Runs work item `item` of op on this block.  op.corr is the correction
// mode (CM_*) of the operation that applies the defect correction, and of
// the outer pass.
template <class T, int NU, bool RESTRICT>
__device__ __forceinline__ void run_smooth(const BatchDev &B, TileEntry e, const Op &op, unsigned char *smem)
{
    if constexpr (sizeof(T) == 8) op_smooth<T, NU, CM_NONE, RESTRICT>(B, e, op.l, op.zero, op.src, op.dst, smem);
    else if (op.corr == CM_PAIR) op_smooth<T, NU, CM_PAIR, RESTRICT>(B, e, op.l, op.zero, op.src, op.dst, smem);
    else if (op.corr == CM_F64) op_smooth<T, NU, CM_F64, RESTRICT>(B, e, op.l, op.zero, op.src, op.dst, smem);
    else op_smooth<T, NU, CM_NONE, RESTRICT>(B, e, op.l, op.zero, op.src, op.dst, smem);
}
template <class T, int NU>
__device__ __forceinline__ void run_prolong(const BatchDev &B, TileEntry e, const Op &op, unsigned char *smem)
{
    if constexpr (sizeof(T) == 8) op_prolong<T, NU, CM_NONE>(B, e, op.l, op.src, op.dst, smem);
    else if (op.corr == CM_PAIR) op_prolong<T, NU, CM_PAIR>(B, e, op.l, op.src, op.dst, smem);
    else if (op.corr == CM_F64) op_prolong<T, NU, CM_F64>(B, e, op.l, op.src, op.dst, smem);
    else op_prolong<T, NU, CM_NONE>(B, e, op.l, op.src, op.dst, smem);
}

template <class T, bool FIRST>
__device__ __forceinline__ void run_outer(const BatchDev &B, TileEntry e, int item, const double *const *f_p,
                                          const Op &op, unsigned char *smem)
{
    const void *const *fp = (const void *const *)f_p;
    if constexpr (sizeof(T) == 8) op_outer<T, CM_NONE, FIRST>(B, e, item, fp, op.aux, smem);
    else if (op.corr == CM_PAIR) op_outer<T, CM_PAIR, FIRST>(B, e, item, fp, op.aux, smem);
    else if (op.corr == CM_F64) op_outer<T, CM_F64, FIRST>(B, e, item, fp, op.aux, smem);
    else op_outer<T, CM_NONE, FIRST>(B, e, item, fp, op.aux, smem);
}

template <class T>
__device__ __forceinline__ void run_item(const BatchDev &B, const TileEntry *tiles, const double *const *f_p,
                                         const Op &op, int item, int nu1, int nu2, unsigned char *smem)
{
    switch (op.kind) {
    case OP_SMOOTH: {
        const TileEntry e = tiles[op.off + item];
        if (!B.active[e.p]) return;
        if (op.nu == 2) run_smooth<T, 2, false>(B, e, op, smem);
        else run_smooth<T, 1, false>(B, e, op, smem);
        return;
    }
    case OP_SMOOTH_R: {
        const TileEntry e = tiles[op.off + item];
        if (!B.active[e.p]) return;
        if (op.nu == 2) op_smooth<T, 2, CM_NONE, true>(B, e, op.l, op.zero, op.src, op.dst, smem);
        else op_smooth<T, 1, CM_NONE, true>(B, e, op.l, op.zero, op.src, op.dst, smem);
        return;
    }
    case OP_PROLONG: {
        const TileEntry e = tiles[op.off + item];
        if (!B.active[e.p]) return;
        if (op.nu == 2) run_prolong<T, 2>(B, e, op, smem);
        else if (op.nu == 1) run_prolong<T, 1>(B, e, op, smem);
        else run_prolong<T, 0>(B, e, op, smem);
        return;
    }
    case OP_LOCAL:
        if (!B.active[item]) return;
        op_local<T>(B, item, nu1, nu2, op.aux & 1, (op.aux >> 1) & 1, (op.aux >> 2) & 1, smem);
        return;
    case OP_OUTER:
        if (op.nu) run_outer<T, true>(B, tiles[op.off + item], item, f_p, op, smem);
        else run_outer<T, false>(B, tiles[op.off + item], item, f_p, op, smem);
        return;
    case OP_COPYBACK: {
        const TileEntry e = tiles[op.off + item];
        if (B.active[e.p]) op_copyback(B, e);
        return;
    }
    default:
        return;
    }
}

// The coarse levels of every problem below its tiled levels (graph path):
// one block of LOCAL_THREADS per problem.
#define LOCAL_THREADS 512
// Programmatic dependent launch (the graph path's kernels are launched with
// programmatic stream serialization): a kernel may be scheduled while its
// predecessor's last blocks still run, and waits here until that
// predecessor has completed and its writes are visible; it then lets its own
// successor be scheduled.  This hides the launch gap between the
// level-synchronous operations.  Without the attribute both return at once.
__device__ __forceinline__ void grid_dependency_wait()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <class T>
__global__ void __launch_bounds__(LOCAL_THREADS) k_local(BatchDev B, Op op, int nu1, int nu2)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    grid_dependency_wait();
    if (!B.active[blockIdx.x]) return;
    op_local<T>(B, blockIdx.x, nu1, nu2, op.aux & 1, (op.aux >> 1) & 1, (op.aux >> 2) & 1, smem_raw);
}

// One kernel launch per operation (graph path).
// The prolongation variants fit five blocks' shared tiles per SM and are
// held to the registers of five, except those that also apply the defect
// correction (eight more values per thread: held to four, where they need no
// spills); the outer pass is held to four.
template <int KIND, int CM> struct OpMinBlocks {
    static constexpr int value = KIND == OP_PROLONG ? (CM == CM_NONE ? 5 : 4) : (KIND == OP_OUTER ? 4 : 1);
};
template <class T, int KIND, int NU, int CM>
__global__ void __launch_bounds__(TILE_THREADS, (OpMinBlocks<KIND, CM>::value)) k_op(BatchDev B, const TileEntry *tiles, const double *const *f_p,
                                                     Op op, int nu1, int nu2)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    grid_dependency_wait();
    if (KIND == OP_FINALIZE) {
        const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
        if (p < B.nprob) op_finalize(B, p, op.aux);
        return;
    }
    Op o = op;
    o.kind = KIND;
    o.nu = NU;
    o.corr = CM;
    run_item<T>(B, tiles, f_p, o, blockIdx.x, nu1, nu2, smem_raw);
}

// The whole solve in one launch: the first iteration's operations, then
// further iterations until every problem has converged (or hit the cycle
// limit).  Must be launched cooperatively (all blocks resident).
template <class T>
__global__ void __launch_bounds__(TILE_THREADS, 3) k_persistent(BatchDev B, const TileEntry *tiles,
                                                             const double *const *f_p, const Op *ops0, int n0,
                                                             const Op *ops, int nops, int nu1, int nu2,
                                                             int max_iter, GridSync gs)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warps_total = gridDim.x * (blockDim.x >> 5);
    const int gwarp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (int it = 0; it <= max_iter; ++it) {
        const Op *list = it == 0 ? ops0 : ops;
        const int cnt_ops = it == 0 ? n0 : nops;
        for (int k = 0; k < cnt_ops; ++k) {
            const Op op = list[k];
            if (op.kind == OP_OUTER && blockIdx.x == 0 && threadIdx.x == 0) *B.num_active = 0;
            if (op.kind == OP_FINALIZE) {
                for (int p = gwarp; p < B.nprob; p += warps_total) op_finalize(B, p, op.aux);
            } else {
                for (int item = blockIdx.x; item < op.cnt; item += gridDim.x)
                    run_item<T>(B, tiles, f_p, op, item, nu1, nu2, smem_raw);
            }
            if (!grid_sync(gs)) return;
            if (op.kind == OP_FINALIZE && *(volatile int *)B.num_active == 0) return;
        }
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct gb_batch {
    int nprob = 0, precision = 0, nu1 = 2, nu2 = 2, max_cycles = 100;
    int inner = 1;                      // V-cycles per outer iteration (mixed)
    int local_n = LOCAL_N;              // levels with n <= local_n run in one block per problem
    int fuse = 1;                       // red-black sweeps fused into one tile operation (1 or 2)
    int exec = GB_BATCH_EXEC_GRAPH;
    double rtol = 1e-10;
    std::vector<int> n, L, dloc;
    long long total = 0;
    std::vector<long long> off0;        // level-0 offsets in the packed user arrays
    int maxdepth_global = 0;            // levels 0..maxdepth_global-1 have tile work
    void *pool = nullptr;               // per-level x (two buffers), f (T = double or float)
    size_t pool_bytes = 0;
    int *d_int = nullptr;
    double *d_dbl = nullptr;
    void *d_spacing = nullptr;          // h^2 and 1/h^2 per (problem, level): FP64 then FP32
    float2 *d_fpairs = nullptr;         // mixed: the right-hand side as float pairs (total)
    void **d_ptrs = nullptr;
    TileEntry *d_tiles = nullptr;
    std::vector<int> ft_off, ft_cnt;    // per level: tiles of problems with l < dloc
    int ot_off = 0, ot_cnt = 0;         // level-0 tiles of every problem (outer pass)
    BatchDev dev;
    double **d_psi_tab = nullptr, **d_f_tab = nullptr;
    std::vector<void *> hx, hf;
    size_t local_smem = 0;
    int *h_pinned = nullptr;
    double *host_stage = nullptr;       // f and psi of gb_batch_solve_host, allocated on first use
    // pipelined host-buffer solves (gb_batch_submit_host): two slots of f and
    // psi, an upload and a download stream, and the one submitted call whose
    // solve has not run yet
    double *pipe_buf = nullptr;
    cudaStream_t up = nullptr, down = nullptr;
    cudaEvent_t ev_up[2] = {nullptr, nullptr}, ev_solved[2] = {nullptr, nullptr}, ev_down[2] = {nullptr, nullptr};
    int pipe_next = 0;
    bool pend = false;
    int pend_slot = 0;
    double *pend_psi = nullptr, *pend_relres = nullptr;
    int *pend_cycles = nullptr;
    cudaStream_t stream = nullptr;
    // operation lists (first iteration, later iterations) and their device copies
    std::vector<Op> ops0, ops;
    Op *d_ops = nullptr;
    size_t nops_max = 0;
    int plan_inner = -1;
    // persistent launch
    unsigned *d_sync = nullptr;         // count, gen, err
    long long wait_limit = GB_GRID_WAIT_LIMIT_DEFAULT;   // polls a barrier wait may take
    int pgrid = 0;
    size_t psmem = 0;
    // graph path
    cudaGraphExec_t cycle_graph = nullptr;
    long long launches = 0, launches_per_cycle = 0;
    // profiling: CUDA events around every level-0 operation and outer pass
    int profile = 0, graph_profile = -1, graph_ev = 0;
    std::vector<cudaEvent_t> ev;
    std::vector<int> ev_kind;           // operation kind of each recorded event pair
    std::vector<int> graph_kind;        // the same for the captured iteration graph's event pairs
    int ev_used = 0;
    double prof_ms = 0.0, prof_bytes = 0.0;   // persistent launches / the finest-level OP_SMOOTH_R
    long long prof_launches = 0;
    double kind_ms[8] = {0}, kind_bytes[8] = {0};
    long long kind_launches[8] = {0};
    int *h_active = nullptr;            // page-locked: the active flags after a profiled iteration
    int nsm = 0;                        // the device's SMs (grid-stride element-wise launches)
    std::vector<int> prof_prev;         // the flags before it: the problems its outer pass covered
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

// Inner cycles in FP32 (either mixed mode), and the correction mode the
// defect correction applies psi's updates and forms its residual with.
static bool inner32(const gb_batch *b) { return b->precision != GB_BATCH_FP64; }
static int corr_mode(const gb_batch *b)
{
    return b->precision == GB_BATCH_MIXED ? CM_PAIR : b->precision == GB_BATCH_MIXED_F64OUTER ? CM_F64 : CM_NONE;
}

// Two colour-split arrays (x and f) of a tile with halo H (TileLayout).
template <class T> static size_t smem_tile(int H)
{
    const int SXH = (TX + 2 * H) / 2, SY = TY + 2 * H, W = 128 / (int)sizeof(T);
    const size_t half = (size_t)((SY * SXH + W - 1) / W) * W + W / 2;
    return 2 * sizeof(T) * 2 * half;
}
static size_t smem_outer() { return sizeof(double) * ((size_t)(TX + 2) * (TY + 2) + 32); }

template <class T> static size_t smem_of(const gb_batch *b, const Op &op)
{
    switch (op.kind) {
    case OP_SMOOTH: return smem_tile<T>(2 * op.nu);
    case OP_SMOOTH_R: return smem_tile<T>(2 * op.nu + 2);
    case OP_PROLONG: return smem_tile<T>(2 * op.nu);
    case OP_LOCAL: return b->local_smem;
    case OP_OUTER: return smem_outer();
    default: return 0;
    }
}

// Sweeps fused into one smoothing operation (b->fuse, at most 2): by
// default two in FP32; one in FP64, whose pipe is the bottleneck and would
// pay for the wider halo's redundant updates.
static int sweeps_per_op(const gb_batch *b, int nu) { return std::max(1, std::min(nu, b->fuse)); }
static int ops_for(const gb_batch *b, int nu)
{
    int k = 0;
    while (nu > 0) { nu -= sweeps_per_op(b, nu); ++k; }
    return k;
}
// Sweeps of the last pre-smoothing operation (the one that also restricts).
static int sweeps_of_last_pre(const gb_batch *b)
{
    int nu = b->nu1, k = 1;
    while (nu > 0) { k = sweeps_per_op(b, nu); nu -= k; }
    return k;
}

// Operations of one V-cycle.  Tile operations read one buffer of a level
// and write the other; the plan picks the buffers so that every coarse level
// ends in buffer 0 (where the local operation also leaves its levels) and
// the plain solve's level 0 ends in the caller's psi (buffer 0).  Mixed:
// zero0 = the level-0 correction starts at zero (first inner cycle),
// corr0 = the last level-0 operation adds the correction to psi (last inner
// cycle); between inner cycles the correction waits in level-0 buffer *cur0.
template <class T>
static void plan_vcycle(gb_batch *b, std::vector<Op> &v, bool zero0, bool corr0, int *cur0)
{
    const bool mixed = inner32(b);
    const int cm = corr_mode(b);
    int cur[BP_MAXL] = {0};
    const int k1 = ops_for(b, b->nu1);
    const int pro = std::min(b->nu2, b->fuse);  // sweeps fused into the prolongation
    const int k2 = ops_for(b, b->nu2 - pro);
    for (int l = 0; l < b->maxdepth_global; ++l) {
        if (b->ft_cnt[l] == 0) continue;
        const bool zero = l > 0 || (mixed && zero0);
        const int writes = k1 + 1 + k2;
        int src, dst;
        if (zero) { dst = (writes - 1) & 1; src = 1 - dst; }
        else if (mixed) { src = *cur0; dst = 1 - src; }    // level 0, later inner cycle
        else { src = 0; dst = 1; }                         // level 0 of the plain solve: psi
        int nu = b->nu1;
        for (int i = 0; i < k1; ++i) {
            const int k = sweeps_per_op(b, nu);
            Op o{};
            o.kind = (i == k1 - 1) ? OP_SMOOTH_R : OP_SMOOTH;
            o.l = l; o.nu = k; o.zero = (zero && i == 0) ? 1 : 0; o.src = src; o.dst = dst; o.corr = 0;
            o.off = b->ft_off[l]; o.cnt = b->ft_cnt[l];
            v.push_back(o);
            nu -= k;
            src = dst;
            dst = 1 - dst;
        }
        cur[l] = src;
    }
    {
        Op o{};
        o.kind = OP_LOCAL;
        o.cnt = b->nprob;
        o.aux = ((mixed && zero0) ? 1 : 0) | ((mixed && corr0) ? 2 : 0) | (cm == CM_F64 ? 4 : 0);
        v.push_back(o);
    }
    for (int l = b->maxdepth_global - 1; l >= 0; --l) {
        if (b->ft_cnt[l] == 0) continue;
        const int correct_last = (mixed && l == 0 && corr0) ? cm : CM_NONE;
        int src = cur[l], dst = 1 - cur[l];
        Op o{};
        o.kind = OP_PROLONG; o.l = l; o.nu = pro; o.src = src; o.dst = dst;
        o.corr = k2 == 0 ? correct_last : CM_NONE;
        o.off = b->ft_off[l]; o.cnt = b->ft_cnt[l];
        v.push_back(o);
        src = dst;
        dst = 1 - dst;
        int nu = b->nu2 - pro;
        for (int i = 0; i < k2; ++i) {
            const int k = sweeps_per_op(b, nu);
            Op q{};
            q.kind = OP_SMOOTH; q.l = l; q.nu = k; q.zero = 0; q.src = src; q.dst = dst;
            q.corr = (i == k2 - 1) ? correct_last : CM_NONE;
            q.off = b->ft_off[l]; q.cnt = b->ft_cnt[l];
            v.push_back(q);
            nu -= k;
            src = dst;
            dst = 1 - dst;
        }
        cur[l] = src;
        if (!mixed && l == 0 && cur[0] != 0) {
            Op c{};
            c.kind = OP_COPYBACK; c.off = b->ft_off[0]; c.cnt = b->ft_cnt[0];
            v.push_back(c);
        }
    }
    if (mixed) *cur0 = cur[0];
}

// One outer iteration: the FP64 residual norm of level 0 (mixed: also its
// FP32 copy as the inner right-hand side), convergence bookkeeping, then
// b->inner V-cycles (mixed: the last one's final level-0 operation adds the
// correction to psi).
template <class T>
static void plan_iteration(gb_batch *b, std::vector<Op> &v, int first)
{
    v.clear();
    const bool mixed = inner32(b);
    Op o{};
    o.kind = OP_OUTER; o.off = b->ot_off; o.cnt = b->ot_cnt; o.aux = mixed ? 1 : 0; o.corr = corr_mode(b);
    o.nu = first ? 1 : 0;   // the first pass of a solve: psi = 0
    v.push_back(o);
    Op f{};
    f.kind = OP_FINALIZE; f.cnt = b->nprob; f.aux = first;
    v.push_back(f);
    int cur0 = 0;
    const int inner = mixed ? b->inner : 1;
    for (int k = 0; k < inner; ++k) plan_vcycle<T>(b, v, k == 0, k == inner - 1, &cur0);
}

static void build_plans(gb_batch *b)
{
    if (inner32(b)) {
        plan_iteration<float>(b, b->ops0, 1);
        plan_iteration<float>(b, b->ops, 0);
    } else {
        plan_iteration<double>(b, b->ops0, 1);
        plan_iteration<double>(b, b->ops, 0);
    }
    b->plan_inner = b->inner;
}

// Correction modes a kernel of inner precision T is built for: the plain
// FP64 solve never corrects; the FP32 inner cycles correct psi as float
// pairs or in FP64.
template <class T, int KIND, int NU>
static cudaError_t smem_attr_cm(size_t sz)
{
    cudaError_t e = cudaFuncSetAttribute(k_op<T, KIND, NU, CM_NONE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sz);
    if constexpr (sizeof(T) == 4) {
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_op<T, KIND, NU, CM_PAIR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sz);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_op<T, KIND, NU, CM_F64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sz);
    }
    return e;
}

template <class T> static cudaError_t set_smem_attrs(size_t local, size_t persistent)
{
    cudaError_t e;
#define SA(call) if ((e = (call)) != cudaSuccess) return e
    SA((smem_attr_cm<T, OP_SMOOTH, 1>(smem_tile<T>(2))));
    SA((smem_attr_cm<T, OP_SMOOTH, 2>(smem_tile<T>(4))));
    SA((cudaFuncSetAttribute(k_op<T, OP_SMOOTH_R, 1, CM_NONE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_tile<T>(4))));
    SA((cudaFuncSetAttribute(k_op<T, OP_SMOOTH_R, 2, CM_NONE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_tile<T>(6))));
    SA((smem_attr_cm<T, OP_PROLONG, 0>(smem_tile<T>(0))));
    SA((smem_attr_cm<T, OP_PROLONG, 1>(smem_tile<T>(2))));
    SA((smem_attr_cm<T, OP_PROLONG, 2>(smem_tile<T>(4))));
    SA((smem_attr_cm<T, OP_OUTER, 0>(smem_outer())));
    SA((smem_attr_cm<T, OP_OUTER, 1>(smem_outer())));
    SA((cudaFuncSetAttribute(k_local<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)local)));
    SA((cudaFuncSetAttribute(k_persistent<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)persistent)));
#undef SA
    return cudaSuccess;
}

// A kernel launch with programmatic stream serialization (see
// grid_dependency_wait).
template <typename... P, typename... A>
static void launch_pdl(void (*k)(P...), int grid, int block, size_t sm, cudaStream_t s, A... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = sm;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, ((P)args)...);
}

// Launches k_op<T, KIND, NU, cm> (graph path).
template <class T, int KIND, int NU>
static void launch_k(const gb_batch *b, int cm, int g, size_t sm, cudaStream_t s, const Op &op)
{
    const TileEntry *t = b->d_tiles;
    const double *const *fp = (const double *const *)b->d_f_tab;
    const int n1 = b->nu1, n2 = b->nu2;
    if constexpr (sizeof(T) == 4) {
        if (cm == CM_PAIR) { launch_pdl(k_op<T, KIND, NU, CM_PAIR>, g, TILE_THREADS, sm, s, b->dev, t, fp, op, n1, n2); return; }
        if (cm == CM_F64) { launch_pdl(k_op<T, KIND, NU, CM_F64>, g, TILE_THREADS, sm, s, b->dev, t, fp, op, n1, n2); return; }
    }
    launch_pdl(k_op<T, KIND, NU, CM_NONE>, g, TILE_THREADS, sm, s, b->dev, t, fp, op, n1, n2);
}

// Launches one operation as its own kernel (graph path).
template <class T>
static void launch_op(gb_batch *b, const Op &op, cudaStream_t s)
{
    const size_t sm = smem_of<T>(b, op);
    const int g = op.cnt;
    if (g <= 0) return;
    switch (op.kind) {
    case OP_SMOOTH:
        if (op.nu == 2) launch_k<T, OP_SMOOTH, 2>(b, op.corr, g, sm, s, op);
        else launch_k<T, OP_SMOOTH, 1>(b, op.corr, g, sm, s, op);
        break;
    case OP_SMOOTH_R:
        if (op.nu == 2) launch_k<T, OP_SMOOTH_R, 2>(b, CM_NONE, g, sm, s, op);
        else launch_k<T, OP_SMOOTH_R, 1>(b, CM_NONE, g, sm, s, op);
        break;
    case OP_PROLONG:
        if (op.nu == 2) launch_k<T, OP_PROLONG, 2>(b, op.corr, g, sm, s, op);
        else if (op.nu == 1) launch_k<T, OP_PROLONG, 1>(b, op.corr, g, sm, s, op);
        else launch_k<T, OP_PROLONG, 0>(b, op.corr, g, sm, s, op);
        break;
    case OP_LOCAL:
        launch_pdl(k_local<T>, g, LOCAL_THREADS, sm, s, b->dev, op, b->nu1, b->nu2);
        break;
    case OP_OUTER:
        if (op.nu) launch_k<T, OP_OUTER, 1>(b, op.corr, g, sm, s, op);
        else launch_k<T, OP_OUTER, 0>(b, op.corr, g, sm, s, op);
        break;
    case OP_FINALIZE:
        launch_k<T, OP_FINALIZE, 0>(b, CM_NONE, gb_ceil_div(b->nprob, TILE_THREADS / 32), 0, s, op);
        break;
    case OP_COPYBACK:
        launch_k<T, OP_COPYBACK, 0>(b, CM_NONE, g, 0, s, op);
        break;
    }
    b->launches += 1;
}

// Creates a handle with every tunable given (gb_batch_create passes the
// defaults, gb_batch_create_tuned an autotuner's choice).
static int batch_create(int nprob, const int *n, int precision, int nu1, int nu2, double rtol, int max_cycles,
                        int local_n, int fuse, int inner, int exec, gb_batch **out)
{
    if (!out || !n || nprob <= 0 ||
        (precision != GB_BATCH_FP64 && precision != GB_BATCH_MIXED && precision != GB_BATCH_MIXED_F64OUTER) || nu1 < 1 ||
        nu1 > 8 || nu2 < 0 || nu2 > 8 || max_cycles < 0 || !(rtol >= 0.0)) {
        gb_set_error("gb_batch_create: invalid argument (need nprob > 0, 1 <= nu1 <= 8, 0 <= nu2 <= 8)");
        return GB_ERR_INVALID;
    }
    const int local_max = precision == GB_BATCH_FP64 ? 65 : 129;
    if ((local_n != 33 && local_n != 65 && local_n != 129) || local_n > local_max || fuse < 1 || fuse > 2 ||
        inner < 1 || inner > 16 || (precision == GB_BATCH_FP64 && inner != 1) ||
        (exec != GB_BATCH_EXEC_GRAPH && exec != GB_BATCH_EXEC_PERSISTENT)) {
        gb_set_error("gb_batch_create: invalid tuning (local_n 33, 65 or 129 (65 at most in FP64), fuse 1..2, "
                     "inner 1..16 (1 in FP64), exec GRAPH or PERSISTENT)");
        return GB_ERR_INVALID;
    }
    *out = nullptr;
    gb_batch *b = new gb_batch();
    b->nprob = nprob;
    b->precision = precision;
    b->nu1 = nu1;
    b->nu2 = nu2;
    b->local_n = local_n;
    b->fuse = fuse;
    b->inner = inner;
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
        while (nl[d] > b->local_n) ++d;
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
        smax = std::max(smax, 2 * sz * esz);
    }
    b->local_smem = smax;
    // tile tables
    std::vector<TileEntry> tiles;
    b->ft_off.assign(BP_MAXL + 1, 0);
    b->ft_cnt.assign(BP_MAXL + 1, 0);
    std::vector<int> pb0(nprob), pnb0(nprob);
    auto add_tiles = [&](int p, int nn) {
        for (int ty = 0; ty * TY < nn - 1; ++ty)
            for (int tx = 0; tx * TX < nn - 1; ++tx) tiles.push_back({p, (short)tx, (short)ty});
    };
    for (int l = 0; l < BP_MAXL; ++l) {
        b->ft_off[l] = (int)tiles.size();
        for (int p = 0; p < nprob; ++p)
            if (l < b->dloc[p]) add_tiles(p, nof[(size_t)p * BP_MAXL + l]);
        b->ft_cnt[l] = (int)tiles.size() - b->ft_off[l];
    }
    b->ot_off = (int)tiles.size();
    for (int p = 0; p < nprob; ++p) {
        pb0[p] = (int)tiles.size() - b->ot_off;
        add_tiles(p, n[p]);
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
    const size_t nsp = (size_t)nprob * BP_MAXL;
    BTRY(cudaMalloc(&b->d_spacing, (sizeof(double) + sizeof(float)) * 2 * nsp));
    if (precision == GB_BATCH_MIXED) BTRY(cudaMalloc(&b->d_fpairs, sizeof(float2) * (size_t)std::max<long long>(b->total, 1)));
    {
        std::vector<double> hd(2 * nsp, 0.0);
        std::vector<float> hf(2 * nsp, 0.0f);
        for (size_t k = 0; k < nsp; ++k) {
            const int m = nof[k];
            if (m < 2) continue;
            const double h = 1.0 / (double)(m - 1);
            hd[k] = h * h;
            hd[nsp + k] = 1.0 / hd[k];
            const float hs = 1.0f / (float)(m - 1);
            hf[k] = hs * hs;
            hf[nsp + k] = 1.0f / hf[k];
        }
        BTRY(cudaMemcpy(b->d_spacing, hd.data(), sizeof(double) * 2 * nsp, cudaMemcpyHostToDevice));
        BTRY(cudaMemcpy((char *)b->d_spacing + sizeof(double) * 2 * nsp, hf.data(), sizeof(float) * 2 * nsp,
                        cudaMemcpyHostToDevice));
    }
    // pointer tables: x (two buffers per level), f (one per level), psi and f of level 0
    const size_t nptr = 2 * (size_t)nprob * BP_MAXL + (size_t)nprob * BP_MAXL + 2 * (size_t)nprob;
    BTRY(cudaMalloc(&b->d_ptrs, sizeof(void *) * nptr));
    BTRY(cudaMalloc(&b->d_tiles, sizeof(TileEntry) * tiles.size()));
    BTRY(cudaMalloc(&b->d_sync, sizeof(unsigned) * 4));
    BTRY(cudaMemset(b->d_sync, 0, sizeof(unsigned) * 4));
    BTRY(cudaMallocHost(&b->h_pinned, sizeof(int) * 16));
    BTRY(cudaMallocHost(&b->h_active, sizeof(int) * (size_t)nprob));
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
    D.h2d = (const double *)b->d_spacing;
    D.ih2d = D.h2d + nsp;
    D.h2f = (const float *)(D.h2d + 2 * nsp);
    D.ih2f = D.h2f + nsp;
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
    D.inner = b->inner;
    D.rtol = rtol;
    // persistent launch: shared memory of the largest operation, grid of
    // every block that can be resident at once
    build_plans(b);
    size_t ps = b->local_smem;
    for (const Op &o : b->ops)
        ps = std::max(ps, precision == GB_BATCH_FP64 ? smem_of<double>(b, o) : smem_of<float>(b, o));
    b->psmem = ps;
    if (precision == GB_BATCH_FP64) BTRY(set_smem_attrs<double>(b->local_smem, b->psmem));
    else BTRY(set_smem_attrs<float>(b->local_smem, b->psmem));
    int dev = 0, nsm = 0, per = 0, coop = 0;
    BTRY(cudaGetDevice(&dev));
    BTRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    BTRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (precision == GB_BATCH_FP64) BTRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_persistent<double>, TILE_THREADS, b->psmem));
    else BTRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_persistent<float>, TILE_THREADS, b->psmem));
    b->nsm = nsm;
    b->pgrid = nsm * per;
    if (!coop) b->pgrid = 0;
    // room for the operation lists of any inner count (set_inner_cycles)
    const size_t nops_max = 4 * (b->ops.size() + 8) * 16;
    BTRY(cudaMalloc(&b->d_ops, sizeof(Op) * nops_max));
    b->nops_max = nops_max;
#undef BTRY
    if (exec == GB_BATCH_EXEC_PERSISTENT && b->pgrid <= 0) {
        gb_set_error("gb_batch_create: cooperative launch unavailable on this device");
        gb_batch_destroy(b);
        return GB_ERR_INVALID;
    }
    b->exec = exec;
    *out = b;
    return GB_OK;
}

extern "C" int gb_batch_create(int nprob, const int *n, int precision, int nu1, int nu2, double rtol,
                               int max_cycles, gb_batch **out)
{
    return batch_create(nprob, n, precision, nu1, nu2, rtol, max_cycles, LOCAL_N,
                        precision == GB_BATCH_FP64 ? 1 : 2, 1, GB_BATCH_EXEC_GRAPH, out);
}

extern "C" int gb_batch_create_tuned(int nprob, const int *n, int precision, double rtol, int max_cycles,
                                     const gb_batch_tuning *t, gb_batch **out)
{
    if (!t) {
        gb_set_error("gb_batch_create_tuned: null tuning");
        return GB_ERR_INVALID;
    }
    return batch_create(nprob, n, precision, t->nu1, t->nu2, rtol, max_cycles, t->local_n, t->fuse, t->inner,
                        t->exec, out);
}

extern "C" int gb_batch_destroy(gb_batch *b)
{
    if (!b) return GB_OK;
    if (b->cycle_graph) cudaGraphExecDestroy(b->cycle_graph);
    for (auto &e : b->ev) cudaEventDestroy(e);
    cudaFree(b->pool);
    cudaFree(b->d_int);
    cudaFree(b->d_dbl);
    cudaFree(b->d_spacing);
    cudaFree(b->d_fpairs);
    cudaFree(b->d_ptrs);
    cudaFree(b->d_tiles);
    cudaFree(b->d_ops);
    cudaFree(b->d_sync);
    cudaFree(b->host_stage);
    if (b->up) cudaStreamSynchronize(b->up);
    if (b->down) cudaStreamSynchronize(b->down);
    for (int i = 0; i < 2; ++i) {
        if (b->ev_up[i]) cudaEventDestroy(b->ev_up[i]);
        if (b->ev_solved[i]) cudaEventDestroy(b->ev_solved[i]);
        if (b->ev_down[i]) cudaEventDestroy(b->ev_down[i]);
    }
    if (b->up) cudaStreamDestroy(b->up);
    if (b->down) cudaStreamDestroy(b->down);
    cudaFree(b->pipe_buf);
    if (b->h_pinned) cudaFreeHost(b->h_pinned);
    if (b->h_active) cudaFreeHost(b->h_active);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return GB_OK;
}

extern "C" long long gb_batch_total_points(const gb_batch *b) { return b ? b->total : 0; }
extern "C" long long gb_batch_last_launches(const gb_batch *b) { return b ? b->launches : 0; }

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
    build_plans(b);
    if (b->nops_max < b->ops0.size() + b->ops.size()) {
        gb_set_error("gb_batch_set_inner_cycles: operation list too long");
        return GB_ERR_INVALID;
    }
    return GB_OK;
}

extern "C" int gb_batch_set_wait_limit(gb_batch *b, long long polls)
{
    if (!b || polls < 0) {
        gb_set_error("gb_batch_set_wait_limit: need a handle and polls >= 0");
        return GB_ERR_INVALID;
    }
    b->wait_limit = polls;
    return GB_OK;
}

extern "C" int gb_batch_set_exec(gb_batch *b, int mode)
{
    if (!b || (mode != GB_BATCH_EXEC_GRAPH && mode != GB_BATCH_EXEC_PERSISTENT)) {
        gb_set_error("gb_batch_set_exec: mode must be GB_BATCH_EXEC_GRAPH or GB_BATCH_EXEC_PERSISTENT");
        return GB_ERR_INVALID;
    }
    if (mode == GB_BATCH_EXEC_PERSISTENT && b->pgrid <= 0) {
        gb_set_error("gb_batch_set_exec: cooperative launch unavailable on this device");
        return GB_ERR_INVALID;
    }
    b->exec = mode;
    return GB_OK;
}

// Records a timing event: as an event node of the graph while the stream is
// being captured, as a plain record otherwise.
static void prof_record(cudaEvent_t e, cudaStream_t s)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cs);
    if (cs == cudaStreamCaptureStatusActive) cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    else cudaEventRecord(e, s);
}

// Graph path: the operations of one iteration, each its own kernel; the
// finest-level pre-smoothing operation (the largest FP32 kernel) is
// bracketed by timing events when profiling.
static void enqueue_iteration(gb_batch *b, const std::vector<Op> &v, cudaStream_t s)
{
    cudaMemsetAsync(b->dev.num_active, 0, sizeof(int), s);
    for (const Op &op : v) {
        const bool timed = (op.l == 0 && op.kind != OP_FINALIZE && op.kind != OP_LOCAL) || op.kind == OP_OUTER;
        const bool ev = b->profile && timed && b->ev_used + 2 <= (int)b->ev.size();
        if (ev) prof_record(b->ev[b->ev_used], s);
        if (inner32(b)) launch_op<float>(b, op, s);
        else launch_op<double>(b, op, s);
        if (ev) {
            prof_record(b->ev[b->ev_used + 1], s);
            b->ev_kind[b->ev_used / 2] = op.kind | (op.kind == OP_OUTER && op.nu ? 0x100 : 0);
            b->ev_used += 2;
        }
    }
    cudaMemcpyAsync(b->h_pinned, b->dev.num_active, sizeof(int), cudaMemcpyDeviceToHost, s);
    // profiled iterations also bring back the active flags (part of the
    // graph: read after the iteration's own synchronisation)
    if (b->profile) cudaMemcpyAsync(b->h_active, b->dev.active, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost, s);
}

// Algorithmic bytes of one V-cycle per interior point (24.7 words: four
// sweeps of 3 words, residual 3, restriction 1.25, prolongation 2.25, all
// levels x 4/3) at the inner precision, and of one outer step (read psi
// and f, 8 B each as FP64 or float pairs, write the FP32 residual; read e,
// read and write psi).
static double cycle_bytes(const gb_batch *b) { return 24.7 * (b->precision == GB_BATCH_FP64 ? 8.0 : 4.0); }
static double outer_bytes(const gb_batch *b) { return b->precision == GB_BATCH_FP64 ? 16.0 : 40.0; }

// Graph path, after an iteration: adds the recorded times per operation kind
// and each operation's algorithmic bytes for the problems that took part.
// Per interior point (words of the inner precision unless noted):
//   OP_SMOOTH_R  sweeps x 3 (psi read, f read, psi written) + residual 3 +
//                restriction 1.25;
//   OP_PROLONG   prolongation 2.25 + sweeps x 3 (+ 16 B of psi when it
//                applies the correction);
//   OP_SMOOTH    sweeps x 3;
//   OP_OUTER     FP64 psi and f read (16 B) + FP32 residual written (4 B);
//                the first pass of a solve reads f alone (12 B).
static void batch_profile_collect(gb_batch *b, cudaStream_t s)
{
    if (!b->profile || b->ev_used == 0) return;
    cudaStreamSynchronize(s);   // a no-op after the iteration's own synchronisation
    // the outer pass runs before the iteration's convergence test and covers
    // the problems active when the iteration began; the cycles after the
    // test cover those still active when it ends
    double pts_tile = 0.0, pts_outer = 0.0;
    for (int p = 0; p < b->nprob; ++p) {
        const double pts = (double)(b->n[p] - 2) * (double)(b->n[p] - 2);
        if (b->prof_prev[p]) pts_outer += pts;
        if (b->h_active[p] && b->dloc[p] > 0) pts_tile += pts;
    }
    const double esz = b->precision == GB_BATCH_FP64 ? 8.0 : 4.0;
    const bool mixed = inner32(b);
    const int pre = sweeps_of_last_pre(b);
    const int post = std::min(b->nu2, b->fuse);
    for (int i = 0; i + 1 < b->ev_used; i += 2) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, b->ev[i], b->ev[i + 1]) != cudaSuccess) {
            cudaGetLastError();  // timing is advisory: never let it fail a solve
            continue;
        }
        const int k = b->ev_kind[i / 2] & 0xff;
        const bool first_outer = (b->ev_kind[i / 2] & 0x100) != 0;
        double bytes = 0.0;
        switch (k) {
        case OP_SMOOTH_R: bytes = (3.0 * pre + 3.0 + 1.25) * esz * pts_tile; break;
        case OP_PROLONG: bytes = ((2.25 + 3.0 * post) * esz + (mixed ? 16.0 : 0.0)) * pts_tile; break;
        case OP_SMOOTH: bytes = 3.0 * esz * pts_tile; break;
        case OP_OUTER: bytes = (first_outer ? 12.0 : 20.0) * pts_outer; break;   // the first reads f alone
        default: break;
        }
        const int slot = first_outer ? OP_PROFILE_OUTER_FIRST : k;   // first passes apart
        b->kind_ms[slot] += ms;
        b->kind_bytes[slot] += bytes;
        b->kind_launches[slot] += 1;
        if (k == OP_SMOOTH_R) {
            b->prof_ms += ms;
            b->prof_launches += 1;
            b->prof_bytes += bytes;
        }
    }
    b->prof_prev.assign(b->h_active, b->h_active + b->nprob);
}

extern "C" int gb_batch_profile(gb_batch *b, int enable)
{
    if (!b) return GB_ERR_INVALID;
    if (enable && b->ev.empty()) {
        b->ev.resize(2 * (4 * b->inner + 8));
        b->ev_kind.assign(b->ev.size() / 2, 0);
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
        for (int k = 0; k < 8; ++k) {
            b->kind_ms[k] = 0.0;
            b->kind_bytes[k] = 0.0;
            b->kind_launches[k] = 0;
        }
    }
    return GB_OK;
}

extern "C" int gb_batch_profile_read_kind(gb_batch *b, int kind, double *ms, long long *launches, double *alg_bytes)
{
    if (!b || kind < 0 || kind >= 8) return GB_ERR_INVALID;
    if (ms) *ms = b->kind_ms[kind];
    if (launches) *launches = b->kind_launches[kind];
    if (alg_bytes) *alg_bytes = b->kind_bytes[kind];
    return GB_OK;
}

static int batch_bind_io(gb_batch *b, const double *d_f, double *d_psi, cudaStream_t s)
{
    std::vector<const void *> pf(b->nprob), pp(b->nprob);
    const bool mixed = b->precision == GB_BATCH_MIXED;   // float-pair right-hand side
    for (int p = 0; p < b->nprob; ++p) {
        pf[p] = mixed ? (const void *)(b->d_fpairs + b->off0[p]) : (const void *)(d_f + b->off0[p]);
        pp[p] = d_psi + b->off0[p];
    }
    if (mixed && b->total > 0) {
        k_split_pairs<<<b->nsm * 8, 256, 0, s>>>(d_f, b->d_fpairs, b->total);
        GB_CUDA_TRY(cudaGetLastError());
    }
    GB_CUDA_TRY(cudaMemcpyAsync(b->d_f_tab, pf.data(), sizeof(void *) * b->nprob, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemcpyAsync(b->d_psi_tab, pp.data(), sizeof(void *) * b->nprob, cudaMemcpyHostToDevice, s));
    if (b->precision == GB_BATCH_FP64) {
        // level-0 x (buffer 0) and f of the plain cycle are the caller's arrays
        for (int p = 0; p < b->nprob; ++p) {
            b->hx[(size_t)p * BP_MAXL] = d_psi + b->off0[p];
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

static int solve_graph(gb_batch *b, cudaStream_t s)
{
    b->ev_used = 0;
    b->prof_prev.assign(b->nprob, 1);   // every problem starts active
    enqueue_iteration(b, b->ops0, s);
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
        enqueue_iteration(b, b->ops, cs);
        GB_CUDA_TRY(cudaStreamEndCapture(cs, &g));
        b->launches_per_cycle = b->launches - l0;
        b->launches = l0;
        GB_CUDA_TRY(cudaGraphInstantiate(&b->cycle_graph, g, 0));
        cudaGraphDestroy(g);
        b->graph_profile = b->profile;
        b->graph_ev = b->ev_used;
        b->graph_kind.assign(b->ev_kind.begin(), b->ev_kind.begin() + b->ev_used / 2);
    }
    for (int it = 0; it <= b->max_cycles + 1 && *b->h_pinned > 0; ++it) {
        GB_CUDA_TRY(cudaGraphLaunch(b->cycle_graph, s));
        b->launches += b->launches_per_cycle;
        GB_CUDA_TRY(cudaStreamSynchronize(s));
        // the first iteration of each solve (run outside the graph) rewrote
        // ev_kind: classify the replay's events by the kinds captured with it
        std::copy(b->graph_kind.begin(), b->graph_kind.end(), b->ev_kind.begin());
        b->ev_used = b->graph_ev;
        batch_profile_collect(b, s);
    }
    return GB_OK;
}

static int solve_persistent(gb_batch *b, cudaStream_t s)
{
    const int n0 = (int)b->ops0.size(), n1 = (int)b->ops.size();
    GB_CUDA_TRY(cudaMemcpyAsync(b->d_ops, b->ops0.data(), sizeof(Op) * n0, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemcpyAsync(b->d_ops + n0, b->ops.data(), sizeof(Op) * n1, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemsetAsync(b->d_sync, 0, sizeof(unsigned) * 4, s));
    GridSync gs;
    gs.count = b->d_sync;
    gs.gen = b->d_sync + 1;
    gs.err = (int *)(b->d_sync + 2);
    gs.limit = b->wait_limit;
    gs.tally = nullptr;
    const Op *ops0 = b->d_ops, *ops = b->d_ops + n0;
    const TileEntry *tiles = b->d_tiles;
    const double *const *fp = (const double *const *)b->d_f_tab;
    int nu1 = b->nu1, nu2 = b->nu2;
    int max_iter = b->max_cycles / std::max(1, b->inner) + 2;
    BatchDev D = b->dev;
    void *args[] = {&D, &tiles, &fp, &ops0, (void *)&n0, &ops, (void *)&n1, &nu1, &nu2, &max_iter, &gs};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (b->profile && b->ev.size() >= 2) {
        e0 = b->ev[0];
        e1 = b->ev[1];
        cudaEventRecord(e0, s);
    }
    cudaError_t err;
    if (b->precision == GB_BATCH_FP64)
        err = cudaLaunchCooperativeKernel((void *)k_persistent<double>, b->pgrid, TILE_THREADS, args, b->psmem, s);
    else
        err = cudaLaunchCooperativeKernel((void *)k_persistent<float>, b->pgrid, TILE_THREADS, args, b->psmem, s);
    if (err != cudaSuccess) {
        gb_set_error("persistent launch (%d blocks, %zu B shared): %s", b->pgrid, b->psmem, cudaGetErrorString(err));
        return GB_ERR_CUDA;
    }
    b->launches += 1;
    if (e1) cudaEventRecord(e1, s);
    unsigned sync[4];
    GB_CUDA_TRY(cudaMemcpyAsync(sync, b->d_sync, sizeof(sync), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (sync[2]) {
        gb_set_error("persistent solve: a grid barrier wait timed out");
        return GB_TIMEOUT;
    }
    if (e1) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) {
            std::vector<int> cyc(b->nprob);
            cudaMemcpy(cyc.data(), b->dev.cycles, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost);
            double bytes = 0.0;
            for (int p = 0; p < b->nprob; ++p) {
                const double pts = (double)(b->n[p] - 2) * (double)(b->n[p] - 2);
                const int outer = cyc[p] / std::max(1, b->inner) + 1;
                bytes += pts * (cyc[p] * cycle_bytes(b) + outer * outer_bytes(b));
            }
            b->prof_ms += ms;
            b->prof_launches += 1;
            b->prof_bytes += bytes;
        } else {
            cudaGetLastError();
        }
    }
    return GB_OK;
}

extern "C" int gb_batch_solve_device(gb_batch *b, const double *d_f, double *d_psi, int *cycles, double *relres,
                                     void *stream)
{
    if (!b || !d_f || !d_psi) { gb_set_error("gb_batch_solve_device: null argument"); return GB_ERR_INVALID; }
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    BatchDev &D = b->dev;
    b->launches = 0;
    if (b->plan_inner != b->inner) build_plans(b);
    int st = batch_bind_io(b, d_f, d_psi, s);
    if (st != GB_OK) return st;
    GB_CUDA_TRY(cudaMemsetAsync(d_psi, 0, sizeof(double) * (size_t)b->total, s));
    std::vector<int> ones(b->nprob, 1);
    GB_CUDA_TRY(cudaMemcpyAsync(D.active, ones.data(), sizeof(int) * b->nprob, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemsetAsync(D.cycles, 0, sizeof(int) * b->nprob, s));
    GB_CUDA_TRY(cudaMemsetAsync(D.failed, 0, sizeof(int) * b->nprob, s));
    st = b->exec == GB_BATCH_EXEC_PERSISTENT ? solve_persistent(b, s) : solve_graph(b, s);
    if (st != GB_OK) return st;
    if (b->precision == GB_BATCH_MIXED && b->total > 0) {
        // the mixed solve held psi as float pairs in place: back to FP64
        k_join_pairs<<<b->nsm * 8, 256, 0, s>>>(d_psi, b->total);
        GB_CUDA_TRY(cudaGetLastError());
    }
    std::vector<int> fl(b->nprob);
    GB_CUDA_TRY(cudaMemcpyAsync(fl.data(), D.failed, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost, s));
    if (cycles) GB_CUDA_TRY(cudaMemcpyAsync(cycles, D.cycles, sizeof(int) * b->nprob, cudaMemcpyDeviceToHost, s));
    if (relres) GB_CUDA_TRY(cudaMemcpyAsync(relres, D.relres, sizeof(double) * b->nprob, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    GB_CUDA_TRY(cudaGetLastError());
    int st_out = GB_OK;
    for (int p = 0; p < b->nprob; ++p) {
        if (fl[p] == 2) {
            gb_set_error("gb_batch_solve: problem %d has a residual norm that is not finite (NaN or infinity in "
                         "f or in the iterates)", p);
            return GB_NAN;
        }
        if (fl[p]) st_out = GB_MAXSWEEPS;
    }
    return st_out;
}

extern "C" int gb_batch_solve_host(gb_batch *b, const double *h_f, double *h_psi, int *cycles, double *relres)
{
    if (!b || !h_f || !h_psi) { gb_set_error("gb_batch_solve_host: null argument"); return GB_ERR_INVALID; }
    // the staging buffer stays with the handle: an allocation of 2 x total
    // doubles per call costs as much as a third of a copy (the stream-ordered
    // pool hands the memory back at every synchronisation)
    if (!b->host_stage) {
        const cudaError_t e = cudaMalloc((void **)&b->host_stage, sizeof(double) * 2 * (size_t)b->total);
        if (e != cudaSuccess) {
            b->host_stage = nullptr;
            gb_set_error("gb_batch_solve_host: staging buffer: %s", cudaGetErrorString(e));
            return GB_ERR_ALLOC;
        }
    }
    double *d = b->host_stage;
    GB_CUDA_TRY(cudaMemcpyAsync(d, h_f, sizeof(double) * (size_t)b->total, cudaMemcpyHostToDevice, b->stream));
    int st = gb_batch_solve_device(b, d, d + b->total, cycles, relres, b->stream);
    cudaMemcpyAsync(h_psi, d + b->total, sizeof(double) * (size_t)b->total, cudaMemcpyDeviceToHost, b->stream);
    GB_CUDA_TRY(cudaStreamSynchronize(b->stream));
    return st;
}

// Pipelined host-buffer solves.  Call k's right-hand side goes up on the
// upload stream while call k-1 solves on the solve stream, and call k-1's
// solution comes down on the download stream while call k solves: the
// copies of a stream of calls hide behind the solves.
static int pipe_alloc(gb_batch *b)
{
    if (b->pipe_buf) return GB_OK;
    cudaError_t e = cudaMalloc((void **)&b->pipe_buf, sizeof(double) * 4 * (size_t)b->total);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->up, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->down, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = cudaEventCreateWithFlags(&b->ev_up[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_solved[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_down[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        gb_set_error("gb_batch_submit_host: pipeline buffers: %s", cudaGetErrorString(e));
        return GB_ERR_ALLOC;
    }
    return GB_OK;
}

// Runs the solve of the submitted call and queues its solution's download.
static int pipe_finish(gb_batch *b)
{
    b->pend = false;
    const int slot = b->pend_slot;
    double *f = b->pipe_buf + (size_t)slot * 2 * (size_t)b->total, *psi = f + b->total;
    GB_CUDA_TRY(cudaStreamWaitEvent(b->stream, b->ev_up[slot], 0));
    GB_CUDA_TRY(cudaStreamWaitEvent(b->stream, b->ev_down[slot], 0));   // the slot's previous download
    const int st = gb_batch_solve_device(b, f, psi, b->pend_cycles, b->pend_relres, b->stream);
    GB_CUDA_TRY(cudaEventRecord(b->ev_solved[slot], b->stream));
    GB_CUDA_TRY(cudaStreamWaitEvent(b->down, b->ev_solved[slot], 0));
    GB_CUDA_TRY(cudaMemcpyAsync(b->pend_psi, psi, sizeof(double) * (size_t)b->total, cudaMemcpyDeviceToHost, b->down));
    GB_CUDA_TRY(cudaEventRecord(b->ev_down[slot], b->down));
    return st;
}

extern "C" int gb_batch_submit_host(gb_batch *b, const double *h_f, double *h_psi, int *cycles, double *relres)
{
    if (!b || !h_f || !h_psi) { gb_set_error("gb_batch_submit_host: null argument"); return GB_ERR_INVALID; }
    int st = pipe_alloc(b);
    if (st != GB_OK) return st;
    const int slot = b->pipe_next;
    b->pipe_next ^= 1;
    double *f = b->pipe_buf + (size_t)slot * 2 * (size_t)b->total;
    // the slot's f was last read by a solve that has returned (solves run
    // on this thread, one call behind)
    GB_CUDA_TRY(cudaMemcpyAsync(f, h_f, sizeof(double) * (size_t)b->total, cudaMemcpyHostToDevice, b->up));
    GB_CUDA_TRY(cudaEventRecord(b->ev_up[slot], b->up));
    st = b->pend ? pipe_finish(b) : GB_OK;
    // call k-2 (this slot's last user) has its solution on the host when
    // this returns
    GB_CUDA_TRY(cudaEventSynchronize(b->ev_down[slot]));
    b->pend = true;
    b->pend_slot = slot;
    b->pend_psi = h_psi;
    b->pend_cycles = cycles;
    b->pend_relres = relres;
    return st;
}

extern "C" int gb_batch_drain(gb_batch *b)
{
    if (!b) { gb_set_error("gb_batch_drain: null handle"); return GB_ERR_INVALID; }
    const int st = b->pend ? pipe_finish(b) : GB_OK;
    if (b->down) GB_CUDA_TRY(cudaStreamSynchronize(b->down));
    if (b->up) GB_CUDA_TRY(cudaStreamSynchronize(b->up));
    return st;
}

// ---------------------------------------------------------------------------
// Self-check of the integer-pipe conversions against the hardware ones.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long cvt_mix(unsigned long long z)
{
    // splitmix64 finaliser (Steele, Lea and Flood, 2014)
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ bool cvt_same_f(float a, float b)
{
    return __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
}
__device__ __forceinline__ bool cvt_same_d(double a, double b)
{
    return __double_as_longlong(a) == __double_as_longlong(b) || (a != a && b != b);
}

// Every float bit pattern through f2d.
__global__ void k_cvt_check_f2d(unsigned long long *bad)
{
    unsigned long long cnt = 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < (1ull << 32); i += stride) {
        const float v = __uint_as_float((unsigned int)i);
        if (!cvt_same_d(f2d(v), (double)v)) ++cnt;
    }
    if (cnt) atomicAdd(bad, cnt);
}

// n seeded double bit patterns through d2f_rn: exponents drawn over the
// whole range or around the float range, fractions random or with the
// dropped bits set to a tie or one unit either side of it.
__global__ void k_cvt_check_d2f(unsigned long long n, unsigned long long seed, unsigned long long *bad)
{
    unsigned long long cnt = 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned long long h = cvt_mix(seed ^ cvt_mix(i)), h2 = cvt_mix(h);
        unsigned long long bits = h;
        const unsigned int kind = (unsigned int)(h2 & 7u);
        if (kind != 0u) {
            const unsigned long long e = (kind == 1u) ? (h2 >> 8) & 0x7ffull : 850ull + ((h2 >> 8) % 310ull);
            unsigned long long m = h & 0xFFFFFFFFFFFFFull;
            // bits dropped by the rounding: 29 in the normal range, more below
            const int sh = (e >= 897ull) ? 29 : (int)min(52ull, 926ull - e);
            const unsigned long long low = (1ull << sh) - 1ull, half = 1ull << (sh - 1);
            const unsigned int tie = (unsigned int)((h2 >> 24) & 7u);
            if (tie == 0u) m = (m & ~low) | half;
            else if (tie == 1u) m = (m & ~low) | (half - 1ull);
            else if (tie == 2u) m = (m & ~low) | (half + 1ull);
            else if (tie == 3u) m = (m & ~low) | low;
            bits = (h & 0x8000000000000000ull) | (e << 52) | m;
        }
        const double x = __longlong_as_double((long long)bits);
        if (!cvt_same_f(d2f_rn(x), __double2float_rn(x))) ++cnt;
    }
    if (cnt) atomicAdd(bad, cnt);
}

extern "C" int gb_check_conversions(long long n_random, unsigned long long seed, long long *mismatches_f2d,
                                    long long *mismatches_d2f)
{
    if (n_random < 0 || !mismatches_f2d || !mismatches_d2f) {
        gb_set_error("gb_check_conversions: invalid arguments");
        return GB_ERR_INVALID;
    }
    int dev = 0, sms = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    unsigned long long *d = nullptr;
    GB_CUDA_TRY(cudaMalloc(&d, 2 * sizeof(unsigned long long)));
    cudaError_t e = cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) {
        k_cvt_check_f2d<<<sms * 8, 256>>>(d);
        if (n_random > 0) k_cvt_check_d2f<<<sms * 8, 256>>>((unsigned long long)n_random, seed, d + 1);
        e = cudaGetLastError();
    }
    unsigned long long h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        gb_set_error("gb_check_conversions: %s", cudaGetErrorString(e));
        return GB_ERR_CUDA;
    }
    *mismatches_f2d = (long long)h[0];
    *mismatches_d2f = (long long)h[1];
    return GB_OK;
}
