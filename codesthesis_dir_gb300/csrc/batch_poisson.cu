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
#define PTS_PER_BLOCK 1024   // interior points per block of the level tables
#define BP_THREADS 256

template <class T> __device__ __forceinline__ T fmaT(T a, T b, T c);
template <> __device__ __forceinline__ double fmaT<double>(double a, double b, double c) { return __fma_rn(a, b, c); }
template <> __device__ __forceinline__ float fmaT<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }

struct BlkEntry {
    int p;       // problem
    int start;   // first interior point (row-major over the (n-2)^2 interior)
};

struct BatchDev {
    int nprob;
    const int *n_of;          // [p*BP_MAXL + l] level sizes (0 past the last level)
    const int *nlev;          // [p]
    const int *dloc;          // [p] first level solved locally
    void *const *x;           // [p*BP_MAXL + l] solution / correction of level l (T*)
    void *const *f;           // right-hand side of level l (T*)
    void *const *r;           // residual scratch of level l (T*)
    int *active;              // [p]
    int *cycles;              // [p]
    int *failed;              // [p]
    double *fnorm, *relres;   // [p]
    double *partial;          // per level-0 block
    const int *p_blk0, *p_nblk0;  // level-0 table range of each problem
    int *num_active;
    int max_cycles;
    double rtol;
};

template <class T> __device__ __forceinline__ T *XP(const BatchDev &B, int p, int l) { return (T *)B.x[p * BP_MAXL + l]; }
template <class T> __device__ __forceinline__ T *FP(const BatchDev &B, int p, int l) { return (T *)B.f[p * BP_MAXL + l]; }
template <class T> __device__ __forceinline__ T *RP(const BatchDev &B, int p, int l) { return (T *)B.r[p * BP_MAXL + l]; }

// ---------------------------------------------------------------------------
// Level-synchronous kernels (one table entry per block)
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(BP_THREADS) k_rb_half(BatchDev B, const BlkEntry *tbl, int l, int color)
{
    const BlkEntry e = tbl[blockIdx.x];
    if (!B.active[e.p]) return;
    const int n = B.n_of[e.p * BP_MAXL + l], m = n - 2;
    T *x = XP<T>(B, e.p, l);
    const T *f = FP<T>(B, e.p, l);
    const T h = (T)1 / (T)(n - 1), h2 = h * h;
    const int end = min(e.start + PTS_PER_BLOCK, m * m);
    for (int q = e.start + threadIdx.x; q < end; q += blockDim.x) {
        const int j = q / m + 1, i = q - (j - 1) * m + 1;
        if (((i + j) & 1) != color) continue;
        const size_t c = (size_t)j * n + i;
        const T s = (x[c - 1] + x[c + 1]) + (x[c - n] + x[c + n]);
        x[c] = fmaT<T>(-h2, f[c], s) * (T)0.25;
    }
}

template <class T>
__global__ void __launch_bounds__(BP_THREADS) k_residual(BatchDev B, const BlkEntry *tbl, int l)
{
    const BlkEntry e = tbl[blockIdx.x];
    if (!B.active[e.p]) return;
    const int n = B.n_of[e.p * BP_MAXL + l], m = n - 2;
    const T *x = XP<T>(B, e.p, l);
    const T *f = FP<T>(B, e.p, l);
    T *r = RP<T>(B, e.p, l);
    const T h = (T)1 / (T)(n - 1), ih2 = (T)1 / (h * h);
    const int end = min(e.start + PTS_PER_BLOCK, m * m);
    for (int q = e.start + threadIdx.x; q < end; q += blockDim.x) {
        const int j = q / m + 1, i = q - (j - 1) * m + 1;
        const size_t c = (size_t)j * n + i;
        const T s = (x[c - 1] + x[c + 1]) + (x[c - n] + x[c + n]);
        const T lap = fmaT<T>((T)-4, x[c], s);
        r[c] = fmaT<T>(-ih2, lap, f[c]);
    }
}

// Full weighting onto the coarse interior (rotann2.f:773-785 summation
// order); the coarse solution is zeroed.  tbl is the table of level l+1.
template <class T>
__global__ void __launch_bounds__(BP_THREADS) k_restrict(BatchDev B, const BlkEntry *tbl, int l)
{
    const BlkEntry e = tbl[blockIdx.x];
    if (!B.active[e.p]) return;
    const int n = B.n_of[e.p * BP_MAXL + l], nc = B.n_of[e.p * BP_MAXL + l + 1], mc = nc - 2;
    const T *r = RP<T>(B, e.p, l);
    T *fc = FP<T>(B, e.p, l + 1);
    T *xc = XP<T>(B, e.p, l + 1);
    const int end = min(e.start + PTS_PER_BLOCK, mc * mc);
    for (int q = e.start + threadIdx.x; q < end; q += blockDim.x) {
        const int j = q / mc + 1, i = q - (j - 1) * mc + 1;
        const size_t c = (size_t)(2 * j) * n + (size_t)(2 * i);
        T t = r[c];
        t = t * (T)2 + r[c + 1] + r[c - 1];
        t = t + r[c + n] + r[c - n];
        t = t * (T)2 + r[c + 1 + n] + r[c - 1 - n];
        t = t + r[c + 1 - n] + r[c - 1 + n];
        fc[(size_t)j * nc + i] = t * (T)0.0625;
        xc[(size_t)j * nc + i] = (T)0;
    }
}

// Bilinear prolongation of level l+1 added into level l (rotann2.f:821-858).
template <class T>
__global__ void __launch_bounds__(BP_THREADS) k_prolong_add(BatchDev B, const BlkEntry *tbl, int l)
{
    const BlkEntry e = tbl[blockIdx.x];
    if (!B.active[e.p]) return;
    const int n = B.n_of[e.p * BP_MAXL + l], nc = B.n_of[e.p * BP_MAXL + l + 1], m = n - 2;
    T *x = XP<T>(B, e.p, l);
    const T *ec = XP<T>(B, e.p, l + 1);
    const int end = min(e.start + PTS_PER_BLOCK, m * m);
    for (int q = e.start + threadIdx.x; q < end; q += blockDim.x) {
        const int j = q / m + 1, i = q - (j - 1) * m + 1;
        const T *ep = ec + (size_t)(j / 2) * nc + (i / 2);
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
        const size_t c = (size_t)j * n + i;
        x[c] = x[c] + v;
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
__global__ void __launch_bounds__(BP_THREADS) k_local_vcycle(BatchDev B, int nu1, int nu2)
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
        const int n = B.n_of[p * BP_MAXL + d0];
        const T *gx = XP<T>(B, p, d0), *gf = FP<T>(B, p, d0);
        for (int q = threadIdx.x; q < n * n; q += blockDim.x) { X[q] = gx[q]; F[q] = gf[q]; }
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
        const int n = B.n_of[p * BP_MAXL + d0];
        T *gx = XP<T>(B, p, d0);
        for (int q = threadIdx.x; q < n * n; q += blockDim.x) gx[q] = X[q];
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

// FP64 residual of level 0 (psi, f user arrays); mode 0: norm only (plain),
// mode 1: also store the residual as the FP32 right-hand side of the inner
// cycle and zero the FP32 correction (mixed).
__global__ void __launch_bounds__(BP_THREADS) k_outer_residual(BatchDev B, const BlkEntry *tbl, const double *const *psi_p,
                                                               const double *const *f_p, int mode)
{
    __shared__ double s_red[32];
    const BlkEntry e = tbl[blockIdx.x];
    if (!B.active[e.p]) return;
    const int n = B.n_of[e.p * BP_MAXL], m = n - 2;
    const double *x = psi_p[e.p], *f = f_p[e.p];
    const double h = 1.0 / (double)(n - 1), ih2 = 1.0 / (h * h);
    float *f32 = mode ? FP<float>(B, e.p, 0) : nullptr;
    float *x32 = mode ? XP<float>(B, e.p, 0) : nullptr;
    double acc = 0.0;
    const int end = min(e.start + PTS_PER_BLOCK, m * m);
    for (int q = e.start + threadIdx.x; q < end; q += blockDim.x) {
        const int j = q / m + 1, i = q - (j - 1) * m + 1;
        const size_t c = (size_t)j * n + i;
        const double s = (x[c - 1] + x[c + 1]) + (x[c - n] + x[c + n]);
        const double lap = __fma_rn(-4.0, x[c], s);
        const double r = __fma_rn(-ih2, lap, f[c]);
        acc = __fma_rn(r, r, acc);
        if (mode) {
            f32[c] = (float)r;
            x32[c] = 0.0f;
        }
    }
    const double tot = blk_sum(acc, s_red);
    if (threadIdx.x == 0) B.partial[blockIdx.x] = tot;
}

// psi += (double) e over the interior (mixed mode).
__global__ void __launch_bounds__(BP_THREADS) k_correct(BatchDev B, const BlkEntry *tbl, double *const *psi_p)
{
    const BlkEntry e = tbl[blockIdx.x];
    if (!B.active[e.p]) return;
    const int n = B.n_of[e.p * BP_MAXL], m = n - 2;
    double *x = psi_p[e.p];
    const float *ev = XP<float>(B, e.p, 0);
    const int end = min(e.start + PTS_PER_BLOCK, m * m);
    for (int q = e.start + threadIdx.x; q < end; q += blockDim.x) {
        const int j = q / m + 1, i = q - (j - 1) * m + 1;
        const size_t c = (size_t)j * n + i;
        x[c] = x[c] + (double)ev[c];
    }
}

// One thread per problem: sums the block partials in order, decides whether
// the problem keeps cycling.  first != 0 records ||f|| (psi = 0).
__global__ void k_finalize(BatchDev B, int first)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= B.nprob) return;
    if (!B.active[p]) return;
    double s = 0.0;
    const int b0 = B.p_blk0[p], nb = B.p_nblk0[p];
    for (int b = 0; b < nb; ++b) s += B.partial[b0 + b];
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
        B.cycles[p] += 1;
        atomicAdd(B.num_active, 1);
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct gb_batch {
    int nprob = 0, precision = 0, nu1 = 2, nu2 = 2, max_cycles = 100;
    double rtol = 1e-10;
    std::vector<int> n, L, dloc;
    long long total = 0;
    std::vector<long long> off0;      // level-0 offsets in the packed user arrays
    int maxdepth_global = 0;          // levels 0..maxdepth_global-1 have global work
    // device
    void *pool = nullptr;             // T levels (T = double or float)
    size_t pool_bytes = 0;
    int *d_int = nullptr;             // n_of, nlev, dloc, active, cycles, failed, p_blk0, p_nblk0, num_active
    double *d_dbl = nullptr;          // fnorm, relres, partial
    void **d_ptrs = nullptr;          // x, f, r tables + psi/f level-0 pointer tables
    BlkEntry *d_tbl = nullptr;
    std::vector<int> tbl_off, tbl_cnt;    // per level: smoothing table segment
    std::vector<int> rtbl_off, rtbl_cnt;  // per level: restriction-target table segment
    int tbl0_off = 0, tbl0_cnt = 0;     // level-0 table over all problems (norms)
    BatchDev dev;
    double **d_psi_tab = nullptr, **d_f_tab = nullptr;
    std::vector<void *> hx, hf, hr;     // host copies of the pointer tables
    size_t local_smem = 0;
    int *h_pinned = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t cycle_graph = nullptr;
    const double *graph_f = nullptr;
    double *graph_psi = nullptr;
    long long launches = 0, launches_per_cycle = 0;
    // optional per-launch timing of the finest-level smoothing kernel
    int profile = 0, graph_profile = -1, graph_ev = 0;
    std::vector<cudaEvent_t> ev;
    int ev_used = 0;
    double prof_ms = 0.0, prof_bytes = 0.0;
    long long prof_launches = 0;
    std::vector<int> h_active;
    double level0_points_all = 0.0;
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

extern "C" int gb_batch_create(int nprob, const int *n, int precision, int nu1, int nu2, double rtol,
                               int max_cycles, gb_batch **out)
{
    if (!out || !n || nprob <= 0 || (precision != GB_BATCH_FP64 && precision != GB_BATCH_MIXED) || nu1 < 0 ||
        nu2 < 0 || max_cycles < 0) {
        gb_set_error("gb_batch_create: invalid argument");
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
            const size_t sz = (size_t)nl[l] * nl[l];
            // plain: levels >= 1 need x, f; all levels need r.  mixed: every level x, f, r.
            pool_elems += (precision == GB_BATCH_FP64 && l == 0) ? sz : 3 * sz;
        }
        b->off0[p] = tot;
        tot += (long long)np_ * np_;
    }
    b->total = tot;
    b->maxdepth_global = maxd;
    // local-solve shared memory: x, f, r of levels dloc..L-1
    size_t smax = 0;
    for (int p = 0; p < nprob; ++p) {
        size_t s = 0;
        for (int l = b->dloc[p]; l < b->L[p]; ++l) s += (size_t)nof[(size_t)p * BP_MAXL + l] * nof[(size_t)p * BP_MAXL + l];
        smax = std::max(smax, 3 * s * esz);
    }
    b->local_smem = smax;
    // block tables: smoothing tables per level l (problems with l < dloc),
    // restriction-target tables per level l >= 1 (problems with l <= dloc),
    // and the level-0 table over all problems (norms, defect correction)
    std::vector<BlkEntry> tbl;
    b->tbl_off.assign(BP_MAXL, 0);
    b->tbl_cnt.assign(BP_MAXL, 0);
    b->rtbl_off.assign(BP_MAXL, 0);
    b->rtbl_cnt.assign(BP_MAXL, 0);
    std::vector<int> pb0(nprob), pnb0(nprob);
    for (int l = 0; l < BP_MAXL; ++l) {
        b->tbl_off[l] = (int)tbl.size();
        for (int p = 0; p < nprob; ++p) {
            if (l >= b->dloc[p]) continue;
            const int m = nof[(size_t)p * BP_MAXL + l] - 2;
            for (int s0 = 0; s0 < m * m; s0 += PTS_PER_BLOCK) tbl.push_back({p, s0});
        }
        b->tbl_cnt[l] = (int)tbl.size() - b->tbl_off[l];
        b->rtbl_off[l] = (int)tbl.size();
        for (int p = 0; p < nprob; ++p) {
            if (l < 1 || l > b->dloc[p]) continue;
            const int m = nof[(size_t)p * BP_MAXL + l] - 2;
            for (int s0 = 0; s0 < m * m; s0 += PTS_PER_BLOCK) tbl.push_back({p, s0});
        }
        b->rtbl_cnt[l] = (int)tbl.size() - b->rtbl_off[l];
    }
    b->tbl0_off = (int)tbl.size();
    for (int p = 0; p < nprob; ++p) {
        const int m = n[p] - 2;
        pb0[p] = (int)tbl.size() - b->tbl0_off;
        for (int s = 0; s < m * m; s += PTS_PER_BLOCK) tbl.push_back({p, s});
        pnb0[p] = (int)tbl.size() - b->tbl0_off - pb0[p];
    }
    b->tbl0_cnt = (int)tbl.size() - b->tbl0_off;

#define BTRY(x)                                                                 \
    do {                                                                        \
        cudaError_t _e = (x);                                                   \
        if (_e != cudaSuccess) {                                                \
            gb_set_error("gb_batch_create: %s: %s", #x, cudaGetErrorString(_e)); \
            gb_batch_destroy(b);                                                \
            return GB_ERR_ALLOC;                                                \
        }                                                                       \
    } while (0)
    b->pool_bytes = pool_elems * esz;
    BTRY(cudaMalloc(&b->pool, b->pool_bytes));
    BTRY(cudaMemset(b->pool, 0, b->pool_bytes));
    const size_t nint = (size_t)nprob * BP_MAXL + 2 * (size_t)nprob + 3 * (size_t)nprob + 2 * (size_t)nprob + 1;
    BTRY(cudaMalloc(&b->d_int, sizeof(int) * nint));
    const size_t ndbl = 2 * (size_t)nprob + (size_t)b->tbl0_cnt;
    BTRY(cudaMalloc(&b->d_dbl, sizeof(double) * ndbl));
    BTRY(cudaMalloc(&b->d_ptrs, sizeof(void *) * (3 * (size_t)nprob * BP_MAXL + 2 * (size_t)nprob)));
    BTRY(cudaMalloc(&b->d_tbl, sizeof(BlkEntry) * std::max<size_t>(1, tbl.size())));
    BTRY(cudaMallocHost(&b->h_pinned, sizeof(int) * 16));
    BTRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    // pointer tables
    b->hx.assign((size_t)nprob * BP_MAXL, nullptr);
    b->hf.assign((size_t)nprob * BP_MAXL, nullptr);
    b->hr.assign((size_t)nprob * BP_MAXL, nullptr);
    char *base = (char *)b->pool;
    for (int p = 0; p < nprob; ++p) {
        for (int l = 0; l < b->L[p]; ++l) {
            const size_t sz = (size_t)nof[(size_t)p * BP_MAXL + l] * nof[(size_t)p * BP_MAXL + l] * esz;
            const size_t k = (size_t)p * BP_MAXL + l;
            if (!(precision == GB_BATCH_FP64 && l == 0)) {
                b->hx[k] = base; base += sz;
                b->hf[k] = base; base += sz;
            }
            b->hr[k] = base; base += sz;
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
    if (!tbl.empty()) BTRY(cudaMemcpy(b->d_tbl, tbl.data(), sizeof(BlkEntry) * tbl.size(), cudaMemcpyHostToDevice));
    void **dp = b->d_ptrs;
    BTRY(cudaMemcpy(dp, b->hx.data(), sizeof(void *) * b->hx.size(), cudaMemcpyHostToDevice));
    BTRY(cudaMemcpy(dp + b->hx.size(), b->hf.data(), sizeof(void *) * b->hf.size(), cudaMemcpyHostToDevice));
    BTRY(cudaMemcpy(dp + 2 * b->hx.size(), b->hr.data(), sizeof(void *) * b->hr.size(), cudaMemcpyHostToDevice));
    b->d_psi_tab = (double **)(dp + 3 * b->hx.size());
    b->d_f_tab = (double **)(dp + 3 * b->hx.size() + nprob);
    BatchDev &D = b->dev;
    D.nprob = nprob;
    D.n_of = d_nof;
    D.nlev = d_nlev;
    D.dloc = d_dloc;
    D.x = dp;
    D.f = dp + b->hx.size();
    D.r = dp + 2 * b->hx.size();
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
    D.rtol = rtol;
    if (b->local_smem > 48 * 1024) {
        if (precision == GB_BATCH_FP64)
            BTRY(cudaFuncSetAttribute(k_local_vcycle<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->local_smem));
        else
            BTRY(cudaFuncSetAttribute(k_local_vcycle<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->local_smem));
    }
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
    cudaFree(b->d_tbl);
    if (b->h_pinned) cudaFreeHost(b->h_pinned);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return GB_OK;
}

extern "C" long long gb_batch_total_points(const gb_batch *b) { return b ? b->total : 0; }
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

// The kernels of one V-cycle (descent over the global levels, the local
// coarse solves, ascent), for element type T.
template <class T>
static void enqueue_vcycle(gb_batch *b, cudaStream_t s)
{
    BatchDev &D = b->dev;
    const BlkEntry *tb = b->d_tbl;
    long long &nl = b->launches;
    // descent: level l is global for problems with dloc > l
    for (int l = 0; l < b->maxdepth_global; ++l) {
        const int cnt = b->tbl_cnt[l];
        if (cnt == 0) continue;
        const BlkEntry *t = tb + b->tbl_off[l];
        for (int it = 0; it < b->nu1; ++it) {
            for (int color = 0; color < 2; ++color) {
                const bool ev = b->profile && l == 0 && b->ev_used + 2 <= (int)b->ev.size();
                if (ev) prof_record(b->ev[b->ev_used], s);
                k_rb_half<T><<<cnt, BP_THREADS, 0, s>>>(D, t, l, color);
                if (ev) { prof_record(b->ev[b->ev_used + 1], s); b->ev_used += 2; }
            }
            nl += 2;
        }
        k_residual<T><<<cnt, BP_THREADS, 0, s>>>(D, t, l);
        const int cntc = b->rtbl_cnt[l + 1];
        k_restrict<T><<<cntc, BP_THREADS, 0, s>>>(D, tb + b->rtbl_off[l + 1], l);
        nl += 2;
    }
    k_local_vcycle<T><<<b->nprob, BP_THREADS, b->local_smem, s>>>(D, b->nu1, b->nu2);
    nl += 1;
    for (int l = b->maxdepth_global - 1; l >= 0; --l) {
        const int cnt = b->tbl_cnt[l];
        if (cnt == 0) continue;
        const BlkEntry *t = tb + b->tbl_off[l];
        k_prolong_add<T><<<cnt, BP_THREADS, 0, s>>>(D, t, l);
        nl += 1;
        for (int it = 0; it < b->nu2; ++it) {
            for (int color = 0; color < 2; ++color) {
                const bool ev = b->profile && l == 0 && b->ev_used + 2 <= (int)b->ev.size();
                if (ev) prof_record(b->ev[b->ev_used], s);
                k_rb_half<T><<<cnt, BP_THREADS, 0, s>>>(D, t, l, color);
                if (ev) { prof_record(b->ev[b->ev_used + 1], s); b->ev_used += 2; }
            }
            nl += 2;
        }
    }
}

// One outer iteration: residual norm (and, mixed, the FP32 right-hand side),
// convergence bookkeeping, one V-cycle, and (mixed) the FP64 correction.
static void enqueue_iteration(gb_batch *b, int first, cudaStream_t s)
{
    BatchDev &D = b->dev;
    const BlkEntry *t0 = b->d_tbl + b->tbl0_off;
    cudaMemsetAsync(D.num_active, 0, sizeof(int), s);
    const int mode = b->precision == GB_BATCH_MIXED ? 1 : 0;
    k_outer_residual<<<b->tbl0_cnt, BP_THREADS, 0, s>>>(D, t0, (const double *const *)b->d_psi_tab,
                                                         (const double *const *)b->d_f_tab, mode);
    k_finalize<<<gb_ceil_div(b->nprob, 128), 128, 0, s>>>(D, first);
    b->launches += 2;
    if (b->precision == GB_BATCH_FP64) {
        enqueue_vcycle<double>(b, s);
    } else {
        enqueue_vcycle<float>(b, s);
        k_correct<<<b->tbl0_cnt, BP_THREADS, 0, s>>>(D, t0, b->d_psi_tab);
        b->launches += 1;
    }
    cudaMemcpyAsync(b->h_pinned, D.num_active, sizeof(int), cudaMemcpyDeviceToHost, s);
}

// After an iteration has completed: adds the recorded smoothing-launch times
// and the algorithmic bytes of the problems that took part (1.5 words per
// interior point per half-sweep: psi read, f read, psi written, each for
// half of the points plus the neighbours' half).
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
    for (int i = 0; i + 1 < b->ev_used; i += 2) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, b->ev[i], b->ev[i + 1]) == cudaSuccess) {
            b->prof_ms += ms;
            b->prof_launches += 1;
            b->prof_bytes += 1.5 * esz * pts;
        } else {
            cudaGetLastError();  // timing is advisory: never let it fail a solve
        }
    }
}

extern "C" int gb_batch_profile(gb_batch *b, int enable)
{
    if (!b) return GB_ERR_INVALID;
    if (enable && b->ev.empty()) {
        const int need = 2 * 2 * (b->nu1 + b->nu2) + 4;
        b->ev.resize(need);
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
            b->hx[(size_t)p * BP_MAXL] = d_psi + b->off0[p];
            b->hf[(size_t)p * BP_MAXL] = (void *)(d_f + b->off0[p]);
        }
        GB_CUDA_TRY(cudaMemcpyAsync(b->d_ptrs, b->hx.data(), sizeof(void *) * b->hx.size(), cudaMemcpyHostToDevice, s));
        GB_CUDA_TRY(cudaMemcpyAsync(b->d_ptrs + b->hx.size(), b->hf.data(), sizeof(void *) * b->hf.size(),
                                    cudaMemcpyHostToDevice, s));
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
    if (!b->cycle_graph || b->graph_f != d_f || b->graph_psi != d_psi || b->graph_profile != b->profile) {
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
        b->graph_f = d_f;
        b->graph_psi = d_psi;
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
