// Batched banded line solvers (tdma, ptdma, pdma of
// velvor2dperiodicrbconv.f:3046-3164) for many independent lines, one thread
// per line, matrices allowed to differ per line.  Each line is eliminated
// with the reference's operations in the reference's order (-fmad=false), on
// copies in a scratch buffer, so the caller's inputs survive.
#include <mutex>

#include "gbcommon.cuh"

struct LineView {
    const double *p;
    long long ls, es;
    __device__ double operator()(int line, int j) const { return p[line * ls + (long long)j * es]; }
};

__global__ void k_tdma_batch(LineView a, LineView b, LineView c, LineView r, double *y, long long ls, long long es,
                             int n, int nlines, double *scr)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nlines) return;
    double *bb = scr + (size_t)l * 2 * n, *rr = bb + n;
    for (int j = 0; j < n; ++j) { bb[j] = b(l, j); rr[j] = r(l, j); }
    for (int j = 1; j < n; ++j) {
        const double fact = a(l, j) / bb[j - 1];
        bb[j] = bb[j] - fact * c(l, j - 1);
        rr[j] = rr[j] - fact * rr[j - 1];
    }
    double yy = rr[n - 1] / bb[n - 1];
    y[l * ls + (long long)(n - 1) * es] = yy;
    for (int j = n - 2; j >= 0; --j) {
        yy = (rr[j] - c(l, j) * yy) / bb[j];
        y[l * ls + (long long)j * es] = yy;
    }
}

__global__ void k_ptdma_batch(LineView a0, LineView b0, LineView c0, LineView r0, double *y, long long ls,
                              long long es, int n, int nlines, double *scr)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nlines) return;
    double *a = scr + (size_t)l * 4 * n, *b = a + n, *c = b + n, *r = c + n;
    for (int j = 0; j < n; ++j) { a[j] = a0(l, j); b[j] = b0(l, j); c[j] = c0(l, j); r[j] = r0(l, j); }
    const int N = n - 1;
    double fact;
    for (int j = 1; j <= n - 3; ++j) {
        fact = a[j] / b[j - 1];
        b[j] = b[j] - fact * c[j - 1];
        a[j] = -fact * a[j - 1];
        r[j] = r[j] - fact * r[j - 1];
        fact = c[N] / b[j - 1];
        c[N] = -fact * c[j - 1];
        b[N] = b[N] - fact * a[j - 1];
        r[N] = r[N] - fact * r[j - 1];
    }
    fact = a[n - 2] / b[n - 3];
    b[n - 2] = b[n - 2] - fact * c[n - 3];
    c[n - 2] = c[n - 2] - fact * a[n - 3];
    r[n - 2] = r[n - 2] - fact * r[n - 3];
    fact = c[N] / b[n - 3];
    a[N] = a[N] - fact * c[n - 3];
    b[N] = b[N] - fact * a[n - 3];
    r[N] = r[N] - fact * r[n - 3];
    fact = a[N] / b[n - 2];
    b[N] = b[N] - fact * c[n - 2];
    r[N] = r[N] - fact * r[n - 2];
    const double yN = r[N] / b[N];
    double yy = (r[n - 2] - c[n - 2] * yN) / b[n - 2];
    y[l * ls + (long long)N * es] = yN;
    y[l * ls + (long long)(n - 2) * es] = yy;
    for (int j = n - 3; j >= 0; --j) {
        yy = (r[j] - c[j] * yy - a[j] * yN) / b[j];
        y[l * ls + (long long)j * es] = yy;
    }
}

__global__ void k_pdma_batch(LineView a, LineView b0, LineView c0, LineView d0, LineView e0, LineView r0, double *x,
                             long long ls, long long es, int n, int nlines, double *scr)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nlines) return;
    double *b = scr + (size_t)l * 5 * n, *c = b + n, *d = c + n, *e = d + n, *r = e + n;
    for (int j = 0; j < n; ++j) { b[j] = b0(l, j); c[j] = c0(l, j); d[j] = d0(l, j); e[j] = e0(l, j); r[j] = r0(l, j); }
    for (int k = 0; k <= n - 2; ++k) {
        d[k] = d[k] / c[k];
        e[k] = e[k] / c[k];
        r[k] = r[k] / c[k];
        c[k] = 1.0;
        c[k + 1] = c[k + 1] - b[k + 1] * d[k];
        if (k != n - 2) d[k + 1] = d[k + 1] - b[k + 1] * e[k];
        r[k + 1] = r[k + 1] - b[k + 1] * r[k];
        b[k + 1] = 0.0;
        if (k != n - 2) {
            b[k + 2] = b[k + 2] - a(l, k + 2) * d[k];
            c[k + 2] = c[k + 2] - a(l, k + 2) * e[k];
            r[k + 2] = r[k + 2] - a(l, k + 2) * r[k];
        }
    }
    double x1 = r[n - 1] / c[n - 1];
    double x0 = r[n - 2] - d[n - 2] * x1;
    x[l * ls + (long long)(n - 1) * es] = x1;
    x[l * ls + (long long)(n - 2) * es] = x0;
    for (int j = n - 3; j >= 0; --j) {
        const double xj = r[j] - d[j] * x0 - e[j] * x1;
        x[l * ls + (long long)j * es] = xj;
        x1 = x0;
        x0 = xj;
    }
}

static int check(int n, int nmin, int nlines, const char *who)
{
    if (n < nmin || nlines < 0) {
        gb_set_error("%s: need n >= %d and nlines >= 0 (got n=%d, nlines=%d)", who, nmin, n, nlines);
        return GB_ERR_INVALID;
    }
    return GB_OK;
}

extern "C" int gb_tdma_batch(const double *a, const double *b, const double *c, const double *r, double *y, int n,
                             int nlines, long long ls, long long es, void *stream)
{
    int st = check(n, 1, nlines, "gb_tdma_batch");
    if (st != GB_OK || nlines == 0) return st;
    cudaStream_t s = (cudaStream_t)stream;
    double *scr = nullptr;
    GB_CUDA_TRY(cudaMallocAsync((void **)&scr, sizeof(double) * 2 * (size_t)n * nlines, s));
    k_tdma_batch<<<gb_ceil_div(nlines, 128), 128, 0, s>>>({a, ls, es}, {b, ls, es}, {c, ls, es}, {r, ls, es}, y, ls, es,
                                                          n, nlines, scr);
    GB_CUDA_TRY(cudaFreeAsync(scr, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

extern "C" int gb_ptdma_batch(const double *a, const double *b, const double *c, const double *r, double *y, int n,
                              int nlines, long long ls, long long es, void *stream)
{
    int st = check(n, 3, nlines, "gb_ptdma_batch");
    if (st != GB_OK || nlines == 0) return st;
    cudaStream_t s = (cudaStream_t)stream;
    double *scr = nullptr;
    GB_CUDA_TRY(cudaMallocAsync((void **)&scr, sizeof(double) * 4 * (size_t)n * nlines, s));
    k_ptdma_batch<<<gb_ceil_div(nlines, 128), 128, 0, s>>>({a, ls, es}, {b, ls, es}, {c, ls, es}, {r, ls, es}, y, ls, es,
                                                           n, nlines, scr);
    GB_CUDA_TRY(cudaFreeAsync(scr, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

extern "C" int gb_pdma_batch(const double *a, const double *b, const double *c, const double *d, const double *e,
                             const double *r, double *x, int n, int nlines, long long ls, long long es, void *stream)
{
    int st = check(n, 2, nlines, "gb_pdma_batch");
    if (st != GB_OK || nlines == 0) return st;
    cudaStream_t s = (cudaStream_t)stream;
    double *scr = nullptr;
    GB_CUDA_TRY(cudaMallocAsync((void **)&scr, sizeof(double) * 5 * (size_t)n * nlines, s));
    k_pdma_batch<<<gb_ceil_div(nlines, 128), 128, 0, s>>>({a, ls, es}, {b, ls, es}, {c, ls, es}, {d, ls, es}, {e, ls, es},
                                                          {r, ls, es}, x, ls, es, n, nlines, scr);
    GB_CUDA_TRY(cudaFreeAsync(scr, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

// ---------------------------------------------------------------------------
// gb_pdma_batch_noalloc: the pentadiagonal batch without any allocation.
//
// The per-line work copies live in one file-scope device array of
// GB_PDMA_NOALLOC_MAX_DOUBLES doubles (4 MiB) that every GPU which loads the
// library holds until the process exits.  Host code may not pass the
// array's name to a kernel (on the host it is only a stand-in for the
// device symbol), so its device address is looked up once per device, with
// that device current, and cached for the life of the process (a
// cudaDeviceReset after the first call would leave a stale address: not
// supported).  The kernel writes every scratch element it reads, so nothing
// needs clearing between calls.  Each call waits for its stream before it
// returns, so one host thread's calls never overlap; calls from different
// host threads that overlap on the GPU share the array and race.
// ---------------------------------------------------------------------------
static __device__ __align__(256) double g_pdma_noalloc_scratch[GB_PDMA_NOALLOC_MAX_DOUBLES];

static std::mutex g_noalloc_mu;
static double *g_noalloc_addr[128];
static bool g_noalloc_ready[128];

static int noalloc_scratch(double **out)
{
    int dev = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) {
        gb_set_error("gb_pdma_batch_noalloc: device ordinal %d out of range", dev);
        return GB_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ready[dev]) {
        void *addr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&addr, g_pdma_noalloc_scratch);
        if (e != cudaSuccess) {
            gb_set_error("gb_pdma_batch_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return GB_ERR_CUDA;
        }
        g_noalloc_addr[dev] = (double *)addr;
        g_noalloc_ready[dev] = true;
    }
    *out = g_noalloc_addr[dev];
    return GB_OK;
}

extern "C" int gb_pdma_batch_noalloc(const double *a, const double *b, const double *c, const double *d,
                                     const double *e, const double *r, double *x, int n, int nlines,
                                     long long ls, long long es, void *stream)
{
    int st = check(n, 2, nlines, "gb_pdma_batch_noalloc");
    if (st != GB_OK || nlines == 0) return st;
    const unsigned long long need = 5ull * (unsigned long long)n * (unsigned long long)nlines;
    if (need > (unsigned long long)GB_PDMA_NOALLOC_MAX_DOUBLES) {
        gb_set_error("gb_pdma_batch_noalloc: 5*n*nlines = %llu doubles exceeds the fixed scratch of %u doubles "
                     "(n=%d, nlines=%d); use gb_pdma_batch or split the lines",
                     need, (unsigned)GB_PDMA_NOALLOC_MAX_DOUBLES, n, nlines);
        return GB_ERR_INVALID;
    }
    double *scr = nullptr;
    st = noalloc_scratch(&scr);
    if (st != GB_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    k_pdma_batch<<<gb_ceil_div(nlines, 128), 128, 0, s>>>({a, ls, es}, {b, ls, es}, {c, ls, es}, {d, ls, es}, {e, ls, es},
                                                          {r, ls, es}, x, ls, es, n, nlines, scr);
    GB_CUDA_TRY(cudaGetLastError());
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return GB_OK;
}
