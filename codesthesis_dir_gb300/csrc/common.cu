// Error reporting and version string of the library.
#include <stdarg.h>

#include "gbcommon.cuh"
#include "gridsync.cuh"
#include "divrn.cuh"

static thread_local char g_err[512] = "";

void gb_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

extern "C" const char *gb_last_error(void) { return g_err; }

extern "C" const char *gb_version(void)
{
    return "gb300conv 0.1 sm_103a (fp64 paths built with -fmad=false; explicit fma only)";
}

// ---------------------------------------------------------------------------
// Issue-rate probe: independent chains of FP64 and FP32 fused multiply-adds
// on every SM, timed with CUDA events.  Gives the FP64 and FP32 pipe peaks
// that the FP64-bound kernels are reported against.
// ---------------------------------------------------------------------------
template <class T> __device__ __forceinline__ T probe_fma(T a, T b, T c);
template <> __device__ __forceinline__ double probe_fma<double>(double a, double b, double c) { return __fma_rn(a, b, c); }
template <> __device__ __forceinline__ float probe_fma<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }

template <class T>
__global__ void k_probe_fma(T *out, int iters, T b, T c)
{
    T a0 = (T)threadIdx.x * (T)1e-3, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
    T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
    for (int i = 0; i < iters; ++i) {
        a0 = probe_fma(a0, b, c); a1 = probe_fma(a1, b, c); a2 = probe_fma(a2, b, c); a3 = probe_fma(a3, b, c);
        a4 = probe_fma(a4, b, c); a5 = probe_fma(a5, b, c); a6 = probe_fma(a6, b, c); a7 = probe_fma(a7, b, c);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

template <class T>
static int probe_rate(int blocks, int threads, int iters, double *rate)
{
    T *d = nullptr;
    GB_CUDA_TRY(cudaMalloc(&d, sizeof(T) * (size_t)blocks * threads));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_probe_fma<T><<<blocks, threads>>>(d, iters / 8, (T)0.999999, (T)1e-7);  // warm-up
    cudaEventRecord(e0);
    k_probe_fma<T><<<blocks, threads>>>(d, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    GB_CUDA_TRY(cudaGetLastError());
    *rate = 8.0 * iters * (double)blocks * threads / (ms * 1e-3);
    return GB_OK;
}

extern "C" int gb_measure_issue_rates(double *fp64_fma_per_s, double *fp32_fma_per_s)
{
    int dev = 0, nsm = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    double r64 = 0.0, r32 = 0.0;
    int st = probe_rate<double>(nsm * 8, 256, 2048, &r64);
    if (st != GB_OK) return st;
    st = probe_rate<float>(nsm * 8, 256, 65536, &r32);
    if (st != GB_OK) return st;
    if (fp64_fma_per_s) *fp64_fma_per_s = r64;
    if (fp32_fma_per_s) *fp32_fma_per_s = r32;
    return GB_OK;
}

// ---------------------------------------------------------------------------
// Grid-barrier probe: one cooperative launch of `blocks` x `threads` that
// does nothing but pass `nbarriers` bounded grid barriers.  The time per
// barrier is what a persistent solve launched with that shape pays for each
// of its phases on top of the phase's own work.
// ---------------------------------------------------------------------------
__global__ void k_barrier_probe(GridSync gs, int nbarriers)
{
    for (int i = 0; i < nbarriers; ++i)
        if (!grid_sync(gs)) return;
}

extern "C" int gb_measure_grid_barrier(int blocks, int threads, int nbarriers, double *us_per_barrier)
{
    if (blocks < 1 || threads < 32 || threads > 1024 || (threads & 31) || nbarriers < 1 || !us_per_barrier) {
        gb_set_error("gb_measure_grid_barrier: invalid argument");
        return GB_ERR_INVALID;
    }
    int dev = 0, coop = 0, per = 0, sms = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_barrier_probe, threads, 0));
    if (!coop || blocks > per * sms) {
        gb_set_error("gb_measure_grid_barrier: %d blocks of %d threads cannot all be resident (%d per SM x %d SMs)",
                     blocks, threads, per, sms);
        return GB_ERR_INVALID;
    }
    unsigned *sync = nullptr;
    GB_CUDA_TRY(cudaMalloc(&sync, 4 * sizeof(unsigned)));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0.f;
    unsigned hs[4] = {0, 0, 0, 0};
    for (int rep = 0; rep < 2 && e == cudaSuccess && hs[2] == 0; ++rep) {   // the first launch warms up
        e = cudaMemset(sync, 0, 4 * sizeof(unsigned));
        GridSync gs;
        gs.count = sync;
        gs.gen = sync + 1;
        gs.err = (int *)(sync + 2);
        gs.limit = GB_GRID_WAIT_LIMIT_DEFAULT;
        gs.tally = nullptr;
        int nb = nbarriers;
        void *args[] = {&gs, &nb};
        if (e == cudaSuccess) e = cudaEventRecord(e0);
        if (e == cudaSuccess) e = cudaLaunchCooperativeKernel((void *)k_barrier_probe, blocks, threads, args, 0, 0);
        if (e == cudaSuccess) e = cudaEventRecord(e1);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess) e = cudaMemcpy(hs, sync, sizeof(hs), cudaMemcpyDeviceToHost);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(sync);
    if (e != cudaSuccess) {
        gb_set_error("gb_measure_grid_barrier: %s", cudaGetErrorString(e));
        return GB_ERR_CUDA;
    }
    if (hs[2]) {
        gb_set_error("gb_measure_grid_barrier: a barrier wait reached its limit");
        return GB_TIMEOUT;
    }
    *us_per_barrier = 1e3 * (double)ms / (double)nbarriers;
    return GB_OK;
}

// ---------------------------------------------------------------------------
// Division check: the correctly rounded quotient from a stored reciprocal
// (divrn.cuh) against the hardware division, on seeded operands: random
// significands and signs with exponents in [-300, 300] (quotients well inside
// the normal range), products b q rounded (quotients at or next to a
// representable value), small integers, and zero dividends of either sign.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long mix64(unsigned long long x)
{
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ double make_double(unsigned long long h, int e)
{
    const unsigned long long bits = (h & 0x800fffffffffffffull) | ((unsigned long long)(e + 1023) << 52);
    return __longlong_as_double((long long)bits);
}

__global__ void k_check_division(unsigned long long n, unsigned long long seed, unsigned long long *bad)
{
    unsigned long long cnt = 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned long long h1 = mix64(seed ^ (2 * i)), h2 = mix64(seed ^ (2 * i + 1)), h3 = mix64(h1 ^ h2);
        const int ea = (int)((h1 >> 52) % 601) - 300, eb = (int)((h2 >> 52) % 601) - 300;
        double a, b;
        switch ((int)(h3 & 3)) {
        case 0:
            a = make_double(h1, ea);
            b = make_double(h2, eb);
            break;
        case 1:
            b = make_double(h2, eb / 2);
            a = __dmul_rn(b, make_double(h1, ea / 2));
            break;
        case 2:
            a = (double)((long long)(h1 % 2000001ull) - 1000000);
            b = (double)((long long)(h2 % 1999ull) - 999);
            if (b == 0.0) b = 7.0;
            break;
        default:
            a = (h1 & 1) ? -0.0 : 0.0;
            b = make_double(h2, eb);
            break;
        }
        const double y = 1.0 / b;
        const double q = div_by_rcp(a, b, y);
        const double ref = a / b;
        if (__double_as_longlong(q) != __double_as_longlong(ref)) ++cnt;
    }
    if (cnt) atomicAdd(bad, cnt);
}

extern "C" int gb_check_division(long long n_random, unsigned long long seed, long long *mismatches)
{
    if (n_random < 1 || !mismatches) {
        gb_set_error("gb_check_division: invalid argument");
        return GB_ERR_INVALID;
    }
    int dev = 0, sms = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    unsigned long long *d = nullptr;
    GB_CUDA_TRY(cudaMalloc(&d, sizeof(unsigned long long)));
    cudaError_t e = cudaMemset(d, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) {
        k_check_division<<<sms * 8, 256>>>((unsigned long long)n_random, seed, d);
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        gb_set_error("gb_check_division: %s", cudaGetErrorString(e));
        return GB_ERR_CUDA;
    }
    *mismatches = (long long)h;
    return GB_OK;
}
