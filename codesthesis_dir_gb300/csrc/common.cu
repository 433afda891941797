// Error reporting and version string of the library.
#include <stdarg.h>

#include "gbcommon.cuh"

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
