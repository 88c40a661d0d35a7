// ns_diag.cu -- library diagnostics with no counterpart in the reference.
//
// ns_math_eval: the transport law's exp, log and 1/x (ns_fastmath.cuh) on
// host arrays, for testing them against the library functions.
// ns_transport_eval: mu(T), k(T) as a context's k_first evaluates them.
//
// ns_tma_wait_test: the bounded mbarrier wait of the TMA tile loads, made to
// run out (a barrier whose bytes never arrive), for testing the error path.
//
// ns_fp64_peak: the FP64 FMA throughput of a device, measured with a
// register-only DFMA loop (8 independent chains per thread, 4 blocks of 256
// threads per SM).  On GB300 the FP64 pipe, not HBM, bounds the FP64 stage
// kernels, so this is the denominator of their FP64 roofline fraction.
#include "ns_internal.cuh"
#include "ns_check.cuh"
#include "ns_tma.cuh"

namespace {

__device__ double g_peak_sink[1];

__global__ void k_dfma_loop(int iters, double a, double b)
{
    double x[8];
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = threadIdx.x * 1e-9 + q;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int q = 0; q < 8; q++) x[q] = fma(x[q], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 8; q++) s += x[q];
    if (s == 12345.678) g_peak_sink[0] = s;  // keeps the loop; never true
}

}  // namespace

extern "C" int ns_fp64_peak(int device, double *tflops)
{
    if (!tflops) return NS_ERR_PARAM;
    *tflops = 0.0;
    if (cudaSetDevice(device) != cudaSuccess) return NS_ERR_CUDA;
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return NS_ERR_CUDA;
    const int blocks = nsm * 4, threads = 256, iters = 4096;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return NS_ERR_CUDA;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return NS_ERR_CUDA;
    }
    int rc = NS_OK;
    double best = 0.0;
    k_dfma_loop<<<blocks, threads>>>(64, 0.999, 1e-3);
    for (int r = 0; r < 3 && rc == NS_OK; r++) {
        cudaEventRecord(e0, 0);
        k_dfma_loop<<<blocks, threads>>>(iters, 0.999, 1e-3);
        cudaEventRecord(e1, 0);
        if (cudaEventSynchronize(e1) != cudaSuccess) { rc = NS_ERR_CUDA; break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * blocks * threads * (double)iters * 8.0;
        const double tf = flops / (ms * 1e-3) / 1e12;
        if (tf > best) best = tf;
    }
    if (cudaGetLastError() != cudaSuccess) rc = NS_ERR_CUDA;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = best;
    return rc;
}

extern "C" int ns_math_eval(int fn, const double *x, double *y, int n, int device)
{
    if (fn < 0 || fn > 2 || n < 0 || (n > 0 && (!x || !y))) return NS_ERR_PARAM;
    if (n == 0) return NS_OK;
    if (cudaSetDevice(device) != cudaSuccess) return NS_ERR_CUDA;
    if (ns::ensure_math_tables(device) != cudaSuccess) return NS_ERR_CUDA;
    double *d = nullptr;
    if (cudaMalloc(&d, 2 * (size_t)n * sizeof(double)) != cudaSuccess) return NS_ERR_OOM;
    int rc = NS_OK;
    if (cudaMemcpy(d, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        ns::launch_math_eval(fn, d, d + n, n, 0) != cudaSuccess ||
        cudaMemcpy(y, d + n, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = NS_ERR_CUDA;
    cudaFree(d);
    return rc;
}

extern "C" int ns_transport_eval(ns_ctx *c, const double *T, double *mu, double *k, int n)
{
    if (!c || n < 0 || (n > 0 && (!T || !mu || !k))) return NS_ERR_PARAM;
    if (!c->visc) return NS_ERR_STATE;
    if (n == 0) return NS_OK;
    if (cudaSetDevice(c->dev) != cudaSuccess) return NS_ERR_CUDA;
    double *d = nullptr;
    if (cudaMalloc(&d, 3 * (size_t)n * sizeof(double)) != cudaSuccess) return NS_ERR_OOM;
    int rc = NS_OK;
    const size_t bytes = (size_t)n * sizeof(double);
    if (cudaMemcpyAsync(d, T, bytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
        ns::launch_transport_eval(c, d, d + n, d + 2 * (size_t)n, n, c->stream) != cudaSuccess ||
        cudaMemcpyAsync(mu, d + n, bytes, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaMemcpyAsync(k, d + 2 * (size_t)n, bytes, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
        rc = NS_ERR_CUDA;
    cudaFree(d);
    return rc;
}

namespace {

// One block: the barrier expects 64 bytes that no copy delivers, so every
// thread's bounded wait runs out and sets the error word.
__global__ void k_tma_wait_test(int *err, long long limit)
{
    __shared__ alignas(8) unsigned long long bar;
    if (threadIdx.x == 0) {
        ns::mbar_init(&bar, 1);
        ns::mbar_expect_tx(&bar, 64);
    }
    __syncthreads();
    ns::mbar_wait_bounded(&bar, 0, err, limit);
}

// One warp: lanes 16..31 fail an index check that guards nothing (no access
// follows it), so the checked build records it; the ordinary build has no
// check at all.
__global__ void k_check_selftest(int *err)
{
    NS_CHECK(err, ns::kChkKernels, threadIdx.x < 16);
}

}  // namespace

extern "C" int ns_checked_build(void)
{
#ifdef NS_CHECKED
    return 1;
#else
    return 0;
#endif
}

extern "C" int ns_check_selftest(int device)
{
    if (cudaSetDevice(device) != cudaSuccess) return NS_ERR_CUDA;
    int *d = nullptr;
    if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return NS_ERR_OOM;
    int h = 0;
    cudaError_t e = cudaMemset(d, 0, sizeof(int));
    if (e == cudaSuccess) {
        k_check_selftest<<<1, 32>>>(d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return NS_ERR_CUDA;
    return (h & ns::kCheckTag) ? ns::check_error(h) : NS_OK;
}

extern "C" int ns_tma_wait_test(int device, long long spin_limit)
{
    if (spin_limit < 1 || spin_limit > (1LL << 16)) return NS_ERR_PARAM;
    if (cudaSetDevice(device) != cudaSuccess) return NS_ERR_CUDA;
    int *d = nullptr;
    if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return NS_ERR_OOM;
    int h = 0;
    cudaError_t e = cudaMemset(d, 0, sizeof(int));
    if (e == cudaSuccess) {
        k_tma_wait_test<<<1, 64>>>(d, spin_limit);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return NS_ERR_CUDA;
    return h ? NS_ERR_TIMEOUT : NS_OK;
}
