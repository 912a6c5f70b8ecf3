// bench_hooks.cu -- measurement hooks for the benchmark (include/nrltb_bench.h).
#include <cstring>
#include "nrltb.h"
#include "nrltb_bench.h"
#include "common.cuh"
#include "gemm.cuh"

using namespace nrltb;

struct nrltb_ctx;
extern "C" cudaStream_t nrltb_ctx_stream_internal(nrltb_ctx *c);

// 8 independent FMA chains per thread, long unrolled loop
template <typename T>
__global__ void k_fma_peak(T *out, int iters, T a, T b)
{
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == T(-1.2345)) out[0] = s;   // keeps the chains alive
}

extern "C" int nrltb_bench_peak(nrltb_ctx *ctx, int kind, double *tflops)
{
    if (!ctx || !tflops || (kind != 0 && kind != 1)) return NRLTB_E_ARG;
    cudaStream_t s = nrltb_ctx_stream_internal(ctx);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void *buf = nullptr;
    if (cudaMalloc(&buf, 64) != cudaSuccess) return NRLTB_E_NOMEM;
    const int threads = 512, blocks = sms * 4;
    const int iters = (kind == 0) ? 64 : 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0, s);
        if (kind == 0) k_fma_peak<double><<<blocks, threads, 0, s>>>((double *)buf, iters, 0.999999, 1e-7);
        else k_fma_peak<float><<<blocks, threads, 0, s>>>((float *)buf, iters, 0.9999f, 1e-4f);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (cudaGetLastError() != cudaSuccess) return NRLTB_E_CUDA;
    const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
    *tflops = flops / (best * 1e-3) / 1e12;
    return NRLTB_OK;
}

template <typename T>
static int time_gemm(cudaStream_t s, int n, int batch, int reps, double *ms)
{
    typedef typename cplx<T>::t C2;
    const size_t nn = (size_t)n * n * batch;
    C2 *A = nullptr, *B = nullptr, *C = nullptr;
    if (cudaMalloc(&A, sizeof(C2) * nn) != cudaSuccess) return NRLTB_E_NOMEM;
    if (cudaMalloc(&B, sizeof(C2) * nn) != cudaSuccess) { cudaFree(A); return NRLTB_E_NOMEM; }
    if (cudaMalloc(&C, sizeof(C2) * nn) != cudaSuccess) { cudaFree(A); cudaFree(B); return NRLTB_E_NOMEM; }
    cudaMemsetAsync(A, 0, sizeof(C2) * nn, s);
    cudaMemsetAsync(B, 0, sizeof(C2) * nn, s);
    const C2 one = cmk<T>(1, 0), zero = cmk<T>(0, 0);
    const long st = (long)n * n;
    zgemm<T>(s, n, n, n, batch, one, A, n, st, 0, B, n, st, 0, zero, C, n, st);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    for (int r = 0; r < reps; ++r) zgemm<T>(s, n, n, n, batch, one, A, n, st, 0, B, n, st, 0, zero, C, n, st);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(A); cudaFree(B); cudaFree(C);
    *ms = t / reps;
    return cudaGetLastError() == cudaSuccess ? NRLTB_OK : NRLTB_E_CUDA;
}

extern "C" int nrltb_bench_zgemm(nrltb_ctx *ctx, int precision, int n, int batch, int reps, double *ms_per_launch,
                                 double *flops_per_launch)
{
    if (!ctx || n < 1 || batch < 1 || reps < 1 || !ms_per_launch || !flops_per_launch) return NRLTB_E_ARG;
    cudaStream_t s = nrltb_ctx_stream_internal(ctx);
    int rc = precision == 0 ? time_gemm<double>(s, n, batch, reps, ms_per_launch)
                            : time_gemm<float>(s, n, batch, reps, ms_per_launch);
    *flops_per_launch = 8.0 * n * (double)n * n * batch;
    return rc;
}
