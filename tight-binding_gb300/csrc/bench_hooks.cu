// bench_hooks.cu -- measurement hooks for the benchmark (include/nrltb_bench.h).
#include <cstring>
#include "nrltb.h"
#include "nrltb_bench.h"
#include "common.cuh"
#include "gemm.cuh"
#include "dfgemm.cuh"
#include "ozaki.cuh"

using namespace nrltb;
void nrltb_internal_set_error(const char *msg);

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

// 8 independent accumulators per warp, back-to-back mma.sync (kind 2: bf16
// m16n8k16, kind 3: tf32 m16n8k8; FP32 accumulate)
template <int KIND>
__global__ void k_mma_peak(float *out, int iters)
{
    float c[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i) c[i][0] = c[i][1] = c[i][2] = c[i][3] = 0.f;
    const unsigned a0 = 0x3f803f80u ^ threadIdx.x, b0 = 0x3f803f80u ^ (threadIdx.x << 1);
    const unsigned a[4] = {a0, a0 ^ 1u, a0 ^ 2u, a0 ^ 3u}, b[2] = {b0, b0 ^ 1u};
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            if (KIND == 2)
                asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                             "{%8,%9}, {%0,%1,%2,%3};"
                             : "+f"(c[i][0]), "+f"(c[i][1]), "+f"(c[i][2]), "+f"(c[i][3])
                             : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
            else
                asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                             "{%8,%9}, {%0,%1,%2,%3};"
                             : "+f"(c[i][0]), "+f"(c[i][1]), "+f"(c[i][2]), "+f"(c[i][3])
                             : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
        }
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += c[i][0] + c[i][1] + c[i][2] + c[i][3];
    if (s == -1.2345f) out[0] = s;
}

// L2 read bandwidth: every SM streams a buffer that L2 holds (no L1
// allocation), many times over
__global__ void k_l2_read(const float4 *buf, long n4, int reps, float *out)
{
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const long stride = (long)gridDim.x * blockDim.x;
    for (int r = 0; r < reps; ++r)
        for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n4; i += stride) {
            const float4 v = __ldcg(buf + i);
            acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
        }
    if (acc.x + acc.y + acc.z + acc.w == -1.2345f) out[0] = acc.x;
}

static int l2_read_gbs(cudaStream_t s, int sms, double *gbs)
{
    const long bytes = 48l << 20, n4 = bytes / 16;
    const int reps = 24;
    float4 *buf = nullptr;
    float *out = nullptr;
    if (cudaMalloc(&buf, bytes) != cudaSuccess) return NRLTB_E_NOMEM;
    if (cudaMalloc(&out, 64) != cudaSuccess) { cudaFree(buf); return NRLTB_E_NOMEM; }
    cudaMemsetAsync(buf, 0, bytes, s);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0, s);
        k_l2_read<<<sms * 4, 512, 0, s>>>(buf, n4, reps, out);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess) return NRLTB_E_CUDA;
    *gbs = (double)bytes * reps / (best * 1e-3) / 1e9;
    return NRLTB_OK;
}

extern "C" int nrltb_bench_peak(nrltb_ctx *ctx, int kind, double *tflops)
{
    if (!ctx || !tflops || kind < 0 || kind > 4) return NRLTB_E_ARG;
    cudaStream_t s = nrltb_ctx_stream_internal(ctx);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (kind == 4) return l2_read_gbs(s, sms, tflops);
    void *buf = nullptr;
    if (cudaMalloc(&buf, 64) != cudaSuccess) return NRLTB_E_NOMEM;
    const int threads = (kind >= 2) ? 256 : 512, blocks = sms * 4;
    const int iters = (kind == 0) ? 64 : (kind == 1 ? 4096 : 2048);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0, s);
        if (kind == 0) k_fma_peak<double><<<blocks, threads, 0, s>>>((double *)buf, iters, 0.999999, 1e-7);
        else if (kind == 1) k_fma_peak<float><<<blocks, threads, 0, s>>>((float *)buf, iters, 0.9999f, 1e-4f);
        else if (kind == 2) k_mma_peak<2><<<blocks, threads, 0, s>>>((float *)buf, iters);
        else k_mma_peak<3><<<blocks, threads, 0, s>>>((float *)buf, iters);
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
    double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
    if (kind >= 2) flops = (kind == 2 ? 4096.0 : 2048.0) * 8 * (double)iters * (threads / 32) * blocks;
    *tflops = flops / (best * 1e-3) / 1e12;
    return NRLTB_OK;
}

template <typename T, bool SIMT>
static void one_gemm(cudaStream_t s, int n, int batch, const typename cplx<T>::t *A, const typename cplx<T>::t *B,
                     typename cplx<T>::t *C)
{
    typedef typename cplx<T>::t C2;
    const C2 one = cmk<T>(1, 0), zero = cmk<T>(0, 0);
    const long st = (long)n * n;
    if (SIMT) zgemm_simt<T>(s, n, n, n, batch, one, A, n, st, 0, B, n, st, 0, zero, C, n, st);
    else zgemm<T>(s, n, n, n, batch, one, A, n, st, 0, B, n, st, 0, zero, C, n, st);
}

template <typename T, bool SIMT>
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
    one_gemm<T, SIMT>(s, n, batch, A, B, C);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    for (int r = 0; r < reps; ++r) one_gemm<T, SIMT>(s, n, batch, A, B, C);
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
    if (precision < 0 || precision > 2) return NRLTB_E_ARG;
    int rc = precision == 0   ? time_gemm<double, true>(s, n, batch, reps, ms_per_launch)
             : precision == 1 ? time_gemm<float, false>(s, n, batch, reps, ms_per_launch)
                              : time_gemm<float, true>(s, n, batch, reps, ms_per_launch);
    *flops_per_launch = 8.0 * n * (double)n * n * batch;
    return rc;
}

// the refinement product Y = A X by either method; `work` holds ozaki_work_bytes
static void refprod(cudaStream_t s, int method, int n, int batch, const double2 *A, float2 *X, double2 *Y,
                    void *work)
{
    const long nn = (long)n * n;
    if (method == 0) {
        dfgemm<double2, float2>(s, n, n, n, batch, A, n, nn, 0, X, n, nn, 0, Y, n, nn);
    } else {
        const OzakiX ox = ozaki_prepare_x(s, X, n, batch, work);
        ozaki_gemm(s, ox, A, Y, method == 2 ? 3 : 6);
    }
}

struct DevBufs {
    void *p[4] = {nullptr, nullptr, nullptr, nullptr};
    ~DevBufs() { for (void *q : p) if (q) cudaFree(q); }
};

extern "C" int nrltb_bench_refprod(nrltb_ctx *ctx, int method, int n, int batch, int reps, double *ms_per_launch,
                                   double *flops_per_launch)
{
    if (!ctx || method < 0 || method > 2 || n < 1 || batch < 1 || reps < 1 || !ms_per_launch ||
        !flops_per_launch)
        return NRLTB_E_ARG;
    cudaStream_t s = nrltb_ctx_stream_internal(ctx);
    const size_t nn = (size_t)n * n * batch;
    DevBufs d;
    if (cudaMalloc(&d.p[0], sizeof(double2) * nn) != cudaSuccess ||
        cudaMalloc(&d.p[1], sizeof(double2) * nn) != cudaSuccess ||
        cudaMalloc(&d.p[2], sizeof(float2) * nn) != cudaSuccess ||
        cudaMalloc(&d.p[3], ozaki_work_bytes(n, batch)) != cudaSuccess)
        return NRLTB_E_NOMEM;
    double2 *A = (double2 *)d.p[0], *Y = (double2 *)d.p[1];
    float2 *X = (float2 *)d.p[2];
    cudaMemsetAsync(A, 0, sizeof(double2) * nn, s);
    cudaMemsetAsync(X, 0, sizeof(float2) * nn, s);
    refprod(s, method, n, batch, A, X, Y, d.p[3]);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    for (int r = 0; r < reps; ++r) {
        refprod(s, method, n, batch, A, X, Y, d.p[3]);
        refprod(s, method, n, batch, A, X, Y, d.p[3]);
    }
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_per_launch = t / (2.0 * reps);
    *flops_per_launch = 8.0 * n * (double)n * n * batch;
    return cudaGetLastError() == cudaSuccess ? NRLTB_OK : NRLTB_E_CUDA;
}

extern "C" int nrltb_bench_refprod_run(nrltb_ctx *ctx, int method, int n, int batch, const double *A, float *X,
                                       double *Y)
{
    if (!ctx || method < 0 || method > 2 || n < 1 || batch < 1 || !A || !X || !Y) return NRLTB_E_ARG;
    cudaStream_t s = nrltb_ctx_stream_internal(ctx);
    const size_t nn = (size_t)n * n * batch;
    DevBufs d;
    if (cudaMalloc(&d.p[0], sizeof(double2) * nn) != cudaSuccess ||
        cudaMalloc(&d.p[1], sizeof(double2) * nn) != cudaSuccess ||
        cudaMalloc(&d.p[2], sizeof(float2) * nn) != cudaSuccess ||
        cudaMalloc(&d.p[3], ozaki_work_bytes(n, batch)) != cudaSuccess)
        return NRLTB_E_NOMEM;
    if (cudaMemcpyAsync(d.p[0], A, sizeof(double2) * nn, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(d.p[2], X, sizeof(float2) * nn, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return NRLTB_E_CUDA;
    refprod(s, method, n, batch, (const double2 *)d.p[0], (float2 *)d.p[2], (double2 *)d.p[1], d.p[3]);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(Y, d.p[1], sizeof(double2) * nn, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(X, d.p[2], sizeof(float2) * nn, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        nrltb_internal_set_error(cudaGetErrorString(e));
        return NRLTB_E_CUDA;
    }
    return NRLTB_OK;
}

extern "C" int nrltb_bench_cgemm_run(nrltb_ctx *ctx, int method, int m, int n, int k, int opA, int opB, int triA,
                                     int triB, int triC, const float alpha[2], const float beta[2], const float *A,
                                     int lda, const float *B, int ldb, float *C, int ldc)
{
    if (!ctx || method < 1 || method > 4 || m < 1 || n < 1 || k < 1 || !alpha || !beta || !A || !B || !C)
        return NRLTB_E_ARG;
    if (method == 3 && opA != 0) return NRLTB_E_ARG;
    if (opA < 0 || opA > 1 || opB < 0 || opB > 1 || triA < 0 || triA > 2 || triB < 0 || triB > 2 || triC < 0 ||
        triC > 2)
        return NRLTB_E_ARG;
    const long ra = opA ? k : m, ca = opA ? m : k, rb = opB ? n : k, cb = opB ? k : n;
    if (lda < ra || ldb < rb || ldc < m) return NRLTB_E_ARG;
    const size_t na = (size_t)lda * ca, nb = (size_t)ldb * cb, nc = (size_t)ldc * n;
    cudaStream_t s = nrltb_ctx_stream_internal(ctx);
    DevBufs d;
    if (cudaMalloc(&d.p[0], sizeof(float2) * na) != cudaSuccess ||
        cudaMalloc(&d.p[1], sizeof(float2) * nb) != cudaSuccess ||
        cudaMalloc(&d.p[2], sizeof(float2) * nc) != cudaSuccess)
        return NRLTB_E_NOMEM;
    if (cudaMemcpyAsync(d.p[0], A, sizeof(float2) * na, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(d.p[1], B, sizeof(float2) * nb, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(d.p[2], C, sizeof(float2) * nc, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return NRLTB_E_CUDA;
    const float2 al = make_float2(alpha[0], alpha[1]), be = make_float2(beta[0], beta[1]);
    const float2 *dA = (const float2 *)d.p[0], *dB = (const float2 *)d.p[1];
    float2 *dC = (float2 *)d.p[2];
    const GemmArgs<float> g = gemm_args<float>(m, n, k, 1, al, dA, lda, 0, opA, dB, ldb, 0, opB, be, dC, ldc, 0,
                                               triA, triB, triC);
    if (method == 1)
        zgemm<float>(s, m, n, k, 1, al, dA, lda, 0, opA, dB, ldb, 0, opB, be, dC, ldc, 0, triA, triB, triC);
    else if (method == 2)
        zgemm_simt<float>(s, m, n, k, 1, al, dA, lda, 0, opA, dB, ldb, 0, opB, be, dC, ldc, 0, triA, triB, triC);
    else if (method == 3)
        zgemm_umma_launch(s, g);
    else
        zgemm_tc_launch(s, g);
    if (cudaMemcpyAsync(C, dC, sizeof(float2) * nc, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return NRLTB_E_CUDA;
    return cudaGetLastError() == cudaSuccess ? NRLTB_OK : NRLTB_E_CUDA;
}

extern "C" int nrltb_bench_umma_fault(int clear)
{
    return (int)(zgemm_umma_fault(clear != 0) | (ozaki_fault(clear != 0) << 1));
}
