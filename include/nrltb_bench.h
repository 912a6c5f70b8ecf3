/*
 * nrltb_bench.h -- measurement hooks used by the benchmark, not part of the
 * reference's interface (they have no counterpart in the reference).
 * Both time their own launches with CUDA events on the context's stream.
 */
#ifndef NRLTB_BENCH_H
#define NRLTB_BENCH_H
#include "nrltb.h"
#ifdef __cplusplus
extern "C" {
#endif

/* Peak of one instruction pipe on this GPU: kind 0 = FP64 FMA, 1 = FP32 FMA
 * (2 flops per FMA), 2 = mma.sync bf16 m16n8k16, 3 = mma.sync tf32 m16n8k8
 * (FP32 accumulate; 2 m n k flops per MMA).  Independent chains on every SM;
 * returns TFLOP/s.  kind 4 = L2 read bandwidth (every SM streaming a 48 MiB
 * buffer that L2 holds, loads cached in L2 only); returns GB/s. */
int nrltb_bench_peak(nrltb_ctx *ctx, int kind, double *tflops);

/* One batched complex GEMM launch of the eigensolver's kernel (C = A B, n x n x n,
 * `batch` matrices): precision 0 = FP64 (SIMT FMA pipe), 1 = FP32 (tensor cores,
 * 3xTF32), 2 = FP32 on the SIMT FMA pipe (for comparison); averaged over `reps`
 * launches after a warm-up.  flops_per_launch = 8 n^3 batch. */
int nrltb_bench_zgemm(nrltb_ctx *ctx, int precision, int n, int batch, int reps,
                      double *ms_per_launch, double *flops_per_launch);

/* One FP64-accurate product Y = A X of the mixed form's refinement (A FP64
 * Hermitian, X FP32, both n x n complex, `batch` matrices): method 0 = the
 * double-float SIMT GEMM, 1 = the bf16 tensor-core digit product, 2 = the
 * same with A rounded to 3 digits (the mixed form's Hellmann-Feynman
 * products, FP32-class accuracy).  Averaged
 * over `reps` pairs of launches (H X and S X) after a warm-up;
 * flops_per_launch = 8 n^3 batch for one product. */
int nrltb_bench_refprod(nrltb_ctx *ctx, int method, int n, int batch, int reps,
                        double *ms_per_launch, double *flops_per_launch);

/* The same product on caller data, for accuracy checks: host arrays A
 * (batch x n x n complex FP64, column-major, interleaved re/im, Hermitian),
 * X (batch x n x n complex FP32; methods 1 and 2 round it in place to the
 * digits they use) and Y (batch x n x n complex FP64, out). */
int nrltb_bench_refprod_run(nrltb_ctx *ctx, int method, int n, int batch, const double *A, float *X,
                            double *Y);

/* One FP32 complex GEMM of the eigensolver's kernel on caller data, for
 * accuracy checks: C = alpha op(A) op(B) + beta C with the kernel's op and
 * triangle flags (gemm.cuh), one matrix; method 1 = the library's dispatch,
 * 2 = SIMT, 3 = the tcgen05 kernel (op A = N only), 4 = the mma.sync
 * tensor-core kernel.
 * A, B, C are host arrays (column-major complex FP32, leading dimensions
 * lda, ldb, ldc); alpha, beta are {re, im}. */
int nrltb_bench_cgemm_run(nrltb_ctx *ctx, int method, int m, int n, int k, int opA, int opB, int triA,
                          int triB, int triC, const float alpha[2], const float beta[2], const float *A,
                          int lda, const float *B, int ldb, float *C, int ldc);

/* Fault flags of the tcgen05 kernels: bit 0 the FP32 GEMM, bit 1 the
 * refinement's digit product; a bit is set once a bounded barrier wait inside
 * that kernel ran out (the kernel then leaves its output untouched).
 * clear = 1 resets both. */
int nrltb_bench_umma_fault(int clear);

/* Raise the context's own bounded-wait expiry word, as a tcgen05 kernel of
 * that context does when one of its barrier waits runs out.  The next solve
 * or Hellmann-Feynman step of the context then marks its k points
 * NRLTB_K_TIMEOUT and the call returns NRLTB_E_TIMEOUT; the word is cleared
 * when it is read.  For tests of that path (no device wait is made to expire). */
int nrltb_bench_raise_fault_word(nrltb_ctx *ctx);

/* Kernel-class timing of the context's own calls: with on = 1 every later
 * launch of a timed class (0 = FP32 tensor-core GEMM, 1 = SIMT GEMM, 2 = the
 * refinement's tensor-core digit product, 3 = the tridiagonalisation panel
 * kernel) is bracketed by CUDA events on the launching stream and tagged with
 * its algorithmic work (flops: 8 per complex multiply-add a GEMM needs, zeros
 * of triangular operands and a skipped triangle of C excluded; bytes: the
 * trailing lower triangles a panel reads).  Turning it on clears
 * the records; stats synchronizes the stream and sums one class. */
int nrltb_bench_kernel_timing(nrltb_ctx *ctx, int on);
int nrltb_bench_kernel_stats(nrltb_ctx *ctx, int cls, double *ms, double *work, int *launches);

#ifdef __cplusplus
}
#endif
#endif
