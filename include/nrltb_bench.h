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

/* Peak of the FMA pipe on this GPU: kind 0 = FP64 (DFMA), 1 = FP32 (FFMA).
 * Independent FMA chains on every SM; returns TFLOP/s (2 flops per FMA). */
int nrltb_bench_peak(nrltb_ctx *ctx, int kind, double *tflops);

/* One batched complex GEMM launch of the eigensolver's kernel (C = A B, n x n x n,
 * `batch` matrices), precision 0 = FP64, 1 = FP32; averaged over `reps` launches
 * after a warm-up.  flops_per_launch = 8 n^3 batch. */
int nrltb_bench_zgemm(nrltb_ctx *ctx, int precision, int n, int batch, int reps,
                      double *ms_per_launch, double *flops_per_launch);

#ifdef __cplusplus
}
#endif
#endif
