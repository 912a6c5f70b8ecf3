// ozaki.cuh -- FP64-accurate products Y = A X (A FP64 Hermitian, X FP32) on the
// bf16 tensor cores by exact digit splitting (ozaki.cu).
#pragma once
#include <cuda_bf16.h>
#include "common.cuh"

namespace nrltb {

struct OzakiX {
    __nv_bfloat16 *DA, *DX;    // digit planes of A (reused for each A) and of X
    int *exA, *exX;            // per-row (A) and per-column (X) binary exponents
    int n, np, batch;          // order, order padded to a multiple of 128, matrices
};

size_t ozaki_work_bytes(int n, int batch);
// Rounds X in place to its 3-digit representation (a change of at most 2^-23
// of each column's largest element) and splits it; work holds
// ozaki_work_bytes(n, batch) bytes, 256-byte aligned.
OzakiX ozaki_prepare_x(cudaStream_t s, float2 *X, int n, int batch, void *work);
// Y = A X for the batch, A column-major n x n Hermitian (both triangles stored).
// adigits = 6: A cut after 48 bits, digit levels up to 5 (FP64-accurate);
// adigits = 3: A rounded to 24 bits of its row scale, all 9 digit pairs
// (the exact product of the rounded A and X, FP32-class accuracy).
void ozaki_gemm(cudaStream_t s, const OzakiX &ox, const double2 *A, double2 *Y, int adigits = 6);
// A's digits prepared ahead of the product (on another stream, while other
// work runs): digit blocks and row exponents in caller-owned memory of
// ozaki_a_bytes(n, batch, adigits) bytes, 256-byte aligned.
struct OzakiA {
    const unsigned char *D;   // digit blocks of A (adigits planes)
    const int *ex;            // per-row binary exponents
    int sa;                   // digits: 6 or 3
};
size_t ozaki_a_bytes(int n, int batch, int adigits);
OzakiA ozaki_prepare_a(cudaStream_t s, const double2 *A, int n, int batch, int adigits, void *work);
// Y = A X with A's digits from ozaki_prepare_a (the same result as ozaki_gemm)
void ozaki_gemm_prepared(cudaStream_t s, const OzakiX &ox, const OzakiA &oa, double2 *Y);
// fault flag of the product kernel (a barrier wait that ran out); clear resets it
unsigned ozaki_fault(bool clear);

}  // namespace nrltb
