// dfgemm.cuh -- complex GEMM with double-float (FP32 pair) accumulation.
//
//   C = op(A) op(B)  (+ beta C), C stored as FP64 (double2)
//
// Operands are FP64 (double2, split on load into hi + lo FP32 parts) or FP32
// (float2, exact).  Every real product x*y is formed exactly as p + e with an
// FMA (e = fma(x, y, -p)) plus the lo cross terms, and p is added to a
// (hi, lo) FP32 accumulator with Knuth's TwoSum, so the result carries ~44
// significant bits: FP64-class accuracy at FP32 pipe rates.  This is the
// workhorse of the mixed-precision refinement (X^H H X, X^H S X) and of the
// mixed form's Hellmann-Feynman products.
#pragma once
#include "common.cuh"

namespace nrltb {

template <typename TA, typename TB> struct DfArgs {
    int m, n, k, batch;
    const TA *A; long lda, sA; int opA;
    const TB *B; long ldb, sB; int opB;
    double2 *C; long ldc, sC;
    double beta;                    // real beta (0 or 1)
    int triA, triC;                 // as in zgemm: triA 2 = op(A) upper; triC 1/2 = lower/upper tiles
};

__device__ __forceinline__ void split2(double2 v, float2 &h, float2 &l)
{
    h.x = (float)v.x; h.y = (float)v.y;
    l.x = (float)(v.x - (double)h.x); l.y = (float)(v.y - (double)h.y);
}
__device__ __forceinline__ void split2(float2 v, float2 &h, float2 &l) { h = v; l.x = 0.f; l.y = 0.f; }

template <typename T> struct is64 { static constexpr bool v = false; };
template <> struct is64<double2> { static constexpr bool v = true; };

// acc (hi, lo) += x*y with x = xh + xl, y = yh + yl (lo parts optional)
template <bool XL, bool YL>
__device__ __forceinline__ void dfmac(float &ah, float &al, float xh, float xl, float yh, float yl)
{
    float p = xh * yh;
    float e = fmaf(xh, yh, -p);
    if (YL) e = fmaf(xh, yl, e);
    if (XL) e = fmaf(xl, yh, e);
    float s = ah + p;
    float bb = s - ah;
    float err = (ah - (s - bb)) + (p - bb);
    ah = s;
    al += err + e;
}

template <typename TA, typename TB, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN)) k_dfgemm(DfArgs<TA, TB> g)
{
    constexpr bool AL = is64<TA>::v, BL = is64<TB>::v;
    constexpr int NT = (BM / TM) * (BN / TN);
    __shared__ float2 Ah[BK][BM + 1], Al[AL ? BK : 1][AL ? BM + 1 : 1];
    __shared__ float2 Bh[BK][BN + 1], Bl[BL ? BK : 1][BL ? BN + 1 : 1];
    const int b = blockIdx.z, m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    if (g.triC == 1 && m0 + BM - 1 < n0) return;
    if (g.triC == 2 && n0 + BN - 1 < m0) return;
    const TA *A = g.A + b * g.sA;
    const TB *B = g.B + b * g.sB;
    double2 *C = g.C + b * g.sC;
    int kbeg = 0, kend = g.k;
    if (g.triA == 2) kbeg = (m0 / BK) * BK;
    const int tid = threadIdx.x, tx = tid % (BM / TM), ty = tid / (BM / TM);
    float acc[TM][TN][4];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;
    for (int k0 = kbeg; k0 < kend; k0 += BK) {
        for (int e = tid; e < BM * BK; e += NT) {
            int i, kk;
            if (g.opA == 0) { i = e % BM; kk = e / BM; } else { kk = e % BK; i = e / BK; }
            const int m = m0 + i, k = k0 + kk;
            TA v;
            v.x = 0; v.y = 0;
            bool ok = m < g.m && k < kend && (g.triA != 2 || k >= m);
            if (ok) {
                v = (g.opA == 0) ? A[m + (long)k * g.lda] : A[k + (long)m * g.lda];
                if (g.opA == 1) v.y = -v.y;
            }
            float2 h, l;
            split2(v, h, l);
            Ah[kk][i] = h;
            if (AL) Al[kk][i] = l;
        }
        for (int e = tid; e < BN * BK; e += NT) {
            int j, kk;
            if (g.opB == 0) { kk = e % BK; j = e / BK; } else { j = e % BN; kk = e / BN; }
            const int n = n0 + j, k = k0 + kk;
            TB v;
            v.x = 0; v.y = 0;
            if (n < g.n && k < kend) {
                v = (g.opB == 0) ? B[k + (long)n * g.ldb] : B[n + (long)k * g.ldb];
                if (g.opB == 1) v.y = -v.y;
            }
            float2 h, l;
            split2(v, h, l);
            Bh[kk][j] = h;
            if (BL) Bl[kk][j] = l;
        }
        __syncthreads();
#pragma unroll 2
        for (int kk = 0; kk < BK; ++kk) {
            float2 ah[TM], al[TM], bh[TN], bl[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) {
                ah[i] = Ah[kk][tx + i * (BM / TM)];
                if (AL) al[i] = Al[kk][tx + i * (BM / TM)]; else al[i] = make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int j = 0; j < TN; ++j) {
                bh[j] = Bh[kk][ty + j * (BN / TN)];
                if (BL) bl[j] = Bl[kk][ty + j * (BN / TN)]; else bl[j] = make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) {
                    float *a = acc[i][j];
                    // re += ar br - ai bi ; im += ar bi + ai br
                    dfmac<AL, BL>(a[0], a[1], ah[i].x, al[i].x, bh[j].x, bl[j].x);
                    dfmac<AL, BL>(a[0], a[1], -ah[i].y, -al[i].y, bh[j].y, bl[j].y);
                    dfmac<AL, BL>(a[2], a[3], ah[i].x, al[i].x, bh[j].y, bl[j].y);
                    dfmac<AL, BL>(a[2], a[3], ah[i].y, al[i].y, bh[j].x, bl[j].x);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        const int m = m0 + tx + i * (BM / TM);
        if (m >= g.m) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int n = n0 + ty + j * (BN / TN);
            if (n >= g.n) continue;
            double2 v = make_double2((double)acc[i][j][0] + (double)acc[i][j][1],
                                     (double)acc[i][j][2] + (double)acc[i][j][3]);
            double2 *c = C + m + (long)n * g.ldc;
            if (g.beta != 0.0) { v.x += g.beta * c->x; v.y += g.beta * c->y; }
            *c = v;
        }
    }
}

template <typename TA, typename TB>
void dfgemm(cudaStream_t s, int m, int n, int k, int batch, const TA *A, long lda, long sA, int opA, const TB *B,
            long ldb, long sB, int opB, double2 *C, long ldc, long sC, double beta = 0.0, int triA = 0, int triC = 0)
{
    if (m <= 0 || n <= 0 || batch <= 0) return;
    DfArgs<TA, TB> g;
    g.m = m; g.n = n; g.k = k; g.batch = batch;
    g.A = A; g.lda = lda; g.sA = sA; g.opA = opA;
    g.B = B; g.ldb = ldb; g.sB = sB; g.opB = opB;
    g.C = C; g.ldc = ldc; g.sC = sC; g.beta = beta; g.triA = triA; g.triC = triC;
    constexpr int BM = 64, BN = 64, BK = 8, TM = 4, TN = 4;
    dim3 grid(cdiv(m, BM), cdiv(n, BN), batch);
    NRLTB_LAUNCH((k_dfgemm<TA, TB, BM, BN, BK, TM, TN>), grid, (BM / TM) * (BN / TN), 0, s, g);
}

}  // namespace nrltb
