// gemm.cuh -- batched complex GEMM for the eigensolver's blocked updates.
//
//   C[b] = alpha * op(A[b]) * op(B[b]) + beta * C[b],   op in {N, C = conj-transpose}
//
// Column-major interleaved complex storage (LAPACK layout), any m, n, k.
// Triangular structure is exploited by trimming each tile's k range:
//   triA = 1: op(A) lower (k <= m), 2: op(A) upper (k >= m)
//   triB = 1: op(B) upper (k <= n), 2: op(B) lower (k >= n)
// and elements outside the triangle are read as zero, so the other half of a
// triangular operand may hold anything.  triC = 1 (2) computes only the tiles
// that touch the lower (upper) triangle of C.
//
// SIMT register-tiled kernel: a BM x BN tile per CTA, BK-deep k slices staged
// through shared memory, TM x TN complex outputs per thread.  FP64 runs here
// (GB300 has no FP64 tensor path); FP32 goes to the tensor cores
// (gemm_umma.cu, gemm_tc.cu).
#pragma once
#include <algorithm>
#include "common.cuh"

namespace nrltb {

template <typename T> struct GemmArgs {
    typedef typename cplx<T>::t C2;
    int m, n, k, batch;
    const C2 *A; long lda, sA; int opA;
    const C2 *B; long ldb, sB; int opB;
    C2 *C; long ldc, sC;
    C2 alpha, beta;
    int triA, triB, triC;
};

template <typename T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
zgemm_kernel(GemmArgs<T> g)
{
    typedef typename cplx<T>::t C2;
    constexpr int NT = (BM / TM) * (BN / TN);
    __shared__ C2 As[BK][BM + 1];
    __shared__ C2 Bs[BK][BN + 1];
    const int b = blockIdx.z;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    if (g.triC == 1 && m0 + BM - 1 < n0) return;
    if (g.triC == 2 && n0 + BN - 1 < m0) return;
    const C2 *A = g.A + b * g.sA;
    const C2 *B = g.B + b * g.sB;
    C2 *Cm = g.C + b * g.sC;
    int kbeg = 0, kend = g.k;
    if (g.triA == 1) kend = min(kend, m0 + BM);
    if (g.triA == 2) kbeg = max(kbeg, m0);
    if (g.triB == 1) kend = min(kend, n0 + BN);
    if (g.triB == 2) kbeg = max(kbeg, n0);
    kbeg = (kbeg / BK) * BK;

    const int tid = threadIdx.x;
    const int tx = tid % (BM / TM), ty = tid / (BM / TM);
    C2 acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = cmk<T>(0, 0);

    for (int k0 = kbeg; k0 < kend; k0 += BK) {
        // ---- stage op(A)[m0:m0+BM, k0:k0+BK] as As[kk][i] ----
        if (g.opA == 0) {
            for (int e = tid; e < BM * BK; e += NT) {
                int i = e % BM, kk = e / BM;
                int m = m0 + i, k = k0 + kk;
                C2 v = cmk<T>(0, 0);
                bool ok = m < g.m && k < kend;
                if (g.triA == 1) ok = ok && k <= m;
                if (g.triA == 2) ok = ok && k >= m;
                if (ok) v = A[m + (long)k * g.lda];
                As[kk][i] = v;
            }
        } else {
            for (int e = tid; e < BM * BK; e += NT) {
                int kk = e % BK, i = e / BK;
                int m = m0 + i, k = k0 + kk;
                C2 v = cmk<T>(0, 0);
                bool ok = m < g.m && k < kend;
                if (g.triA == 1) ok = ok && k <= m;
                if (g.triA == 2) ok = ok && k >= m;
                if (ok) v = cconj(A[k + (long)m * g.lda]);
                As[kk][i] = v;
            }
        }
        // ---- stage op(B)[k0:k0+BK, n0:n0+BN] as Bs[kk][j] ----
        if (g.opB == 0) {
            for (int e = tid; e < BN * BK; e += NT) {
                int kk = e % BK, j = e / BK;
                int n = n0 + j, k = k0 + kk;
                C2 v = cmk<T>(0, 0);
                bool ok = n < g.n && k < kend;
                if (g.triB == 1) ok = ok && k <= n;
                if (g.triB == 2) ok = ok && k >= n;
                if (ok) v = B[k + (long)n * g.ldb];
                Bs[kk][j] = v;
            }
        } else {
            for (int e = tid; e < BN * BK; e += NT) {
                int j = e % BN, kk = e / BN;
                int n = n0 + j, k = k0 + kk;
                C2 v = cmk<T>(0, 0);
                bool ok = n < g.n && k < kend;
                if (g.triB == 1) ok = ok && k <= n;
                if (g.triB == 2) ok = ok && k >= n;
                if (ok) v = cconj(B[n + (long)k * g.ldb]);
                Bs[kk][j] = v;
            }
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            C2 a[TM], bb[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) a[i] = As[kk][tx + i * (BM / TM)];
#pragma unroll
            for (int j = 0; j < TN; ++j) bb[j] = Bs[kk][ty + j * (BN / TN)];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) cfma(acc[i][j], a[i], bb[j]);
        }
        __syncthreads();
    }
    const bool beta0 = (g.beta.x == T(0) && g.beta.y == T(0));
    // FP32: the old C first (loads in flight together: a load after a store to
    // C could alias it and would wait for it); FP64 keeps the registers for
    // occupancy and loads each element before its store
    constexpr bool PRE = sizeof(T) == 4;
    C2 cold[PRE ? TM : 1][PRE ? TN : 1];
    if (PRE && !beta0) {
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j) {
                const int m = m0 + tx + i * (BM / TM), n = n0 + ty + j * (BN / TN);
                cold[PRE ? i : 0][PRE ? j : 0] = (m < g.m && n < g.n) ? Cm[m + (long)n * g.ldc] : cmk<T>(0, 0);
            }
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        int m = m0 + tx + i * (BM / TM);
        if (m >= g.m) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            int n = n0 + ty + j * (BN / TN);
            if (n >= g.n) continue;
            C2 *c = Cm + m + (long)n * g.ldc;
            C2 v = cmul(g.alpha, acc[i][j]);
            if (!beta0) v = cadd(v, cmul(g.beta, PRE ? cold[PRE ? i : 0][PRE ? j : 0] : *c));
            *c = v;
        }
    }
}

// FP32 on the tensor cores: tcgen05 with tensor-memory accumulators for
// op(A) = A (gemm_umma.cu), mma.sync otherwise (gemm_tc.cu)
void zgemm_tc_launch(cudaStream_t s, const GemmArgs<float> &g);
bool zgemm_umma_supported(const GemmArgs<float> &g);
void zgemm_umma_launch(cudaStream_t s, const GemmArgs<float> &g);
// fault flag of the tcgen05 kernel (a barrier wait that ran out); clear resets it
unsigned zgemm_umma_fault(bool clear);

// dst = src^H for `batch` rows x cols matrices (src leading dimension lds,
// stride ss; dst leading dimension ldd, stride ds), 32 x 32 tiles through
// shared memory so both sides are coalesced
template <typename C2>
__global__ void k_conj_transpose(const C2 *src, long lds, long ss, C2 *dst, long ldd, long ds, int rows, int cols)
{
    __shared__ C2 t[32][33];
    const C2 *S = src + blockIdx.z * ss;
    C2 *D = dst + blockIdx.z * ds;
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int r = r0 + threadIdx.x, c = c0 + q;
        if (r < rows && c < cols) t[q][threadIdx.x] = S[r + (long)c * lds];
    }
    __syncthreads();
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int c = c0 + threadIdx.x, r = r0 + q;   // D(c, r) = conj(S(r, c))
        if (r < rows && c < cols) {
            C2 v = t[threadIdx.x][q];
            v.y = -v.y;
            D[c + (long)r * ldd] = v;
        }
    }
}
template <typename T>
void conj_transpose(cudaStream_t s, const typename cplx<T>::t *src, long lds, long ss, typename cplx<T>::t *dst,
                    long ldd, long ds, int rows, int cols, int batch)
{
    NRLTB_LAUNCH(k_conj_transpose<typename cplx<T>::t>, dim3(cdiv(cols, 32), cdiv(rows, 32), batch), dim3(32, 8), 0,
                 s, src, lds, ss, dst, ldd, ds, rows, cols);
}
template <typename T>
void conj_transpose(cudaStream_t s, const typename cplx<T>::t *src, typename cplx<T>::t *dst, int n, int batch)
{
    conj_transpose<T>(s, src, n, (long)n * n, dst, n, (long)n * n, n, n, batch);
}

// complex multiply-adds a GEMM with these triangle flags needs (the zeros of a
// triangular operand and the skipped triangle of C excluded); for the
// kernel-class timing, evaluated only while it is on
inline double gemm_useful_macs(int m, int n, int k, int triA, int triB, int triC)
{
    auto krange = [&](int i, int j) {
        int lo = 0, hi = k;
        if (triA == 1) hi = std::min(hi, i + 1);
        if (triA == 2) lo = std::max(lo, i);
        if (triB == 1) hi = std::min(hi, j + 1);
        if (triB == 2) lo = std::max(lo, j);
        return (double)std::max(hi - lo, 0);
    };
    if (!triA && !triB && !triC) return (double)m * n * k;
    double sum = 0;
    if (!triB && !triC) {
        for (int i = 0; i < m; ++i) sum += krange(i, 0);
        return sum * n;
    }
    if (!triA && !triC) {
        for (int j = 0; j < n; ++j) sum += krange(0, j);
        return sum * m;
    }
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < n; ++j) {
            if (triC == 1 && j > i) continue;
            if (triC == 2 && j < i) continue;
            sum += krange(i, j);
        }
    return sum;
}

template <typename T>
GemmArgs<T> gemm_args(int m, int n, int k, int batch, typename cplx<T>::t alpha,
                      const typename cplx<T>::t *A, long lda, long sA, int opA,
                      const typename cplx<T>::t *B, long ldb, long sB, int opB,
                      typename cplx<T>::t beta, typename cplx<T>::t *C, long ldc, long sC,
                      int triA, int triB, int triC)
{
    GemmArgs<T> g;
    g.m = m; g.n = n; g.k = k; g.batch = batch;
    g.A = A; g.lda = lda; g.sA = sA; g.opA = opA;
    g.B = B; g.ldb = ldb; g.sB = sB; g.opB = opB;
    g.C = C; g.ldc = ldc; g.sC = sC;
    g.alpha = alpha; g.beta = beta;
    g.triA = triA; g.triB = triB; g.triC = triC;
    return g;
}

// the SIMT kernel in either precision
template <typename T>
void zgemm_simt(cudaStream_t s, int m, int n, int k, int batch, typename cplx<T>::t alpha,
                const typename cplx<T>::t *A, long lda, long sA, int opA,
                const typename cplx<T>::t *B, long ldb, long sB, int opB,
                typename cplx<T>::t beta, typename cplx<T>::t *C, long ldc, long sC,
                int triA = 0, int triB = 0, int triC = 0)
{
    if (m <= 0 || n <= 0 || batch <= 0) return;
    const GemmArgs<T> g = gemm_args<T>(m, n, k, batch, alpha, A, lda, sA, opA, B, ldb, sB, opB, beta, C, ldc, sC,
                                       triA, triB, triC);
    constexpr int BM = 64, BN = 64, TM = 4, TN = 4;
    dim3 grid(cdiv(m, BM), cdiv(n, BN), batch);
    cudaEvent_t ev = kt_begin(s);
    // short k (the rank-32 panel updates): the whole k range in one or two
    // shared-memory stages instead of four to eight; n <= 32 (the Cholesky
    // panel solves) on 64 x 32 tiles.  Every element's k loop is the same in
    // each form.
    constexpr int BKS = sizeof(T) == 4 ? 32 : 16;
    if (k <= 64 && n <= 32)
        NRLTB_LAUNCH((zgemm_kernel<T, BM, 32, BKS, TM, 2>), dim3(cdiv(m, BM), 1, batch), (BM / TM) * (32 / 2), 0,
                     s, g);
    else if (k <= 64)
        NRLTB_LAUNCH((zgemm_kernel<T, BM, BN, BKS, TM, TN>), grid, (BM / TM) * (BN / TN), 0, s, g);
    else
        NRLTB_LAUNCH((zgemm_kernel<T, BM, BN, 8, TM, TN>), grid, (BM / TM) * (BN / TN), 0, s, g);
    if (ev) kt_end(ev, s, KC_GEMM_SIMT, 8.0 * gemm_useful_macs(m, n, k, triA, triB, triC) * batch);
}

// FP64: SIMT FMA pipe; FP32: tensor cores (3xTF32, FP32-class accuracy)
template <typename T>
void zgemm(cudaStream_t s, int m, int n, int k, int batch, typename cplx<T>::t alpha,
           const typename cplx<T>::t *A, long lda, long sA, int opA,
           const typename cplx<T>::t *B, long ldb, long sB, int opB,
           typename cplx<T>::t beta, typename cplx<T>::t *C, long ldc, long sC,
           int triA = 0, int triB = 0, int triC = 0)
{
    if (m <= 0 || n <= 0 || batch <= 0) return;
    // tensor cores for m >= 128, n >= 64: tcgen05 (op(A) = A) from k = 32,
    // mma.sync (op(A) = A^H) from k = 128; the rest on the FMA pipe
    if constexpr (sizeof(T) == 4) {
        const GemmArgs<float> g = gemm_args<T>(m, n, k, batch, alpha, A, lda, sA, opA, B, ldb, sB, opB, beta, C,
                                               ldc, sC, triA, triB, triC);
        const bool umma = zgemm_umma_supported(g);
        if (m < 128 || n < 64 || k < (umma ? 32 : 128)) {
            zgemm_simt<T>(s, m, n, k, batch, alpha, A, lda, sA, opA, B, ldb, sB, opB, beta, C, ldc, sC, triA, triB,
                          triC);
            return;
        }
        cudaEvent_t ev = kt_begin(s);
        if (umma) zgemm_umma_launch(s, g);
        else zgemm_tc_launch(s, g);
        if (ev) kt_end(ev, s, KC_GEMM_TC, 8.0 * gemm_useful_macs(m, n, k, triA, triB, triC) * batch);
    } else {
        zgemm_simt<T>(s, m, n, k, batch, alpha, A, lda, sA, opA, B, ldb, sB, opB, beta, C, ldc, sC, triA, triB,
                      triC);
    }
}

}  // namespace nrltb
