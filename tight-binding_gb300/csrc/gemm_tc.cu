// gemm_tc.cu -- batched complex FP32 GEMM on the tensor cores ("3xTF32").
//
// Same contract as zgemm<float> (gemm.cuh): C = alpha op(A) op(B) + beta C,
// op in {N, C}, triangular trimming triA / triB / triC.  Each FP32 operand x
// is split in registers into a TF32 head h = tf32(x) and a TF32 tail
// l = tf32(x - h); every real product is formed as l_a h_b + h_a l_b + h_a h_b
// with mma.sync.m16n8k8 (FP32 accumulate), which carries ~FP32 accuracy (the
// dropped l_a l_b is 2^-22 relative) at tensor-core rates.  A complex
// multiply-add is four real products: 12 MMAs.
//
// CTA tile 64 x 64 (8 warps, warp tile 32 x 16, two CTAs per SM), 16-deep k
// slices staged through shared memory; the next slice is fetched into
// registers while the tensor cores work on the current one.
#include "common.cuh"
#include "gemm.cuh"

namespace nrltb {

constexpr int TC_BM = 64, TC_BN = 64, TC_BK = 16;
constexpr int TC_NT = 2;                                  // n8 tiles per warp (warp tile 32 x 16)
constexpr int TC_LDA = TC_BM + 4, TC_LDB = TC_BN + 4;   // [k][row] strides == 4 mod 16: conflict-free fragment loads
constexpr int TC_THREADS = 256;
constexpr int TC_AE = TC_BM * TC_BK / TC_THREADS;       // staged A elements per thread (8)
constexpr int TC_BE = TC_BN * TC_BK / TC_THREADS;       // staged B elements per thread (4)

__device__ __forceinline__ unsigned tf32_of(float x)
{
    unsigned r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}
// head and tail of x as TF32 bit patterns
__device__ __forceinline__ void tf32_split(float x, unsigned &h, unsigned &l)
{
    h = tf32_of(x);
    l = tf32_of(x - __uint_as_float(h));
}

__device__ __forceinline__ void mma_tf32(float c[4], const unsigned a[4], const unsigned b[2])
{
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// element (m, k) of op(A), zero outside the matrix, the k range or the triangle
__device__ __forceinline__ float2 tc_fetch_a(const GemmArgs<float> &g, const float2 *A, int m, int k, int kend)
{
    bool ok = m < g.m && k < kend;
    if (g.triA == 1) ok = ok && k <= m;
    if (g.triA == 2) ok = ok && k >= m;
    if (!ok) return make_float2(0.f, 0.f);
    if (g.opA == 0) return A[m + (long)k * g.lda];
    const float2 v = A[k + (long)m * g.lda];
    return make_float2(v.x, -v.y);
}
// element (k, n) of op(B)
__device__ __forceinline__ float2 tc_fetch_b(const GemmArgs<float> &g, const float2 *B, int k, int n, int kend)
{
    bool ok = n < g.n && k < kend;
    if (g.triB == 1) ok = ok && k <= n;
    if (g.triB == 2) ok = ok && k >= n;
    if (!ok) return make_float2(0.f, 0.f);
    if (g.opB == 0) return B[k + (long)n * g.ldb];
    const float2 v = B[n + (long)k * g.ldb];
    return make_float2(v.x, -v.y);
}
// staging maps: consecutive threads walk the contiguous global index
__device__ __forceinline__ void tc_a_pos(int opA, int e, int &i, int &kk)
{
    if (opA == 0) { i = e % TC_BM; kk = e / TC_BM; } else { kk = e % TC_BK; i = e / TC_BK; }
}
__device__ __forceinline__ void tc_b_pos(int opB, int e, int &kk, int &j)
{
    if (opB == 0) { kk = e % TC_BK; j = e / TC_BK; } else { j = e % TC_BN; kk = e / TC_BN; }
}

// Shared-memory layouts: an operand staged k-fastest (op(A) = A^H, op(B) = B,
// so that its global reads are coalesced) is kept [row][k] with a row stride of
// TC_LDK = 20 complex, otherwise [k][row]; both give conflict-free stores and
// fragment loads.
constexpr int TC_LDK = TC_BK + 4;
template <int KM>   // KM = 1: [row][k]
struct TcTile {
    float2 *p;
    int ld;   // [k][row] row stride
    __device__ float2 &at(int k, int row) const { return KM ? p[row * TC_LDK + k] : p[k * ld + row]; }
};

template <int TA, int TB>
__global__ void __launch_bounds__(TC_THREADS, 2) zgemm_tc_kernel(GemmArgs<float> g)
{
    __shared__ float2 As_[TA ? TC_BM * TC_LDK : TC_BK * TC_LDA];
    __shared__ float2 Bs_[TB ? TC_BN * TC_LDK : TC_BK * TC_LDB];
    const TcTile<TA> As{As_, TC_LDA};
    const TcTile<TB> Bs{Bs_, TC_LDB};
    const int b = blockIdx.z;
    const int m0 = blockIdx.x * TC_BM, n0 = blockIdx.y * TC_BN;
    if (g.triC == 1 && m0 + TC_BM - 1 < n0) return;
    if (g.triC == 2 && n0 + TC_BN - 1 < m0) return;
    const float2 *A = g.A + b * g.sA;
    const float2 *B = g.B + b * g.sB;
    float2 *Cm = g.C + b * g.sC;
    int kbeg = 0, kend = g.k;
    if (g.triA == 1) kend = min(kend, m0 + TC_BM);
    if (g.triA == 2) kbeg = max(kbeg, m0);
    if (g.triB == 1) kend = min(kend, n0 + TC_BN);
    if (g.triB == 2) kbeg = max(kbeg, n0);
    kbeg = (kbeg / TC_BK) * TC_BK;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wm = (warp & 1) * 32, wn = (warp >> 1) * (8 * TC_NT);
    const int gq = lane >> 2, tq = lane & 3;
    float accr[2][TC_NT][4], acci[2][TC_NT][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int c = 0; c < TC_NT; ++c)
#pragma unroll
            for (int q = 0; q < 4; ++q) accr[a][c][q] = acci[a][c][q] = 0.f;

    float2 ra[TC_AE], rb[TC_BE];
    auto fetch = [&](int k0) {
#pragma unroll
        for (int u = 0; u < TC_AE; ++u) {
            int i, kk;
            tc_a_pos(g.opA, tid + u * TC_THREADS, i, kk);
            ra[u] = tc_fetch_a(g, A, m0 + i, k0 + kk, kend);
        }
#pragma unroll
        for (int u = 0; u < TC_BE; ++u) {
            int kk, j;
            tc_b_pos(g.opB, tid + u * TC_THREADS, kk, j);
            rb[u] = tc_fetch_b(g, B, k0 + kk, n0 + j, kend);
        }
    };
    if (kbeg < kend) fetch(kbeg);
    for (int k0 = kbeg; k0 < kend; k0 += TC_BK) {
        __syncthreads();
#pragma unroll
        for (int u = 0; u < TC_AE; ++u) {
            int i, kk;
            tc_a_pos(g.opA, tid + u * TC_THREADS, i, kk);
            As.at(kk, i) = ra[u];
        }
#pragma unroll
        for (int u = 0; u < TC_BE; ++u) {
            int kk, j;
            tc_b_pos(g.opB, tid + u * TC_THREADS, kk, j);
            Bs.at(kk, j) = rb[u];
        }
        __syncthreads();
        if (k0 + TC_BK < kend) fetch(k0 + TC_BK);
#pragma unroll
        for (int ks = 0; ks < TC_BK; ks += 8) {
            // B fragments (k8 x n8) of the warp's 4 column tiles: head/tail of re, im
            unsigned brh[TC_NT][2], brl[TC_NT][2], bih[TC_NT][2], bil[TC_NT][2];
#pragma unroll
            for (int c = 0; c < TC_NT; ++c)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float2 v = Bs.at(ks + tq + 4 * h, wn + c * 8 + gq);
                    tf32_split(v.x, brh[c][h], brl[c][h]);
                    tf32_split(v.y, bih[c][h], bil[c][h]);
                }
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                // A fragment (m16 x k8): regs (g, tq), (g+8, tq), (g, tq+4), (g+8, tq+4)
                unsigned arh[4], arl[4], aih[4], ail[4], anh[4], anl[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int r = wm + a * 16 + gq + 8 * (q & 1), kq = ks + tq + 4 * (q >> 1);
                    const float2 v = As.at(kq, r);
                    tf32_split(v.x, arh[q], arl[q]);
                    tf32_split(v.y, aih[q], ail[q]);
                    anh[q] = aih[q] ^ 0x80000000u;
                    anl[q] = ail[q] ^ 0x80000000u;
                }
                // small terms first, then the head products; 8 independent chains per round
#pragma unroll
                for (int c = 0; c < TC_NT; ++c) { mma_tf32(accr[a][c], arl, brh[c]); mma_tf32(acci[a][c], arl, bih[c]); }
#pragma unroll
                for (int c = 0; c < TC_NT; ++c) { mma_tf32(accr[a][c], arh, brl[c]); mma_tf32(acci[a][c], arh, bil[c]); }
#pragma unroll
                for (int c = 0; c < TC_NT; ++c) { mma_tf32(accr[a][c], anl, bih[c]); mma_tf32(acci[a][c], ail, brh[c]); }
#pragma unroll
                for (int c = 0; c < TC_NT; ++c) { mma_tf32(accr[a][c], anh, bil[c]); mma_tf32(acci[a][c], aih, brl[c]); }
#pragma unroll
                for (int c = 0; c < TC_NT; ++c) { mma_tf32(accr[a][c], arh, brh[c]); mma_tf32(acci[a][c], arh, bih[c]); }
#pragma unroll
                for (int c = 0; c < TC_NT; ++c) { mma_tf32(accr[a][c], anh, bih[c]); mma_tf32(acci[a][c], aih, brh[c]); }
            }
        }
    }
    const bool beta0 = (g.beta.x == 0.f && g.beta.y == 0.f);
    // the old C first (loads in flight together: a load after a store to C
    // could alias it and would wait for it)
    float2 cold[2][TC_NT][4];
    if (!beta0) {
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int c = 0; c < TC_NT; ++c)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int m = m0 + wm + a * 16 + gq + (q >= 2 ? 8 : 0);
                    const int n = n0 + wn + c * 8 + 2 * tq + (q & 1);
                    cold[a][c][q] = (m < g.m && n < g.n) ? Cm[m + (long)n * g.ldc] : make_float2(0.f, 0.f);
                }
    }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int c = 0; c < TC_NT; ++c)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int m = m0 + wm + a * 16 + gq + (q >= 2 ? 8 : 0);
                const int n = n0 + wn + c * 8 + 2 * tq + (q & 1);
                if (m >= g.m || n >= g.n) continue;
                float2 *cp = Cm + m + (long)n * g.ldc;
                float2 v = cmul(g.alpha, make_float2(accr[a][c][q], acci[a][c][q]));
                if (!beta0) v = cadd(v, cmul(g.beta, cold[a][c][q]));
                *cp = v;
            }
}

void zgemm_tc_launch(cudaStream_t s, const GemmArgs<float> &g)
{
    dim3 grid(cdiv(g.m, TC_BM), cdiv(g.n, TC_BN), g.batch);
    const bool ta = g.opA == 1, tb = g.opB == 0;
    if (ta && tb) NRLTB_LAUNCH((zgemm_tc_kernel<1, 1>), grid, TC_THREADS, 0, s, g);
    else if (ta) NRLTB_LAUNCH((zgemm_tc_kernel<1, 0>), grid, TC_THREADS, 0, s, g);
    else if (tb) NRLTB_LAUNCH((zgemm_tc_kernel<0, 1>), grid, TC_THREADS, 0, s, g);
    else NRLTB_LAUNCH((zgemm_tc_kernel<0, 0>), grid, TC_THREADS, 0, s, g);
}

}  // namespace nrltb
