// ozaki.cu -- FP64-accurate complex products Y = A X on the bf16 tensor cores.
//
// A (FP64, n x n, Hermitian: H or S) and X (FP32, n x n) are cut into exact
// integer digits (Ozaki's error-free splitting): row i of A is scaled by
// 2^-(e_i+1) (|A_ik| < 2^e_i) and written as sum_s d_s 256^-(s+1), s < 6,
// |d_s| <= 128; column j of X likewise with 3 digits.  X is first rounded in
// place to what its 3 digits hold (a change of at most 2^-23 of the column's
// largest element, far below the FP32 eigensolver's own error), so the
// products are formed for exactly the X every later step uses.
// Every digit is an integer that bf16 holds exactly and every digit product is
// <= 2^14.  A complex product takes three real ones (p1 = Ar Xr, p2 = Ai Xi,
// p3 = (Ar + Ai)(Xr + Xi), digit sums <= 256 are exact in bf16 too).  For a
// 64-wide k chunk each sum over the (at most 3) digit pairs of one weight
// 256^-(L+2), L = s + t, stays below 2^24 (p3: 64 * 3 * 2^16), so the tensor
// core's FP32 accumulation of one level and one chunk is exact, and so are
// re = p1 - p2 and im = p3 - (p1 + p2) (both below 2^23 in magnitude).  Each chunk's level sums are folded,
// scaled by 256^-(L+2), into a double-float (FP32 pair) accumulator.  Levels
// L <= 5 are kept (15 digit pairs); the dropped ones and the 6-digit cut of A
// are below 2^-48 of |A row| |X column| per term, the accuracy of the
// double-float SIMT product this replaces.  15 digit pairs x 3 real products
// = 45 bf16 MMAs per complex multiply-add, issued as mma.sync.m16n8k16.
//
// Because A is Hermitian, its row scale equals its column scale and row m is
// the conjugate of column m, so both are read with coalesced column accesses.
#include "common.cuh"
#include "ozaki.cuh"

namespace nrltb {

constexpr int OZ_SA = 6, OZ_SB = 3;       // digits of A (FP64) and X (FP32)
constexpr int OZ_T = 64;                  // CTA tile (m, n) and k chunk
constexpr int OZ_KP = OZ_T + 8;           // padded k stride in smem (bf16 units): 36 words
constexpr int OZ_THREADS = 256;           // 8 warps: 2 (m) x 4 (n), warp tile 32 x 16

static inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }
static inline int pad64(int n) { return (n + OZ_T - 1) / OZ_T * OZ_T; }

size_t ozaki_work_bytes(int n, int batch)
{
    const size_t np = (size_t)pad64(n), nb = (size_t)batch;
    return al256(sizeof(__nv_bfloat16) * np * np * nb * 2 * OZ_SA)   // A digits [s][re|im][b][m][k]
         + al256(sizeof(__nv_bfloat16) * np * np * nb * 2 * OZ_SB)   // X digits [t][re|im][b][n][k]
         + 2 * al256(sizeof(int) * np * nb) + 256;                    // exponents
}

// column exponents: e_j = smallest e with |M_kj| < 2^e for all k (re and im)
template <typename C2>
__global__ void k_oz_colexp(const C2 *M, int n, int np, int *ex, int batch)
{
    const int warp = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (warp >= np * batch) return;
    const int b = warp / np, j = warp % np;
    float mx = 0.f;
    if (j < n) {
        const C2 *col = M + (long)b * n * n + (long)j * n;
        for (int k = lane; k < n; k += 32) {
            const C2 v = col[k];
            mx = fmaxf(mx, fmaxf(fabsf((float)v.x), fabsf((float)v.y)));
        }
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) {
        int e;
        if (mx > 0.f) { frexpf(mx * 1.0000001f, &e); } else e = 0;   // |v| < 2^e (float max rounded up)
        ex[(long)b * np + j] = max(e, -100);   // keeps the digit scales 2^(23-e), 2^(47-e) finite
    }
}

// 2^k for -1022 <= k <= 1023, exact
__device__ __forceinline__ double pow2d(int k) { return __longlong_as_double((long long)(1023 + k) << 52); }
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }

// Balanced base-256 digits of an integer U (|U| <= 2^(8 nd - 1)), lowest first
// in d[nd-1]: every digit in [-128, 127] except the top one, which is in
// [-128, 128]; U = sum_s d[s] 256^(nd-1-s).
template <int ND>
__device__ __forceinline__ void digits_of(long long U, float d[ND])
{
#pragma unroll
    for (int s = ND - 1; s > 0; --s) {
        const int lo = (int)((U + 128) & 255) - 128;
        d[s] = (float)lo;
        U = (U - lo) >> 8;
    }
    d[0] = (float)U;
}

// A digits, written row-major per (m, k): D[s][c][b][m][k], c = 0 re, 1 im.
// A is Hermitian: A_mk = conj(A_km) is read down column m (coalesced).
// U = rint(A_mk 2^(47 - e_m)) (|U| <= 2^47, one rounding at 2^-48 of 2^(e_m+1))
// is cut into OZ_SA = 6 digits with integer arithmetic.
__global__ void k_oz_digits_a(const double2 *A, int n, int np, const int *ex, __nv_bfloat16 *D, int batch)
{
    const long npp = (long)np * np;
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= npp * batch) return;
    const int b = (int)(t / npp);
    const long e = t - b * npp;
    const int m = (int)(e / np), k = (int)(e % np);      // row-major: k fastest
    double2 v = make_double2(0.0, 0.0);
    if (m < n && k < n) {
        v = A[(long)b * n * n + k + (long)m * n];
        v.y = -v.y;
    }
    const double sc = pow2d(47 - ex[(long)b * np + m]);
    float dr[OZ_SA], di[OZ_SA];
    digits_of<OZ_SA>(__double2ll_rn(v.x * sc), dr);
    digits_of<OZ_SA>(__double2ll_rn(v.y * sc), di);
#pragma unroll
    for (int s = 0; s < OZ_SA; ++s) {
        D[(((long)s * 2 + 0) * batch + b) * npp + e] = __float2bfloat16_rn(dr[s]);
        D[(((long)s * 2 + 1) * batch + b) * npp + e] = __float2bfloat16_rn(di[s]);
    }
}

// X digits, stored per (n, k): D[t][c][b][n][k] (k fastest), X column-major FP32.
// U = rint(X_kn 2^(23 - f_n)) (|U| <= 2^23) is cut into OZ_SB = 3 digits and X
// itself is overwritten with U 2^(f_n - 23), the value its digits represent
// (exact in FP32).
__global__ void k_oz_digits_x(float2 *X, int n, int np, const int *ex, __nv_bfloat16 *D, int batch)
{
    const long npp = (long)np * np;
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= npp * batch) return;
    const int b = (int)(t / npp);
    const long e = t - b * npp;
    const int j = (int)(e / np), k = (int)(e % np);
    const bool in = j < n && k < n;
    const long xi = (long)b * n * n + k + (long)j * n;
    float2 v = make_float2(0.f, 0.f);
    if (in) v = X[xi];
    const int fj = ex[(long)b * np + j];
    const int ur = __float2int_rn(v.x * pow2f(23 - fj)), ui = __float2int_rn(v.y * pow2f(23 - fj));
    float dr[OZ_SB], di[OZ_SB];
    digits_of<OZ_SB>(ur, dr);
    digits_of<OZ_SB>(ui, di);
#pragma unroll
    for (int s = 0; s < OZ_SB; ++s) {
        D[(((long)s * 2 + 0) * batch + b) * npp + e] = __float2bfloat16_rn(dr[s]);
        D[(((long)s * 2 + 1) * batch + b) * npp + e] = __float2bfloat16_rn(di[s]);
    }
    if (in) X[xi] = make_float2((float)ur * pow2f(fj - 23), (float)ui * pow2f(fj - 23));
}

__device__ __forceinline__ void mma_bf16(float c[4], const unsigned a[4], const unsigned b[2])
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// sum of two packed pairs of bf16 digits: exact, the sums are integers of
// magnitude <= 256
__device__ __forceinline__ unsigned add_bf16x2(unsigned a, unsigned b)
{
    __nv_bfloat162 x = *reinterpret_cast<__nv_bfloat162 *>(&a), y = *reinterpret_cast<__nv_bfloat162 *>(&b);
    __nv_bfloat162 z = __hadd2(x, y);
    return *reinterpret_cast<unsigned *>(&z);
}

// (hi, lo) += v, v exact in FP64's sense once scaled by a power of two
__device__ __forceinline__ void df_add(float &hi, float &lo, float v)
{
    const float s = hi + v, bb = s - hi;
    lo += (hi - (s - bb)) + (v - bb);
    hi = s;
}

// One CTA: a 64 x 64 tile of Y for one matrix.  Shared memory holds, for one
// 64-wide k chunk, all digits of the A rows and X columns of the tile.
__global__ void __launch_bounds__(OZ_THREADS, 1)
k_oz_gemm(const __nv_bfloat16 *DA, const __nv_bfloat16 *DX, const int *exA, const int *exX, double2 *Y,
          int n, int np, int batch)
{
    extern __shared__ __align__(16) unsigned char smem[];
    // sA[s][c][64 rows][OZ_KP], sX[t][c][64 cols][OZ_KP]  (bf16)
    __nv_bfloat16 *sA = (__nv_bfloat16 *)smem;
    __nv_bfloat16 *sX = sA + OZ_SA * 2 * OZ_T * OZ_KP;
    const int b = blockIdx.z, m0 = blockIdx.y * OZ_T, n0 = blockIdx.x * OZ_T;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wm = (warp >> 2) * 32, wn = (warp & 3) * 16;     // warp tile origin
    const int g = lane >> 2, tq = lane & 3;
    const long npp = (long)np * np;
    // double-float accumulators: [mt 2][nt 2][frag 4] x (re, im) x (hi, lo)
    float hr[2][2][4], lr[2][2][4], hi_[2][2][4], li[2][2][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int q = 0; q < 4; ++q) hr[a][c][q] = lr[a][c][q] = hi_[a][c][q] = li[a][c][q] = 0.f;

    for (int k0 = 0; k0 < np; k0 += OZ_T) {
        __syncthreads();
        // stage the chunk: 16-byte vectors (8 bf16) along k
        for (int v = tid; v < OZ_SA * 2 * OZ_T * (OZ_T / 8); v += OZ_THREADS) {
            const int kv = v % (OZ_T / 8), r = (v / (OZ_T / 8)) % OZ_T, sc = v / (OZ_T / 8 * OZ_T);
            const uint4 d = *(const uint4 *)(DA + ((long)sc * batch + b) * npp + (long)(m0 + r) * np + k0 + kv * 8);
            *(uint4 *)(sA + ((long)sc * OZ_T + r) * OZ_KP + kv * 8) = d;
        }
        for (int v = tid; v < OZ_SB * 2 * OZ_T * (OZ_T / 8); v += OZ_THREADS) {
            const int kv = v % (OZ_T / 8), r = (v / (OZ_T / 8)) % OZ_T, sc = v / (OZ_T / 8 * OZ_T);
            const uint4 d = *(const uint4 *)(DX + ((long)sc * batch + b) * npp + (long)(n0 + r) * np + k0 + kv * 8);
            *(uint4 *)(sX + ((long)sc * OZ_T + r) * OZ_KP + kv * 8) = d;
        }
        __syncthreads();
#pragma unroll 1
        for (int L = 0; L <= OZ_SA - 1; ++L) {
            // level sums: p1 = Ar Xr, p2 = Ai Xi, p3 = (Ar + Ai)(Xr + Xi) (three real
            // products per complex one); re = p1 - p2, im = p3 - p1 - p2
            float p1[2][2][4], p2[2][2][4], p3[2][2][4];
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int c = 0; c < 2; ++c)
#pragma unroll
                    for (int q = 0; q < 4; ++q) p1[a][c][q] = p2[a][c][q] = p3[a][c][q] = 0.f;
#pragma unroll 1
            for (int t = 0; t < OZ_SB; ++t) {
                const int s = L - t;
                if (s < 0 || s >= OZ_SA) continue;
                const unsigned *Ar = (const unsigned *)(sA + ((long)(s * 2 + 0) * OZ_T) * OZ_KP);
                const unsigned *Ai = (const unsigned *)(sA + ((long)(s * 2 + 1) * OZ_T) * OZ_KP);
                const unsigned *Xr = (const unsigned *)(sX + ((long)(t * 2 + 0) * OZ_T) * OZ_KP);
                const unsigned *Xi = (const unsigned *)(sX + ((long)(t * 2 + 1) * OZ_T) * OZ_KP);
                constexpr int W = OZ_KP / 2;   // row stride in 32-bit words
#pragma unroll
                for (int kk = 0; kk < OZ_T; kk += 16) {
                    const int kw = kk / 2;
                    unsigned ar[2][4], ai[2][4], as[2][4];
#pragma unroll
                    for (int a = 0; a < 2; ++a) {
                        const int r0 = wm + a * 16 + g;
                        ar[a][0] = Ar[r0 * W + kw + tq];
                        ar[a][1] = Ar[(r0 + 8) * W + kw + tq];
                        ar[a][2] = Ar[r0 * W + kw + 4 + tq];
                        ar[a][3] = Ar[(r0 + 8) * W + kw + 4 + tq];
                        ai[a][0] = Ai[r0 * W + kw + tq];
                        ai[a][1] = Ai[(r0 + 8) * W + kw + tq];
                        ai[a][2] = Ai[r0 * W + kw + 4 + tq];
                        ai[a][3] = Ai[(r0 + 8) * W + kw + 4 + tq];
#pragma unroll
                        for (int q = 0; q < 4; ++q) as[a][q] = add_bf16x2(ar[a][q], ai[a][q]);
                    }
                    unsigned br[2][2], bi[2][2], bs[2][2];
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        const int c0 = wn + c * 8 + g;
                        br[c][0] = Xr[c0 * W + kw + tq];
                        br[c][1] = Xr[c0 * W + kw + 4 + tq];
                        bi[c][0] = Xi[c0 * W + kw + tq];
                        bi[c][1] = Xi[c0 * W + kw + 4 + tq];
                        bs[c][0] = add_bf16x2(br[c][0], bi[c][0]);
                        bs[c][1] = add_bf16x2(br[c][1], bi[c][1]);
                    }
                    // three rounds over the 12 accumulators: no MMA waits on the one before it
#pragma unroll
                    for (int c = 0; c < 2; ++c)
#pragma unroll
                        for (int a = 0; a < 2; ++a) mma_bf16(p1[a][c], ar[a], br[c]);
#pragma unroll
                    for (int c = 0; c < 2; ++c)
#pragma unroll
                        for (int a = 0; a < 2; ++a) mma_bf16(p2[a][c], ai[a], bi[c]);
#pragma unroll
                    for (int c = 0; c < 2; ++c)
#pragma unroll
                        for (int a = 0; a < 2; ++a) mma_bf16(p3[a][c], as[a], bs[c]);
                }
            }
            // fold this level of this chunk: exact integers scaled by 256^-(L+2).
            // Levels 0-2 by an exact two-sum into (hi, lo); from level 3 on the
            // contribution (< 2^-17 of the unit scale) goes straight into lo,
            // whose own rounding (2^-24 |lo|) already bounds the pair's error.
            const float w = ldexpf(1.0f, -8 * (L + 2));
            if (L < 3) {
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int c = 0; c < 2; ++c)
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const float re = p1[a][c][q] - p2[a][c][q];
                            const float im = p3[a][c][q] - (p1[a][c][q] + p2[a][c][q]);
                            df_add(hr[a][c][q], lr[a][c][q], re * w);
                            df_add(hi_[a][c][q], li[a][c][q], im * w);
                        }
            } else {
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int c = 0; c < 2; ++c)
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const float re = p1[a][c][q] - p2[a][c][q];
                            const float im = p3[a][c][q] - (p1[a][c][q] + p2[a][c][q]);
                            lr[a][c][q] = fmaf(re, w, lr[a][c][q]);
                            li[a][c][q] = fmaf(im, w, li[a][c][q]);
                        }
            }
        }
    }
    // scale by 2^(e_m + 1) 2^(f_n + 1) and store
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int m = m0 + wm + a * 16 + g + (q >= 2 ? 8 : 0);
                const int nn = n0 + wn + c * 8 + tq * 2 + (q & 1);
                if (m >= n || nn >= n) continue;
                const int sh = exA[(long)b * np + m] + exX[(long)b * np + nn] + 2;
                const double re = ldexp((double)hr[a][c][q] + (double)lr[a][c][q], sh);
                const double im = ldexp((double)hi_[a][c][q] + (double)li[a][c][q], sh);
                Y[(long)b * n * n + m + (long)nn * n] = make_double2(re, im);
            }
}

OzakiX ozaki_prepare_x(cudaStream_t s, float2 *X, int n, int batch, void *work)
{
    OzakiX ox;
    const int np = pad64(n);
    const size_t npp = (size_t)np * np;
    char *w = (char *)work;
    ox.DA = (__nv_bfloat16 *)w;
    ox.DX = (__nv_bfloat16 *)(w + al256(sizeof(__nv_bfloat16) * npp * batch * 2 * OZ_SA));
    ox.exA = (int *)((char *)ox.DX + al256(sizeof(__nv_bfloat16) * npp * batch * 2 * OZ_SB));
    ox.exX = (int *)((char *)ox.exA + al256(sizeof(int) * (size_t)np * batch));
    ox.n = n; ox.np = np; ox.batch = batch;
    NRLTB_LAUNCH(k_oz_colexp<float2>, cdiv((long)np * batch * 32, 256), 256, 0, s, X, n, np, ox.exX, batch);
    NRLTB_LAUNCH(k_oz_digits_x, cdiv((long)npp * batch, 256), 256, 0, s, X, n, np, ox.exX, ox.DX, batch);
    return ox;
}

void ozaki_gemm(cudaStream_t s, const OzakiX &ox, const double2 *A, double2 *Y)
{
    const int n = ox.n, np = ox.np, batch = ox.batch;
    const size_t npp = (size_t)np * np;
    NRLTB_LAUNCH(k_oz_colexp<double2>, cdiv((long)np * batch * 32, 256), 256, 0, s, A, n, np, ox.exA, batch);
    NRLTB_LAUNCH(k_oz_digits_a, cdiv((long)npp * batch, 256), 256, 0, s, A, n, np, ox.exA, ox.DA, batch);
    const int smem = (OZ_SA + OZ_SB) * 2 * OZ_T * OZ_KP * (int)sizeof(__nv_bfloat16);
    cudaFuncSetAttribute(k_oz_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    dim3 grid(np / OZ_T, np / OZ_T, batch);
    cudaEvent_t ev = kt_begin(s);
    NRLTB_LAUNCH(k_oz_gemm, grid, OZ_THREADS, smem, s, ox.DA, ox.DX, ox.exA, ox.exX, Y, n, np, batch);
    kt_end(ev, s, KC_DIGIT_GEMM, 8.0 * n * (double)n * n * batch);
}

}  // namespace nrltb
