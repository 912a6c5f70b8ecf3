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
// <= 2^14.  A complex digit product takes four real ones.  For a 64-wide k
// chunk each sum over the (at most 3) digit pairs of one weight 256^-(L+2),
// L = s + t, stays below 2^21.6, so the tensor core's FP32 accumulation of one
// level and one chunk is exact, and so are re = Xr Ar - Xi Ai and
// im = Xr Ai + Xi Ar (below 2^22.6).  Each chunk's level sums are folded,
// scaled by 256^-(L+2), into a double-float (FP32 pair) accumulator.  Levels
// L <= 5 are kept (15 digit pairs); the dropped ones and the 6-digit cut of A
// are below 2^-48 of |A row| |X column| per term.  A 3-digit form (A rounded to
// 24 bits of its row scale, all 9 digit pairs, levels 0-4) gives the exact
// product of the rounded operands for the Hellmann-Feynman products.
//
// Tensor cores: tcgen05.mma kind::f16 (bf16 digits, FP32 accumulators in
// tensor memory).  Persistent CTAs, one per SM, take the 128 x 64 tiles of Y
// in turn (the barrier phases run on from tile to tile, so the next tile's
// copies and MMAs start while the folds write the last one).  In a tile the
// MMA's M = 128 rows are rows i of A (digit tiles Ar_s, Ai_s), its N = 128
// columns come
// from the digit rows [-Xi_t | Xr_t | Xi_t] of 64 columns j of X, so that
// Ar_s [Xr_t | Xi_t] + Ai_s [-Xi_t | Xr_t] accumulates [Re | Im] of a digit
// pair's product in one 128-column accumulator.  Digits are written pre-tiled
// in the 128-byte-swizzled K-major layout the MMA reads, so each tile is one
// bulk asynchronous copy (cp.async.bulk with a transaction-count barrier),
// and the planes a few ahead are brought into L2 by cp.async.bulk.prefetch.
// Warp roles: one producer thread (copies), one MMA thread, sixteen fold warps
// (tensor memory -> registers, double-float accumulation, output).  Within a
// chunk the A digit planes s = 0..5 stream through a ring while the chunk's X
// digits stay resident; plane s takes the digit pairs (s, 0), (s, 1), (s, 2),
// so level L is first touched at plane max(0, L - 2) and complete after plane
// L, and four 128-column tensor-memory level buffers let the folds run behind
// the MMAs.  Every barrier wait is bounded (about two seconds); on expiry the
// CTA records a fault flag and leaves Y untouched.
//
// Because A is Hermitian, its row scale equals its column scale and row m is
// the conjugate of column m, so both are read with coalesced column accesses.
#include <algorithm>
#include <cstdint>
#include "common.cuh"
#include "ozaki.cuh"

namespace nrltb {

constexpr int OZ_SA = 6, OZ_SB = 3;       // digits of A (FP64) and X (FP32)
constexpr int OZ_MA = 128;                // rows of A (and of Y) per CTA: tensor-memory lanes
constexpr int OZ_NX = 64;                 // columns of X (and of Y) per CTA
constexpr int OZ_BK = 64;                 // k chunk: one 128-byte swizzled row of bf16
constexpr int OZ_PAD = 128;               // n padded to a multiple of this (rows, columns, k)
constexpr int OZ_ABLK = 2 * OZ_MA * 128;          // A digit block (one s): Ar_s | Ai_s tiles, 32 KB
constexpr int OZ_XBLK = 3 * OZ_NX * 128;          // X digit block (one t): -Xi_t | Xr_t | Xi_t, 24 KB
constexpr int OZ_XSTAGE = OZ_SB * OZ_XBLK;        // a chunk's X digits, 72 KB
constexpr int OZ_NXS = 2;                 // X chunk stages
constexpr int OZ_NAS = 2;                 // A blocks in flight
constexpr int OZ_APF = 4;                 // A blocks ahead of the one being copied brought into L2
constexpr int OZ_NBUF = 4;                // tensor-memory level buffers, 128 columns each
constexpr int OZ_FOLD_WARPS = 16;         // 4 per 32-lane quarter, 16 columns each
constexpr int OZ_THREADS = 32 * (OZ_FOLD_WARPS + 2);   // + producer warp + MMA warp
constexpr int OZ_NBAR = 2 * OZ_NXS + 2 * OZ_NAS + 2 * OZ_NBUF;
constexpr int OZ_SMEM = OZ_NXS * OZ_XSTAGE + OZ_NAS * OZ_ABLK + 1024 + 8 * OZ_NBAR + 16;
constexpr uint32_t OZ_TMEM_COLS = 512;
constexpr unsigned long long OZ_WAIT_NS = 2000000000ull;
// instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28
constexpr uint32_t OZ_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(128 >> 3) << 17) |
                              ((uint32_t)(OZ_MA >> 4) << 24);

static inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }
static inline int padn(int n) { return (n + OZ_PAD - 1) / OZ_PAD * OZ_PAD; }

size_t ozaki_work_bytes(int n, int batch)
{
    const size_t np = (size_t)padn(n), nb = (size_t)batch;
    return al256(sizeof(__nv_bfloat16) * np * np * nb * 2 * OZ_SA)   // A digit blocks: Ar, Ai
         + al256(sizeof(__nv_bfloat16) * np * np * nb * 3 * OZ_SB)   // X digit blocks: -Xi, Xr, Xi
         + 2 * al256(sizeof(int) * np * nb) + 256;                    // exponents
}

__device__ unsigned g_oz_fault;

// column exponents: e_j = smallest e with |M_kj| < 2^e for all k (re and im)
// (from the largest |M_kj| rounded to FP32, with a margin for that rounding).
// FP64 M: the largest magnitude is found on the bit patterns (for finite
// non-negative doubles the integer order of the bits is the numeric order) and
// rounded to FP32 once per column, which gives the same value as rounding
// every element first (rounding is monotonic) without a conversion on the
// FP64 pipe per element.
template <typename C2>
__global__ void k_oz_colexp(const C2 *M, int n, int np, int *ex, int batch)
{
    const int warp = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (warp >= np * batch) return;
    const int b = warp / np, j = warp % np;
    float mx = 0.f;
    if constexpr (sizeof(M->x) == 8) {
        unsigned long long mb = 0;
        if (j < n) {
            const C2 *col = M + (long)b * n * n + (long)j * n;
            for (int k = lane; k < n; k += 32) {
                const C2 v = col[k];
                const unsigned long long ar = (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFull;
                const unsigned long long ai = (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFull;
                mb = max(mb, max(ar, ai));
            }
        }
        for (int o = 16; o > 0; o >>= 1) mb = max(mb, (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)mb, o));
        mx = (float)__longlong_as_double((long long)mb);
    } else {
        if (j < n) {
            const C2 *col = M + (long)b * n * n + (long)j * n;
            for (int k = lane; k < n; k += 32) {
                const C2 v = col[k];
                mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
            }
        }
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (lane == 0) {
        int e;
        if (mx > 0.f) { frexpf(mx * 1.0000001f, &e); } else e = 0;   // |v| < 2^e (float max rounded up)
        ex[(long)b * np + j] = max(e, -100);   // keeps the digit scales 2^(23-e), 2^(47-e) finite
    }
}

// 2^k for -1022 <= k <= 1023, exact
__device__ __forceinline__ double pow2d(int k) { return __longlong_as_double((long long)(1023 + k) << 52); }
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }

// v 2^k, exact: on the exponent field when the result stays a normal number
// (integer operations), else by the FP64 multiply
__device__ __forceinline__ double oz_scale2(double v, int k)
{
    const long long bits = __double_as_longlong(v);
    const int E = (int)((bits >> 52) & 0x7FF);
    if ((bits & 0x7FFFFFFFFFFFFFFFll) == 0) return v;
    if (E == 0 || E + k <= 0 || E + k >= 0x7FF) return v * pow2d(k);
    return __longlong_as_double(bits + ((long long)k << 52));
}

// rint(v 2^p) (round half to even) on the bit pattern of v, with integer
// operations only: the same integer as rounding the exactly scaled double,
// for |v 2^p| < 2^62 (no FP64-pipe multiply or conversion).
__device__ __forceinline__ long long oz_scaled_rint(double v, int p)
{
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const int E = (int)((bits >> 52) & 0x7FF);
    unsigned long long m = bits & 0xFFFFFFFFFFFFFull;
    if (E != 0) m |= 1ull << 52;
    if (m == 0) return 0;
    const int sh = (E == 0 ? 1 : E) - 1075 + p;   // |v| 2^p = m 2^sh
    unsigned long long u;
    if (sh >= 0) {
        u = m << sh;
    } else if (sh < -62) {
        u = 0;   // m 2^sh < 2^-9
    } else {
        const int r = -sh;
        const unsigned long long q = m >> r, rem = m & ((1ull << r) - 1), half = 1ull << (r - 1);
        u = q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
    }
    return (bits >> 63) ? -(long long)u : (long long)u;
}

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

// byte offset of the 16-byte chunk holding k = 8 g .. 8 g + 7 of row r in a
// 128-byte-swizzled K-major tile (chunk index XOR row mod 8)
__device__ __forceinline__ uint32_t oz_swz(int r, int g)
{
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((g ^ (r & 7)) << 4));
}

__device__ __forceinline__ uint4 oz_pack8(const float d[8])
{
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        __nv_bfloat162 p = __floats2bfloat162_rn(d[2 * j], d[2 * j + 1]);   // low half: element 2 j
        w[j] = *reinterpret_cast<uint32_t *>(&p);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// A digits.  Thread: row i, 8 consecutive k.  A is Hermitian: A_ik = conj(A_ki)
// is read down column i (coalesced).  U = rint(A_ik 2^(8 SA - 1 - e_i))
// (|U| <= 2^(8 SA - 1), one rounding at 2^-(8 SA) of 2^(e_i+1)) is cut into SA
// digits; U is formed from the bits of A_ik with integer operations, since
// GB300's FP64 pipe would bound this kernel otherwise.  Layout: blocks [b][i / 128][k / 64][s] of 32 KB = [Ar_s | Ai_s],
// 128 rows each.
template <int SA>
__global__ void k_oz_digits_a(const double2 *A, int n, int np, const int *ex, unsigned char *D, int batch)
{
    const int kg8 = np / 8;
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= (long)batch * np * kg8) return;
    const int b = (int)(t / ((long)np * kg8));
    const long e = t - (long)b * np * kg8;
    const int i = (int)(e / kg8), kq = (int)(e % kg8), k0 = 8 * kq;
    const int p = 8 * SA - 1 - ex[(long)b * np + i];
    float dr[SA][8], di[SA][8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        const int k = k0 + u;
        double2 v = make_double2(0.0, 0.0);
        if (i < n && k < n) {
            v = A[(long)b * n * n + k + (long)i * n];
            v.y = -v.y;
        }
        float xr[SA], xi[SA];
        digits_of<SA>(oz_scaled_rint(v.x, p), xr);
        digits_of<SA>(oz_scaled_rint(v.y, p), xi);
#pragma unroll
        for (int q = 0; q < SA; ++q) { dr[q][u] = xr[q]; di[q][u] = xi[q]; }
    }
    const int KC = np / OZ_BK;
    unsigned char *blk = D + ((((long)b * (np / OZ_MA) + i / OZ_MA) * KC + k0 / OZ_BK) * SA) * OZ_ABLK;
    const uint32_t off = oz_swz(i % OZ_MA, (k0 % OZ_BK) / 8);
#pragma unroll
    for (int q = 0; q < SA; ++q) {
        *(uint4 *)(blk + (long)q * OZ_ABLK + off) = oz_pack8(dr[q]);
        *(uint4 *)(blk + (long)q * OZ_ABLK + OZ_MA * 128 + off) = oz_pack8(di[q]);
    }
}

// X digits.  Thread: column j, 8 consecutive k (X column-major FP32).
// U = rint(X_kj 2^(23 - f_j)) (|U| <= 2^23) is cut into 3 digits and X itself
// is overwritten with U 2^(f_j - 23), the value its digits represent (exact in
// FP32).  Layout: blocks [b][j / 64][k / 64][t] of 24 KB = [-Xi_t | Xr_t | Xi_t],
// 64 rows each (negated digits are exact integers of the same range).
__global__ void k_oz_digits_x(float2 *X, int n, int np, const int *ex, unsigned char *D, int batch)
{
    const int kg8 = np / 8;
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= (long)batch * np * kg8) return;
    const int b = (int)(t / ((long)np * kg8));
    const long e = t - (long)b * np * kg8;
    const int j = (int)(e / kg8), kq = (int)(e % kg8), k0 = 8 * kq;
    const int fj = ex[(long)b * np + j];
    float dr[OZ_SB][8], di[OZ_SB][8], dn[OZ_SB][8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        const int k = k0 + u;
        const bool in = j < n && k < n;
        const long xi = (long)b * n * n + k + (long)j * n;
        float2 v = make_float2(0.f, 0.f);
        if (in) v = X[xi];
        const int ur = __float2int_rn(v.x * pow2f(23 - fj)), ui = __float2int_rn(v.y * pow2f(23 - fj));
        float xr[OZ_SB], xm[OZ_SB];
        digits_of<OZ_SB>(ur, xr);
        digits_of<OZ_SB>(ui, xm);
#pragma unroll
        for (int q = 0; q < OZ_SB; ++q) { dr[q][u] = xr[q]; di[q][u] = xm[q]; dn[q][u] = -xm[q]; }
        if (in) X[xi] = make_float2((float)ur * pow2f(fj - 23), (float)ui * pow2f(fj - 23));
    }
    const int KC = np / OZ_BK;
    unsigned char *blk = D + ((((long)b * (np / OZ_NX) + j / OZ_NX) * KC + k0 / OZ_BK) * OZ_SB) * OZ_XBLK;
    const uint32_t off = oz_swz(j % OZ_NX, (k0 % OZ_BK) / 8);
#pragma unroll
    for (int q = 0; q < OZ_SB; ++q) {
        unsigned char *bq = blk + (long)q * OZ_XBLK;
        *(uint4 *)(bq + off) = oz_pack8(dn[q]);
        *(uint4 *)(bq + OZ_NX * 128 + off) = oz_pack8(dr[q]);
        *(uint4 *)(bq + 2 * OZ_NX * 128 + off) = oz_pack8(di[q]);
    }
}

// ---------------------------------------------------------------------------
// tcgen05 / barrier helpers
__device__ __forceinline__ uint32_t oz_saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 B apart, descriptor version 1 (bits 46-48)
__device__ __forceinline__ uint64_t oz_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

__device__ __forceinline__ void oz_mma(uint32_t tmem, uint64_t da, uint64_t db, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                 :: "r"(tmem), "l"(da), "l"(db), "r"(OZ_IDESC), "r"(acc));
}

__device__ __forceinline__ void oz_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar)
                 : "memory");
}

// one bounded hardware wait (the thread is suspended until the phase completes
// or about a microsecond passes)
__device__ __forceinline__ bool oz_try(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}\n"
                 : "=r"(ok) : "r"(bar), "r"(parity), "r"(1000u) : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long oz_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// wait for the phase of the given parity, at most OZ_WAIT_NS or until another
// role has given up (abort flag)
__device__ __forceinline__ bool oz_wait(uint32_t bar, uint32_t parity, volatile int *abort)
{
    if (oz_try(bar, parity)) return true;
    const unsigned long long t0 = oz_ns();
    for (;;) {
        if (oz_try(bar, parity)) return true;
        if (*abort || oz_ns() - t0 > OZ_WAIT_NS) return false;
    }
}

__device__ __forceinline__ void oz_expect(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void oz_bulk(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

// hint: bring a block of global memory into L2 ahead of its bulk copy
__device__ __forceinline__ void oz_prefetch_l2(const void *src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ void oz_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
}

__device__ __forceinline__ void oz_ld4(uint32_t taddr, float v[4])
{
    uint32_t r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}

// (hi, lo) += v, v exact in FP64's sense once scaled by a power of two
__device__ __forceinline__ void df_add(float &hi, float &lo, float v)
{
    const float s = hi + v, bb = s - hi;
    lo += (hi - (s - bb)) + (v - bb);
    hi = s;
}

// Persistent: each CTA takes tiles t = blockIdx.x, blockIdx.x + gridDim.x, ...,
// a tile being rows i0..i0+127 of Y (A rows) x columns j0..j0+63 (X columns)
// of one matrix (see the file header).  The barrier phases run on across
// tiles, so the producer and the MMA thread start the next tile while the fold
// warps write the previous one out.
// 18 warps: at most 5 per SM sub-partition, whose 16K registers allow 96
// registers a thread
template <int SA>
__global__ void __maxnreg__(96)
k_oz_gemm(const unsigned char *DA, const unsigned char *DX, const int *exA, const int *exX, double2 *Y, int n,
          int np, int batch, unsigned *fault)
{
    extern __shared__ __align__(16) unsigned char oz_raw[];
    const int KC = np / OZ_BK, NJ = np / OZ_NX, NI = np / OZ_MA;
    const int ntiles = NJ * NI * batch;
    const uint32_t raw_s = oz_saddr(oz_raw);
    unsigned char *base = oz_raw + (((raw_s + 1023u) & ~1023u) - raw_s);
    unsigned char *sX = base;                                   // OZ_NXS x 72 KB
    unsigned char *sA = base + OZ_NXS * OZ_XSTAGE;              // OZ_NAS x 32 KB
    uint64_t *bars = (uint64_t *)(sA + OZ_NAS * OZ_ABLK);
    uint32_t *tslot = (uint32_t *)(bars + OZ_NBAR);
    volatile int *abort = (volatile int *)(tslot + 1);
    const uint32_t bar0 = oz_saddr(bars);
    // barrier addresses: X full/empty, A full/empty, level full/empty
    auto full_x = [&](int q) { return bar0 + 8u * q; };
    auto empty_x = [&](int q) { return bar0 + 8u * (OZ_NXS + q); };
    auto full_a = [&](int q) { return bar0 + 8u * (2 * OZ_NXS + q); };
    auto empty_a = [&](int q) { return bar0 + 8u * (2 * OZ_NXS + OZ_NAS + q); };
    auto tfull = [&](int q) { return bar0 + 8u * (2 * OZ_NXS + 2 * OZ_NAS + q); };
    auto tempty = [&](int q) { return bar0 + 8u * (2 * OZ_NXS + 2 * OZ_NAS + OZ_NBUF + q); };
    // a tile's digit blocks: X chunks of its 64 columns, A planes of its 128 rows
    auto tile_x = [&](int t) {
        const int jt = t % NJ, b = t / (NJ * NI);
        return DX + (((long)b * NJ + jt) * KC) * OZ_SB * OZ_XBLK;
    };
    auto tile_a = [&](int t) {
        const int it = (t / NJ) % NI, b = t / (NJ * NI);
        return DA + (((long)b * NI + it) * KC) * SA * OZ_ABLK;
    };

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(oz_saddr(tslot)), "r"(OZ_TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int q = 0; q < OZ_NBAR; ++q) {
            const bool fold = q >= 2 * OZ_NXS + 2 * OZ_NAS + OZ_NBUF;   // level-empty: one arrive per fold warp
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar0 + 8u * q),
                         "r"(fold ? OZ_FOLD_WARPS : 1) : "memory");
        }
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    // digit levels L = s + t kept per chunk: L <= 5 of 6 x 3 digits, all of 3 x 3
    constexpr int NL = SA == 6 ? 6 : SA + OZ_SB - 1;
    const int QA = KC * SA;   // A planes per tile

    if (warp == OZ_FOLD_WARPS) {
        // ---- producer: bulk copies of the pre-swizzled digit tiles ----
        if (lane == 0) {
            bool ok = true;
            // the A ring holds two planes: later planes (of this tile or the next)
            // are brought into L2 ahead of their copies, and so is the next chunk's X
            if (blockIdx.x < ntiles)
                for (int qa = OZ_NAS; qa < min(OZ_APF, QA); ++qa)
                    oz_prefetch_l2(tile_a(blockIdx.x) + (long)qa * OZ_ABLK, OZ_ABLK);
            int ti = 0;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++ti) {
                const int tn = t + gridDim.x;   // the next tile, if any
                const unsigned char *gX = tile_x(t), *gA = tile_a(t);
                for (int kc = 0; kc < KC && ok; ++kc) {
                    const int g = ti * KC + kc, jx = g % OZ_NXS, ux = g / OZ_NXS;
                    if (ux > 0 && !(ok = oz_wait(empty_x(jx), (ux - 1) & 1, abort))) break;
                    oz_expect(full_x(jx), OZ_XSTAGE);
                    for (int q = 0; q < OZ_SB; ++q)
                        oz_bulk(oz_saddr(sX + jx * OZ_XSTAGE + q * OZ_XBLK), gX + ((long)kc * OZ_SB + q) * OZ_XBLK,
                                OZ_XBLK, full_x(jx));
                    const unsigned char *pX = kc + 1 < KC ? gX + (long)(kc + 1) * OZ_XSTAGE
                                                          : (tn < ntiles ? tile_x(tn) : nullptr);
                    if (pX)
                        for (int q = 0; q < OZ_SB; ++q) oz_prefetch_l2(pX + (long)q * OZ_XBLK, OZ_XBLK);
                    for (int sdig = 0; sdig < SA; ++sdig) {
                        const int qa = kc * SA + sdig, qg = ti * QA + qa, ia = qg % OZ_NAS, ua = qg / OZ_NAS;
                        if (qa + OZ_APF < QA) oz_prefetch_l2(gA + (long)(qa + OZ_APF) * OZ_ABLK, OZ_ABLK);
                        else if (tn < ntiles && qa + OZ_APF - QA < QA)
                            oz_prefetch_l2(tile_a(tn) + (long)(qa + OZ_APF - QA) * OZ_ABLK, OZ_ABLK);
                        if (ua > 0 && !(ok = oz_wait(empty_a(ia), (ua - 1) & 1, abort))) break;
                        oz_expect(full_a(ia), OZ_ABLK);
                        oz_bulk(oz_saddr(sA + ia * OZ_ABLK), gA + (long)qa * OZ_ABLK, OZ_ABLK, full_a(ia));
                    }
                }
            }
            if (!ok) { *abort = 1; atomicOr(fault ? fault : &g_oz_fault, 1u); }
        }
    } else if (warp == OZ_FOLD_WARPS + 1) {
        // ---- MMA issue: plane s takes the digit pairs (s, 0), (s, 1), (s, 2) ----
        if (lane == 0) {
            bool ok = true;
            const uint32_t sx0 = oz_saddr(sX), sa0 = oz_saddr(sA);
            int g = 0;   // chunks issued by this CTA, over all its tiles
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                for (int kc = 0; kc < KC && ok; ++kc, ++g) {
                    const int jx = g % OZ_NXS, ux = g / OZ_NXS;
                    if (!(ok = oz_wait(full_x(jx), ux & 1, abort))) break;
                    for (int sdig = 0; sdig < SA; ++sdig) {
                        const int qg = g * SA + sdig, ia = qg % OZ_NAS, ua = qg / OZ_NAS;
                        if (!(ok = oz_wait(full_a(ia), ua & 1, abort))) break;
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const uint32_t ar = sa0 + ia * OZ_ABLK, ai = ar + OZ_MA * 128;
                        for (int tdig = 0; tdig < OZ_SB; ++tdig) {
                            const int L = sdig + tdig;
                            if (L > NL - 1) break;
                            const int ql = g * NL + L, buf = ql % OZ_NBUF;
                            const bool first = sdig == (L > 2 ? L - 2 : 0);
                            if (first && ql >= OZ_NBUF) {
                                // the fold of level ql - OZ_NBUF has emptied this buffer
                                if (!(ok = oz_wait(tempty(buf), ((ql - OZ_NBUF) / OZ_NBUF) & 1, abort))) break;
                                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                            }
                            // X block rows: [-Xi | Xr | Xi]; w1 = [Xr | Xi], w2 = [-Xi | Xr]
                            const uint32_t w2 = sx0 + jx * OZ_XSTAGE + tdig * OZ_XBLK, w1 = w2 + OZ_NX * 128;
                            const uint32_t tl = tmem + 128u * buf;
                            // a 16-deep step is 32 bytes along the swizzled row: 2 in the
                            // descriptor's address field (which no step carries out of)
                            const uint64_t dar = oz_desc(ar), dai = oz_desc(ai), dw1 = oz_desc(w1), dw2 = oz_desc(w2);
                            oz_mma(tl, dar, dw1, first ? 0u : 1u);
                            oz_mma(tl, dai, dw2, 1u);
#pragma unroll
                            for (int ks = 1; ks < OZ_BK / 16; ++ks) {
                                oz_mma(tl, dar + 2 * ks, dw1 + 2 * ks, 1u);
                                oz_mma(tl, dai + 2 * ks, dw2 + 2 * ks, 1u);
                            }
                        }
                        if (!ok) break;
                        oz_commit(empty_a(ia));
                        // level sdig of this chunk is complete; after the last plane, all remaining ones
                        for (int L = sdig; L < (sdig == SA - 1 ? NL : sdig + 1); ++L)
                            oz_commit(tfull((g * NL + L) % OZ_NBUF));
                    }
                    if (!ok) break;
                    oz_commit(empty_x(jx));
                }
            }
            if (ok && g > 0) {
                // the last commit has landed: every MMA of the CTA has finished
                const int jx = (g - 1) % OZ_NXS, ux = (g - 1) / OZ_NXS;
                ok = oz_wait(empty_x(jx), ux & 1, abort);
            }
            if (!ok) { *abort = 1; atomicOr(fault ? fault : &g_oz_fault, 1u); }
        }
    } else {
        // ---- fold warps: level sums -> double-float accumulators -> Y ----
        const int q4 = warp & 3, h = warp >> 2;
        const uint32_t trow = tmem + ((uint32_t)(32 * q4) << 16);
        bool ok = true;
        int g = 0;   // chunks folded by this CTA, over all its tiles
        for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
            float hr[16], lr[16], hi[16], li[16];
#pragma unroll
            for (int c = 0; c < 16; ++c) hr[c] = lr[c] = hi[c] = li[c] = 0.f;
            for (int kc = 0; kc < KC && ok; ++kc, ++g) {
#pragma unroll 1
                for (int L = 0; L < NL; ++L) {
                    const int ql = g * NL + L, buf = ql % OZ_NBUF;
                    ok = __all_sync(0xffffffffu, oz_wait(tfull(buf), (ql / OZ_NBUF) & 1, abort));
                    if (!ok) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const float w = ldexpf(1.0f, -8 * (L + 2));
                    // four groups of 4 columns (fewer live registers); the buffer is
                    // released once all are in registers
#pragma unroll
                    for (int hf = 0; hf < 4; ++hf) {
                        float re[4], im[4];
                        const uint32_t c0 = trow + 128u * buf + 16u * h + 4u * hf;
                        oz_ld4(c0, re);           // Ar Xr - Ai Xi
                        oz_ld4(c0 + 64u, im);     // Ar Xi + Ai Xr
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                        if (hf == 3) {
                            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                            __syncwarp();
                            if (lane == 0) oz_arrive(tempty(buf));
                        }
                        if (L < 3) {
                            // levels 0-2: exact two-sum into (hi, lo)
#pragma unroll
                            for (int c = 0; c < 4; ++c) {
                                df_add(hr[4 * hf + c], lr[4 * hf + c], re[c] * w);
                                df_add(hi[4 * hf + c], li[4 * hf + c], im[c] * w);
                            }
                        } else {
                            // from level 3 on the contribution (< 2^-17 of the unit scale) goes
                            // straight into lo, whose own rounding already bounds the pair's error
#pragma unroll
                            for (int c = 0; c < 4; ++c) {
                                lr[4 * hf + c] = fmaf(re[c], w, lr[4 * hf + c]);
                                li[4 * hf + c] = fmaf(im[c], w, li[4 * hf + c]);
                            }
                        }
                    }
                }
            }
            if (!ok) break;
            // Y[i, j], i = this thread's A row, j = 16 consecutive X columns:
            // scale by 2^(e_i + 1) 2^(f_j + 1)
            const int jt = t % NJ, it = (t / NJ) % NI, b = t / (NJ * NI);
            const int i = it * OZ_MA + 32 * q4 + lane;
            if (i < n) {
                const int ei = exA[(long)b * np + i];
                double2 *yb = Y + (long)b * n * n + i;
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    const int j = jt * OZ_NX + 16 * h + c;
                    if (j >= n) break;
                    // widening and the power-of-two scale with integer operations:
                    // only the double-float sum takes the FP64 pipe
                    const int k2 = ei + exX[(long)b * np + j] + 2;
                    yb[(long)j * n] = make_double2(oz_scale2(f2d_exact(hr[c]) + f2d_exact(lr[c]), k2),
                                                   oz_scale2(f2d_exact(hi[c]) + f2d_exact(li[c]), k2));
                }
            }
        }
        if (!ok && lane == 0) { *abort = 1; atomicOr(fault ? fault : &g_oz_fault, 1u); }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(OZ_TMEM_COLS)
                     : "memory");
    }
}

// SMs of the current device (cached per device)
static int oz_device_sms()
{
    static std::mutex m;
    static std::map<int, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(m);
    auto f = cache.find(dev);
    if (f != cache.end()) return f->second;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return cache[dev] = sms > 0 ? sms : 1;
}

OzakiX ozaki_prepare_x(cudaStream_t s, float2 *X, int n, int batch, void *work)
{
    OzakiX ox;
    const int np = padn(n);
    const size_t npp = (size_t)np * np;
    char *w = (char *)work;
    ox.DA = (__nv_bfloat16 *)w;
    ox.DX = (__nv_bfloat16 *)(w + al256(sizeof(__nv_bfloat16) * npp * batch * 2 * OZ_SA));
    ox.exA = (int *)((char *)ox.DX + al256(sizeof(__nv_bfloat16) * npp * batch * 3 * OZ_SB));
    ox.exX = (int *)((char *)ox.exA + al256(sizeof(int) * (size_t)np * batch));
    ox.n = n; ox.np = np; ox.batch = batch;
    NRLTB_LAUNCH(k_oz_colexp<float2>, cdiv((long)np * batch * 32, 256), 256, 0, s, X, n, np, ox.exX, batch);
    NRLTB_LAUNCH(k_oz_digits_x, cdiv((long)npp / 8 * batch, 256), 256, 0, s, X, n, np, ox.exX,
                 (unsigned char *)ox.DX, batch);
    return ox;
}

// digits and row exponents of A into D, ex
template <int SA> static void ozaki_digits_a(cudaStream_t s, const double2 *A, int n, int np, int batch, int *ex,
                                             unsigned char *D)
{
    const size_t npp = (size_t)np * np;
    NRLTB_LAUNCH(k_oz_colexp<double2>, cdiv((long)np * batch * 32, 256), 256, 0, s, A, n, np, ex, batch);
    NRLTB_LAUNCH(k_oz_digits_a<SA>, cdiv((long)npp / 8 * batch, 256), 256, 0, s, A, n, np, ex, D, batch);
}

template <int SA> static void ozaki_product(cudaStream_t s, const OzakiX &ox, const unsigned char *DA, const int *exA,
                                            double2 *Y)
{
    const int n = ox.n, np = ox.np, batch = ox.batch;
    static const bool attr = [] {
        cudaFuncSetAttribute(k_oz_gemm<SA>, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM);
        return true;
    }();
    (void)attr;
    // one CTA per SM (its shared and tensor memory allow no second), each
    // looping over tiles
    const long ntiles = (long)(np / OZ_NX) * (np / OZ_MA) * batch;
    if (ntiles <= 0) return;
    const int grid = (int)std::min<long>(ntiles, oz_device_sms());
    cudaEvent_t ev = kt_begin(s);
    NRLTB_LAUNCH(k_oz_gemm<SA>, grid, OZ_THREADS, OZ_SMEM, s, DA, (const unsigned char *)ox.DX, exA, ox.exX, Y, n,
                 np, batch, g_fault_word);
    kt_end(ev, s, KC_DIGIT_GEMM, 8.0 * n * (double)n * n * batch);
}

void ozaki_gemm(cudaStream_t s, const OzakiX &ox, const double2 *A, double2 *Y, int adigits)
{
    if (adigits == 3) {
        ozaki_digits_a<3>(s, A, ox.n, ox.np, ox.batch, ox.exA, (unsigned char *)ox.DA);
        ozaki_product<3>(s, ox, (const unsigned char *)ox.DA, ox.exA, Y);
    } else {
        ozaki_digits_a<6>(s, A, ox.n, ox.np, ox.batch, ox.exA, (unsigned char *)ox.DA);
        ozaki_product<6>(s, ox, (const unsigned char *)ox.DA, ox.exA, Y);
    }
}

size_t ozaki_a_bytes(int n, int batch, int adigits)
{
    const size_t np = (size_t)padn(n), nb = (size_t)batch;
    return al256(sizeof(__nv_bfloat16) * np * np * nb * 2 * (adigits == 3 ? 3 : OZ_SA)) +
           al256(sizeof(int) * np * nb) + 256;
}

OzakiA ozaki_prepare_a(cudaStream_t s, const double2 *A, int n, int batch, int adigits, void *work)
{
    const int np = padn(n), sa = adigits == 3 ? 3 : OZ_SA;
    unsigned char *D = (unsigned char *)work;
    int *ex = (int *)(D + al256(sizeof(__nv_bfloat16) * (size_t)np * np * batch * 2 * sa));
    if (sa == 3) ozaki_digits_a<3>(s, A, n, np, batch, ex, D);
    else ozaki_digits_a<6>(s, A, n, np, batch, ex, D);
    OzakiA oa;
    oa.D = D;
    oa.ex = ex;
    oa.sa = sa;
    return oa;
}

void ozaki_gemm_prepared(cudaStream_t s, const OzakiX &ox, const OzakiA &oa, double2 *Y)
{
    if (oa.sa == 3) ozaki_product<3>(s, ox, oa.D, oa.ex, Y);
    else ozaki_product<6>(s, ox, oa.D, oa.ex, Y);
}

unsigned ozaki_fault(bool clear)
{
    unsigned v = 0;
    cudaMemcpyFromSymbol(&v, g_oz_fault, sizeof(v));
    if (clear) {
        const unsigned z = 0;
        cudaMemcpyToSymbol(g_oz_fault, &z, sizeof(z));
    }
    return v;
}

}  // namespace nrltb
