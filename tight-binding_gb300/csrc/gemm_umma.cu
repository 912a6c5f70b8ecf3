// gemm_umma.cu -- batched complex FP32 GEMM on the 5th-generation tensor cores
// (tcgen05, TF32 operands from shared memory, FP32 accumulators in tensor
// memory), for the forms C = alpha A op(B) + beta C with op(B) = B or B^H (the
// eigensolver's large products and its rank-32/64 panel updates).
//
// 3xTF32: each FP32 operand x is split into a TF32 head h = tf32(x) and tail
// l = tf32(x - h); a real product is l_a h_b + h_a l_b + h_a h_b (the dropped
// l_a l_b is 2^-22 relative).  Complex: the B tile is staged as the row
// blocks [Br | Bi] (64 columns each), and two M = 128, N = 128 accumulators in
// tensor memory take P = Ar [Br | Bi] and Q = Ai [Br | Bi]; the epilogue forms
// Re = P[:, j] - Q[:, 64 + j], Im = P[:, 64 + j] + Q[:, j] for a 128 x 64
// complex output tile.  Six MMAs per 8-deep k step.
//
// CTA: 256 threads, two CTAs per SM (96 KB stage each, 256 tensor-memory
// columns each); all threads stage operands (global -> registers -> head/tail
// split -> 128-byte-swizzled K-major shared-memory tiles), thread 0 issues the
// MMAs and commits them to a shared-memory barrier; the next 32-deep slice's
// global loads are in flight while the tensor cores work, and the other CTA
// on the SM fills the tensor pipe while this one stages or stores.
// Epilogue: each warp reads 32 rows x 32 complex columns of tensor memory.
// Every barrier wait is bounded (about two seconds); on expiry the kernel
// records a fault flag and leaves without touching C.
#include <cstdint>
#include "common.cuh"
#include "gemm.cuh"

namespace nrltb {

namespace {
constexpr int UM_BM = 128, UM_BN = 64, UM_BK = 32;
constexpr int UM_THREADS = 256;
constexpr int UM_APL = UM_BM * 128;          // one A plane: 128 rows x 32 TF32 (128 B)
constexpr int UM_BPL = 2 * UM_BN * 128;      // one B plane: rows Br | Bi
constexpr int UM_STAGE = 4 * UM_APL + 2 * UM_BPL;   // A: re h, re l, im h, im l; B: h, l
constexpr int UM_SMEM = UM_STAGE + 1024 + 64;        // one stage, alignment slack, barrier
constexpr uint32_t UM_TMEM_COLS = 256;               // P | Q
constexpr unsigned long long UM_WAIT_NS = 2000000000ull;

// instruction descriptor, kind::tf32: D f32 (bits 4-5 = 1), A and B tf32
// (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28
constexpr uint32_t UM_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(128 >> 3) << 17) |
                              ((uint32_t)(UM_BM >> 4) << 24);
}  // namespace

__device__ unsigned g_umma_fault;

__device__ __forceinline__ uint32_t um_smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 B apart (stride byte offset), descriptor version 1 (bits 46-48)
__device__ __forceinline__ uint64_t um_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;                 // leading byte offset (unused for this layout)
    d |= (uint64_t)(1024 >> 4) << 32;       // stride byte offset
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;                 // 128-byte swizzle
    return d;
}

__device__ __forceinline__ void um_mma(uint32_t tmem, uint64_t da, uint64_t db, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n"
                 :: "r"(tmem), "l"(da), "l"(db), "r"(UM_IDESC), "r"(acc));
}

// one bounded hardware wait (the thread is suspended until the phase completes
// or about a microsecond passes)
__device__ __forceinline__ bool um_test(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}\n"
                 : "=r"(ok) : "r"(bar), "r"(parity), "r"(1000u) : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long um_clock_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// wait for the phase of the given parity to complete, at most UM_WAIT_NS
__device__ bool um_wait(uint32_t bar, uint32_t parity)
{
    if (um_test(bar, parity)) return true;
    const unsigned long long t0 = um_clock_ns();
    for (;;) {
        if (um_test(bar, parity)) return true;
        if (um_clock_ns() - t0 > UM_WAIT_NS) return false;
    }
}

__device__ __forceinline__ void um_ld16(uint32_t taddr, float v[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t um_tf32(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// byte offset of the 16-byte chunk holding k = 4 g .. 4 g + 3 of row r in a
// 128-byte-swizzled K-major tile (chunk index XOR row mod 8)
__device__ __forceinline__ uint32_t um_swz(int r, int g)
{
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((g ^ (r & 7)) << 4));
}

// heads and tails of four values into two planes
__device__ __forceinline__ void um_put4(unsigned char *ph, unsigned char *pl, uint32_t off, const float x[4])
{
    uint4 h, l;
    uint32_t hh[4], ll[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        hh[j] = um_tf32(x[j]);
        ll[j] = um_tf32(x[j] - __uint_as_float(hh[j]));
    }
    h = make_uint4(hh[0], hh[1], hh[2], hh[3]);
    l = make_uint4(ll[0], ll[1], ll[2], ll[3]);
    *(uint4 *)(ph + off) = h;
    *(uint4 *)(pl + off) = l;
}

template <int TB>   // 1: op(B) = B^H
__global__ void __launch_bounds__(UM_THREADS, 2) zgemm_umma_kernel(GemmArgs<float> g, int va, int vb, unsigned *fault)
{
    extern __shared__ __align__(16) unsigned char um_raw[];
    const int b = blockIdx.z;
    const int m0 = blockIdx.x * UM_BM, n0 = blockIdx.y * UM_BN;
    if (g.triC == 1 && m0 + UM_BM - 1 < n0) return;
    if (g.triC == 2 && n0 + UM_BN - 1 < m0) return;
    const float2 *A = g.A + b * g.sA;
    const float2 *B = g.B + b * g.sB;
    float2 *Cm = g.C + b * g.sC;
    int kbeg = 0, kend = g.k;
    if (g.triA == 1) kend = min(kend, m0 + UM_BM);
    if (g.triA == 2) kbeg = max(kbeg, m0);
    if (g.triB == 1) kend = min(kend, n0 + UM_BN);
    if (g.triB == 2) kbeg = max(kbeg, n0);
    kbeg = (kbeg / UM_BK) * UM_BK;
    const int nk = kend > kbeg ? (kend - kbeg + UM_BK - 1) / UM_BK : 0;

    // 1024-aligned tiles (the swizzle pattern follows address bits 4-9)
    const uint32_t raw_s = um_smem_addr(um_raw);
    unsigned char *base = um_raw + (((raw_s + 1023u) & ~1023u) - raw_s);
    uint64_t *bar = (uint64_t *)(base + UM_STAGE);
    uint32_t *tslot = (uint32_t *)(bar + 1);
    const uint32_t bar0 = um_smem_addr(bar);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(um_smem_addr(tslot)), "r"(UM_TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar0) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    // staging maps: A rows 2 ra_p and 2 ra_p + 1, k groups ra_g + 4u (a 16-byte
    // load takes both rows of one k when va and the chunk is interior); B
    // column rb_n, k groups rb_g + 4u (B: four consecutive k of a column are
    // contiguous, two 16-byte loads when vb and the chunk is interior; B^H: the
    // threads of a warp walk consecutive columns)
    const int ra_p = tid & 63, ra_g = tid >> 6, ra_s = (ra_p >> 2) & 1;
    const int rb_n = TB ? (tid & (UM_BN - 1)) : (tid >> 2), rb_g = TB ? (tid >> 6) : (tid & 3);
    float2 ra[16], rb[8];   // ra[8 u + 4 row + j]
    auto fetch = [&](int k0) {
        const int mA = m0 + 2 * ra_p;
        const bool ain = va && m0 + UM_BM <= g.m && k0 + UM_BK <= kend &&
                         (g.triA == 0 || (g.triA == 1 && k0 + UM_BK - 1 <= m0) ||
                          (g.triA == 2 && k0 >= m0 + UM_BM - 1));
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int k = k0 + 4 * (ra_g + 4 * u) + j;
                if (ain) {
                    const float4 v = *reinterpret_cast<const float4 *>(A + mA + (long)k * g.lda);
                    ra[8 * u + j] = make_float2(v.x, v.y);
                    ra[8 * u + 4 + j] = make_float2(v.z, v.w);
                } else {
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int m = mA + h;
                        bool ok = m < g.m && k < kend;
                        if (g.triA == 1) ok = ok && k <= m;
                        if (g.triA == 2) ok = ok && k >= m;
                        ra[8 * u + 4 * h + j] = ok ? A[m + (long)k * g.lda] : make_float2(0.f, 0.f);
                    }
                }
            }
        const int n = n0 + rb_n;
        const bool bin = !TB && vb && n0 + UM_BN <= g.n && k0 + UM_BK <= kend &&
                         (g.triB == 0 || (g.triB == 1 && k0 + UM_BK - 1 <= n0) ||
                          (g.triB == 2 && k0 >= n0 + UM_BN - 1));
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            if (bin) {
                const int k = k0 + 4 * (rb_g + 4 * u);
                const float4 *q = reinterpret_cast<const float4 *>(B + k + (long)n * g.ldb);
                const float4 v0 = q[0], v1 = q[1];
                rb[4 * u + 0] = make_float2(v0.x, v0.y);
                rb[4 * u + 1] = make_float2(v0.z, v0.w);
                rb[4 * u + 2] = make_float2(v1.x, v1.y);
                rb[4 * u + 3] = make_float2(v1.z, v1.w);
                continue;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int k = k0 + 4 * (rb_g + 4 * u) + j;
                bool ok = n < g.n && k < kend;
                if (g.triB == 1) ok = ok && k <= n;
                if (g.triB == 2) ok = ok && k >= n;
                float2 v = make_float2(0.f, 0.f);
                if (ok) {
                    if (TB) { v = B[n + (long)k * g.ldb]; v.y = -v.y; }
                    else v = B[k + (long)n * g.ldb];
                }
                rb[4 * u + j] = v;
            }
        }
    };
    auto store = [&](unsigned char *st) {
        // rows in the order 2 ra_p + ra_s, then the other: the eight row
        // residues mod 8 of each eight threads keep the swizzled stores
        // conflict-free
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const bool second = (hh ^ ra_s) != 0;
                const uint32_t off = um_swz(2 * ra_p + (second ? 1 : 0), ra_g + 4 * u);
                float re[4], im[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float2 v = second ? ra[8 * u + 4 + j] : ra[8 * u + j];   // register select
                    re[j] = v.x;
                    im[j] = v.y;
                }
                um_put4(st, st + UM_APL, off, re);
                um_put4(st + 2 * UM_APL, st + 3 * UM_APL, off, im);
            }
        unsigned char *bh = st + 4 * UM_APL, *bl = bh + UM_BPL;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int gk = rb_g + 4 * u;
            float re[4], im[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) { re[j] = rb[4 * u + j].x; im[j] = rb[4 * u + j].y; }
            um_put4(bh, bl, um_swz(rb_n, gk), re);
            um_put4(bh, bl, um_swz(UM_BN + rb_n, gk), im);
        }
    };

    bool fail = false;
    if (nk > 0) fetch(kbeg);
    for (int c = 0; c < nk; ++c) {
        if (c >= 1) {
            // the MMAs of chunk c - 1 have finished reading the stage
            int ok = 1;
            if (tid == 0) ok = um_wait(bar0, (c - 1) & 1);
            if (__syncthreads_or(!ok)) { fail = true; break; }
        }
        store(base);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (c + 1 < nk) fetch(kbeg + (c + 1) * UM_BK);
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = um_smem_addr(base);
            const uint32_t sb = sa + 4 * UM_APL;
            const uint32_t tp = tmem, tq = tmem + 128;
#pragma unroll
            for (int ks = 0; ks < UM_BK / 8; ++ks) {
                const uint32_t ko = 32u * ks;
                const uint64_t arh = um_desc(sa + ko), arl = um_desc(sa + UM_APL + ko);
                const uint64_t aih = um_desc(sa + 2 * UM_APL + ko), ail = um_desc(sa + 3 * UM_APL + ko);
                const uint64_t bh = um_desc(sb + ko), bl = um_desc(sb + UM_BPL + ko);
                const uint32_t acc = (c > 0 || ks > 0) ? 1u : 0u;
                um_mma(tp, arl, bh, acc);
                um_mma(tq, ail, bh, acc);
                um_mma(tp, arh, bl, 1u);
                um_mma(tq, aih, bl, 1u);
                um_mma(tp, arh, bh, 1u);
                um_mma(tq, aih, bh, 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(bar0) : "memory");
        }
    }
    if (!fail && nk > 0) {
        int ok = 1;
        if (tid == 0) ok = um_wait(bar0, (nk - 1) & 1);
        if (__syncthreads_or(!ok)) fail = true;
    }
    if (fail) {
        if (tid == 0) atomicOr(fault ? fault : &g_umma_fault, 1u);
        // give MMAs still in flight a second bounded wait before the memory is released
        if (tid == 0 && nk > 0) um_wait(bar0, (nk - 1) & 1);
    } else {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int q = warp & 3, h = warp >> 2;
        const int m = m0 + 32 * q + lane;
        const uint32_t trow = tmem + ((uint32_t)(32 * q) << 16);
        const bool beta0 = (g.beta.x == 0.f && g.beta.y == 0.f);
#pragma unroll 1
        for (int cc = 0; cc < 32; cc += 16) {
            float re[16], im[16];
            if (nk > 0) {
                // Re = P[:, j] - Q[:, 64 + j], Im = P[:, 64 + j] + Q[:, j]
                float t[16];
                const uint32_t col = (uint32_t)(32 * h + cc);
                um_ld16(trow + col, re);
                um_ld16(trow + 128 + UM_BN + col, t);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int j = 0; j < 16; ++j) re[j] -= t[j];
                um_ld16(trow + UM_BN + col, im);
                um_ld16(trow + 128 + col, t);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int j = 0; j < 16; ++j) im[j] += t[j];
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) re[j] = im[j] = 0.f;
            }
            if (m < g.m) {
                // the old C of all 16 columns first (their loads in flight together:
                // a load after a store to C could alias it and would wait for it)
                float2 cold[16];
                if (!beta0) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int n = n0 + 32 * h + cc + j;
                        cold[j] = (n < g.n) ? Cm[m + (long)n * g.ldc] : make_float2(0.f, 0.f);
                    }
                }
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int n = n0 + 32 * h + cc + j;
                    if (n >= g.n) break;
                    float2 *cp = Cm + m + (long)n * g.ldc;
                    float2 v = cmul(g.alpha, make_float2(re[j], im[j]));
                    if (!beta0) v = cadd(v, cmul(g.beta, cold[j]));
                    *cp = v;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(UM_TMEM_COLS)
                     : "memory");
    }
}

bool zgemm_umma_supported(const GemmArgs<float> &g)
{
    return g.opA == 0;
}

void zgemm_umma_launch(cudaStream_t s, const GemmArgs<float> &g)
{
    static const bool attr = [] {
        cudaFuncSetAttribute(zgemm_umma_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, UM_SMEM);
        cudaFuncSetAttribute(zgemm_umma_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, UM_SMEM);
        return true;
    }();
    (void)attr;
    dim3 grid(cdiv(g.m, UM_BM), cdiv(g.n, UM_BN), g.batch);
    // 16-byte loads need every element address of an even row (A) or even k (B)
    // 16-byte aligned: an aligned base, even leading dimension and batch stride
    const int va = ((uintptr_t)g.A % 16 == 0) && g.lda % 2 == 0 && g.sA % 2 == 0;
    const int vb = ((uintptr_t)g.B % 16 == 0) && g.ldb % 2 == 0 && g.sB % 2 == 0;
    if (g.opB) NRLTB_LAUNCH(zgemm_umma_kernel<1>, grid, UM_THREADS, UM_SMEM, s, g, va, vb, g_fault_word);
    else NRLTB_LAUNCH(zgemm_umma_kernel<0>, grid, UM_THREADS, UM_SMEM, s, g, va, vb, g_fault_word);
}

unsigned zgemm_umma_fault(bool clear)
{
    unsigned v = 0;
    cudaMemcpyFromSymbol(&v, g_umma_fault, sizeof(v));
    if (clear) {
        const unsigned z = 0;
        cudaMemcpyToSymbol(g_umma_fault, &z, sizeof(z));
    }
    return v;
}

}  // namespace nrltb
