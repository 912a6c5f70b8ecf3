// common.cuh -- shared helpers of the GB300 NRL tight-binding library:
// complex arithmetic on interleaved (re, im) pairs, launch accounting and
// error propagation into the context.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

namespace nrltb {

// ---- complex arithmetic on float2 / double2 --------------------------------
template <typename T> struct cplx;
template <> struct cplx<float> { typedef float2 t; };
template <> struct cplx<double> { typedef double2 t; };

__host__ __device__ __forceinline__ double2 mk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ float2 mk(float r, float i) { return make_float2(r, i); }
template <typename T> __host__ __device__ __forceinline__ typename cplx<T>::t cmk(T r, T i) { return mk(r, i); }

template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b)
{
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
// conj(a) * b
template <typename C> __host__ __device__ __forceinline__ C cmulc(C a, C b)
{
    C r;
    r.x = a.x * b.x + a.y * b.y;
    r.y = a.x * b.y - a.y * b.x;
    return r;
}
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }
template <typename C, typename T> __host__ __device__ __forceinline__ C cscale(C a, T s) { a.x *= s; a.y *= s; return a; }
// acc += a * b (complex FMA in four real FMAs)
template <typename C> __device__ __forceinline__ void cfma(C &acc, C a, C b)
{
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
template <typename C> __device__ __forceinline__ void cfmac(C &acc, C a, C b)
{
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(-a.y, b.x, acc.y);
}

// FP32 -> FP64 (exact) from the bit pattern with integer operations: the same
// value as the hardware conversion, which GB300 runs on its narrow FP64 pipe.
__device__ __forceinline__ double f2d_exact(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    const unsigned E = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
    unsigned long long bits;
    if (E == 0) {
        if (m == 0) return __longlong_as_double((long long)sign);
        const int p = 31 - __clz(m);   // subnormal: m 2^-149 = 1.f 2^(p - 149)
        bits = ((unsigned long long)(p + 874) << 52) | (((unsigned long long)m << (52 - p)) & 0xFFFFFFFFFFFFFull);
    } else if (E == 0xFFu) {
        bits = (0x7FFull << 52) | ((unsigned long long)m << 29);
    } else {
        bits = ((unsigned long long)(E + 896) << 52) | ((unsigned long long)m << 29);
    }
    return __longlong_as_double((long long)(bits | sign));
}

// FP64 -> FP32 rounded to nearest even, from the bit pattern with integer
// operations: the same value as the hardware conversion (overflow to
// infinity, subnormal results, NaN kept a NaN).
__device__ __forceinline__ float d2f_rn(double x)
{
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(bits >> 63) << 31;
    const int E = (int)((bits >> 52) & 0x7FF);
    const unsigned long long m = bits & 0xFFFFFFFFFFFFFull;
    unsigned f;
    if (E == 0x7FF) {
        f = m ? (0x7FC00000u | (unsigned)(m >> 29)) : 0x7F800000u;
    } else if (E == 0) {
        f = 0;   // below 2^-1022: rounds to zero
    } else {
        const int e = E - 1023;
        if (e > 127) {
            f = 0x7F800000u;
        } else if (e >= -126) {
            f = ((unsigned)(e + 127) << 23) | (unsigned)(m >> 29);
            const unsigned long long rem = m & ((1ull << 29) - 1), half = 1ull << 28;
            if (rem > half || (rem == half && (f & 1u))) f += 1;   // a carry moves into the exponent
        } else {
            const unsigned long long M = m | (1ull << 52);
            const int s = -(e + 97);   // subnormal result: M 2^-s units of 2^-149, s > 29
            if (s > 60) {
                f = 0;
            } else {
                const unsigned long long k = M >> s, rem = M & ((1ull << s) - 1), half = 1ull << (s - 1);
                f = (unsigned)k;
                if (rem > half || (rem == half && (k & 1ull))) f += 1;
            }
        }
    }
    return __uint_as_float(f | sign);
}

// order-preserving 64-bit key of a double (not NaN; -0 and +0 share the key
// of 0): key(u) < key(v) exactly when u < v
__device__ __forceinline__ unsigned long long ord_key(double v)
{
    const long long bits = v == 0.0 ? 0ll : __double_as_longlong(v);
    return bits >= 0 ? (unsigned long long)bits ^ 0x8000000000000000ull : ~(unsigned long long)bits;
}

// Rank of L[j] among L[0..n) (ties by index): the number of q with L[q] < L[j]
// or L[q] == L[j] and q < j.  With `keys` (shared memory of n keys, filled
// here by the whole CTA, which must all call this) the comparisons are
// integer ones on order-preserving keys; the same ranks either way.
__device__ __forceinline__ int rank_of(const double *L, int n, int j, unsigned long long *keys)
{
    if (keys) {
        for (int q = threadIdx.x; q < n; q += blockDim.x) keys[q] = ord_key(L[q]);
        __syncthreads();
        if (j >= n) return 0;
        const unsigned long long kv = keys[j];
        int r = 0;
        for (int q = 0; q < n; ++q) {
            const unsigned long long ku = keys[q];
            r += (ku < kv) || (ku == kv && q < j);
        }
        return r;
    }
    if (j >= n) return 0;
    const double v = L[j];
    int r = 0;
    for (int q = 0; q < n; ++q) {
        const double u = L[q];
        r += (u < v) || (u == v && q < j);
    }
    return r;
}
// shared memory for rank_of's keys (0: compare in FP64 from global memory)
inline size_t rank_keys_bytes(int n)
{
    const size_t b = sizeof(unsigned long long) * (size_t)n;
    return b <= 160 * 1024 ? b : 0;
}

template <typename T> __device__ __forceinline__ T warp_sum(T v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of one value; every thread gets the result.  `sh` needs
// blockDim.x / 32 entries.
template <typename T> __device__ __forceinline__ T block_sum(T v, T *sh)
{
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    T t = (threadIdx.x < nw) ? sh[threadIdx.x] : T(0);
    if (wid == 0) t = warp_sum(t);
    if (threadIdx.x == 0) sh[0] = t;
    __syncthreads();
    T r = sh[0];
    __syncthreads();
    return r;
}

__host__ __device__ inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

// Launch accounting: every kernel launch of the library goes through LAUNCH so
// that the context can report how many device kernels a call issued.
extern thread_local long long *g_launch_counter;

// Bounded-wait expiry: the tcgen05 kernels OR 1 into this device word when a
// barrier wait runs out (null: a per-library global flag, read by the test
// hooks).  A context points it at its own word for the duration of a call, so
// concurrent contexts never see each other's faults.
extern thread_local unsigned *g_fault_word;

// Kernel-class timing (off unless a context enables it): CUDA events on the
// launching stream around each launch of a timed class, with the launch's
// algorithmic work (flops or bytes), summed by nrltb_bench_kernel_stats.
enum KClass { KC_GEMM_TC = 0, KC_GEMM_SIMT = 1, KC_DIGIT_GEMM = 2, KC_TRI_PANEL = 3, KC_COUNT = 4 };
// Raise a kernel's dynamic shared-memory limit on the current device to at
// least `bytes`, never lowering it: host threads that launch the same kernel
// with different sizes (the structure batch) must not lower the limit between
// another thread's setting and its launch.  Returns the CUDA status.
inline cudaError_t smem_attr_at_least(const void *func, int bytes)
{
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, int> set;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(mu);
    int &cur = set[std::make_pair(dev, func)];
    if (bytes <= cur) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

struct KTimer {
    bool on = false;
    struct Rec { int cls; cudaEvent_t a, b; double work; };
    std::vector<Rec> recs;          // every timed launch since timing was turned on
    std::vector<cudaEvent_t> pool;  // events, reused from one timing period to the next
    size_t used = 0;
    cudaEvent_t next()
    {
        if (used == pool.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
            pool.push_back(e);
        }
        return pool[used++];
    }
};
extern thread_local KTimer *g_ktimer;
// record the start of a timed launch; returns the event or null (timing off)
inline cudaEvent_t kt_begin(cudaStream_t s)
{
    KTimer *k = g_ktimer;
    if (!k || !k->on) return nullptr;
    cudaEvent_t e = k->next();
    if (e) cudaEventRecord(e, s);
    return e;
}
inline void kt_end(cudaEvent_t a, cudaStream_t s, int cls, double work)
{
    KTimer *k = g_ktimer;
    if (!a || !k) return;
    cudaEvent_t b = k->next();
    if (!b) return;
    cudaEventRecord(b, s);
    k->recs.push_back({cls, a, b, work});
}
#define NRLTB_LAUNCH(kernel, grid, block, smem, stream, ...)                 \
    do {                                                                     \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);          \
        if (::nrltb::g_launch_counter) ++*::nrltb::g_launch_counter;         \
    } while (0)

}  // namespace nrltb
