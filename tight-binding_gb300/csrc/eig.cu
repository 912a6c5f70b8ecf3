// eig.cu -- batched generalized Hermitian eigensolver (see eig.cuh for the plan).
#include <algorithm>
#include <cfloat>
#include "eig.cuh"
#include "tri_panel.cuh"

namespace nrltb {

template <typename T> __host__ __device__ inline T eps_of();
template <> __host__ __device__ inline float eps_of<float>() { return FLT_EPSILON * 0.5f; }
template <> __host__ __device__ inline double eps_of<double>() { return DBL_EPSILON * 0.5; }

static inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

template <typename T> size_t eig_work_bytes(int n, int batch)
{
    EigWork<T> w;
    eig_work_carve<T>(w, nullptr, n, batch);
    return (size_t)w.status + sizeof(int) * (size_t)batch;  // carve from 0 gives the size
}

template <typename T> void eig_work_carve(EigWork<T> &w, void *base, int n, int batch)
{
    typedef typename cplx<T>::t C2;
    size_t off = 0;
    char *b = (char *)base;
    auto take = [&](size_t bytes) { void *p = b + off; off = align256(off + bytes); return p; };
    const size_t nn = (size_t)n * n, nb = (size_t)batch;
    const int ncta = cdiv(n, EIG_ROWS) + 1;
    w.n = n; w.batch = batch; w.ld = n; w.mstride = (long)nn;
    w.L = (C2 *)take(sizeof(C2) * nn * nb);
    w.Wi = (C2 *)take(sizeof(C2) * nn * nb);
    w.A = (C2 *)take(sizeof(C2) * nn * nb);
    w.Y = (C2 *)take(sizeof(C2) * nn * nb);
    w.V = (C2 *)take(sizeof(C2) * nn * nb);
    w.VW = (C2 *)take(sizeof(C2) * n * 3 * EIG_NB * nb);
    w.wps = (long)n * 3 * EIG_NB;
    w.Wp = w.VW + (long)n * EIG_NB;
    w.wq = (C2 *)take(sizeof(C2) * n * nb);
    w.col = (C2 *)take(sizeof(C2) * n * nb);
    w.tau = (C2 *)take(sizeof(C2) * n * nb);
    w.pp = (C2 *)take(sizeof(C2) * 2 * EIG_NB * nb);
    w.part = (C2 *)take(sizeof(C2) * (2 * EIG_NB + 2) * ncta * nb);
    w.sc = (C2 *)take(sizeof(C2) * 4 * nb);
    const size_t nbw = (size_t)std::min(EIG_WY, n), nblk = n > 1 ? (size_t)cdiv(n - 1, (int)nbw) : 0;
    w.Tt = (C2 *)take(sizeof(C2) * (EIG_NAUX + nblk) * nbw * nbw * nb);   // G per aux stream | T of each block
    w.Xt = (C2 *)take(sizeof(C2) * std::max(EIG_NB, (int)nbw) * (size_t)n * nb);
    w.d = (double *)take(sizeof(double) * n * nb);
    w.e = (double *)take(sizeof(double) * n * nb);
    w.lam = (double *)take(sizeof(double) * n * nb);
    // inverse iteration: 6 arrays of n per thread slot, 64 cdiv(n, 64) slots per matrix
    w.ylu = (double *)take(sizeof(double) * 4 * (size_t)n * (64 * (size_t)cdiv(n, 64)) * nb);
    w.yvec = (double *)take(sizeof(double) * nn * nb);
    w.perm = (int *)take(sizeof(int) * 4 * n * nb);
    w.counter = (unsigned *)take(sizeof(unsigned) * nb);
    w.status = (int *)take(sizeof(int) * nb);
    if (!base) w.status = (int *)(uintptr_t)off;  // size query
}

// ---------------------------------------------------------------------------
template <typename C2>
__global__ void k_convert_h(const double2 *__restrict__ src, C2 *__restrict__ dst, long count)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < count; i += (long)gridDim.x * blockDim.x) {
        double2 v = src[i];
        C2 o;
        if constexpr (sizeof(o.x) == 4) {   // rounded with integer operations, off the FP64 pipe
            o.x = d2f_rn(v.x);
            o.y = d2f_rn(v.y);
        } else {
            o.x = v.x;
            o.y = v.y;
        }
        dst[i] = o;
    }
}

// ---------------------------------------------------------------------------
// v s, each part rounded on its own (never contracted into a later add)
__device__ __forceinline__ float2 scale_rn(float2 v, float s) { return make_float2(__fmul_rn(v.x, s), __fmul_rn(v.y, s)); }
__device__ __forceinline__ double2 scale_rn(double2 v, double s)
{
    return make_double2(__dmul_rn(v.x, s), __dmul_rn(v.y, s));
}

// Diagonal block: Cholesky L_jj L_jj^H = S_jj and its inverse, in shared memory.
template <typename T>
__global__ void __launch_bounds__(256) k_potrf_diag(EigWork<T> w, int j0, int jb)
{
    typedef typename cplx<T>::t C2;
    __shared__ C2 a[EIG_NB][EIG_NB + 1];   // a[c][r], updated in place
    __shared__ C2 x[EIG_NB][EIG_NB + 1];   // inverse, x[c][r]
    __shared__ int bad;
    const int b = blockIdx.x, tid = threadIdx.x;
    // lane = row r, warp = columns c = warp, warp + 8, ... (no index division)
    const int r = tid & 31, cg = tid >> 5;
    C2 *L = w.L + b * w.mstride + j0 + (long)j0 * w.ld;
    C2 *Wi = w.Wi + b * w.mstride + j0 + (long)j0 * w.ld;
    if (r < jb)
        for (int c = cg; c < jb; c += 8) a[c][r] = L[r + (long)c * w.ld];
    if (tid == 0) bad = 0;
    __syncthreads();
    // one barrier per column: every thread forms the pivot of column k itself,
    // and the scaled column k = a[k][.] / sqrt(pivot) on the fly for its
    // updates (the values the stored scaled column would hold).  Column k is
    // read but not written in step k; its finished values are written back by
    // its warp at the start of step k + 1, which reads only later columns.
    C2 held = cmk<T>(0, 0);
    int heldk = -1;
    for (int k = 0; k < jb; ++k) {
        if (heldk >= 0) { a[heldk][r] = held; heldk = -1; }
        T piv = a[k][k].x;
        const bool badk = !(piv > T(0));
        if (badk) piv = T(1);
        const T dk = sqrt(piv);
        const T inv = T(1) / dk;
        if (badk && tid == 0) bad = 1;
        if (r < jb && r >= k) {
            const C2 akr = r == k ? cmk<T>(dk, T(0)) : scale_rn(a[k][r], inv);
            if (cg == (k & 7)) { held = akr; heldk = k; }
            if (r > k) {
                int c = k + 1 + ((cg - (k + 1)) & 7);   // first column > k of this warp's group
                for (; c <= r; c += 8) a[c][r] = csub(a[c][r], cmul(akr, cconj(scale_rn(a[k][c], inv))));
            }
        }
        __syncthreads();
    }
    if (heldk >= 0) a[heldk][r] = held;
    __syncthreads();
    // inverse of the lower-triangular block, one column per thread
    if (tid < jb) {
        int c = tid;
        for (int rr = 0; rr < c; ++rr) x[c][rr] = cmk<T>(0, 0);
        x[c][c] = cmk<T>(T(1) / a[c][c].x, T(0));
        for (int rr = c + 1; rr < jb; ++rr) {
            C2 s = cmk<T>(0, 0);
            int k = c;
            for (; k + 8 <= rr; k += 8) {
                C2 av[8], xv[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    av[u] = a[k + u][rr];
                    xv[u] = x[c][k + u];
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) s = cadd(s, cmul(av[u], xv[u]));
            }
            for (; k < rr; ++k) s = cadd(s, cmul(a[k][rr], x[c][k]));
            x[c][rr] = cscale(s, -T(1) / a[rr][rr].x);
        }
    }
    __syncthreads();
    if (r < jb)
        for (int c = cg; c < jb; c += 8) {
            const C2 z = cmk<T>(0, 0);
            L[r + (long)c * w.ld] = (r >= c) ? a[c][r] : z;
            Wi[r + (long)c * w.ld] = (r >= c) ? x[c][r] : z;
        }
    if (tid == 0 && bad) w.status[b] = 1;
}

// ---------------------------------------------------------------------------
// Tridiagonalisation, column i of the panel starting at j0 (c = i - j0).
// KA: finalize W[:, c-1]; update column i; reflector (last CTA).
template <typename T>
__global__ void __launch_bounds__(EIG_ROWS) k_tri_colupd(EigWork<T> w, int i, int j0, int ncta)
{
    typedef typename cplx<T>::t C2;
    __shared__ C2 vi[EIG_NB], wi[EIG_NB];
    __shared__ T red[EIG_ROWS / 32];
    __shared__ unsigned ticket;
    const int b = blockIdx.y, n = w.n, c = i - j0, tid = threadIdx.x;
    const long ld = w.ld;
    C2 *A = w.A + b * w.mstride, *V = w.V + b * w.mstride;
    C2 *Wp = w.Wp + (long)b * w.wps, *wq = w.wq + (long)b * n, *col = w.col + (long)b * n;
    const C2 alpha_prev = w.sc[b * 4 + 1];
    // row i of the panel's V and W (W[i, c-1] recomputed from w', never read from Wp)
    if (tid < c) {
        vi[tid] = V[i + (long)(j0 + tid) * ld];
        if (tid < c - 1) wi[tid] = Wp[i + (long)tid * n];
        else wi[tid] = cadd(wq[i], cmul(alpha_prev, V[i + (long)(i - 1) * ld]));
    }
    __syncthreads();
    const int r = i + blockIdx.x * EIG_ROWS + tid;
    T nrm2 = T(0);
    if (r < n) {
        C2 wlast = cmk<T>(0, 0);
        if (c > 0) {
            wlast = cadd(wq[r], cmul(alpha_prev, V[r + (long)(i - 1) * ld]));
            Wp[r + (long)(c - 1) * n] = wlast;
        }
        C2 a = A[r + (long)i * ld];
        for (int j = 0; j < c; ++j) {
            C2 vrj = V[r + (long)(j0 + j) * ld];
            C2 wrj = (j < c - 1) ? Wp[r + (long)j * n] : wlast;
            a = csub(a, cmul(vrj, cconj(wi[j])));
            a = csub(a, cmul(wrj, cconj(vi[j])));
        }
        col[r] = a;
        if (r == i) w.d[(long)b * n + i] = (double)a.x;
        if (r >= i + 2) nrm2 = a.x * a.x + a.y * a.y;
    }
    __threadfence();   // col[] is read by the last CTA
    nrm2 = block_sum(nrm2, red);
    if (tid == 0) {
        C2 p; p.x = nrm2; p.y = T(0);
        w.part[((long)b * ncta + blockIdx.x) * (2 * EIG_NB + 2)] = p;
        __threadfence();
        ticket = atomicAdd(&w.counter[b], 1u);
    }
    __syncthreads();
    if (ticket != (unsigned)(ncta - 1) || tid != 0) return;
    // last CTA: Householder reflector (zlarfg) from col[i+1:]
    __threadfence();
    T xn2 = T(0);
    for (int q = 0; q < ncta; ++q) xn2 += __ldcg(&w.part[((long)b * ncta + q) * (2 * EIG_NB + 2)].x);
    C2 tau = cmk<T>(0, 0), scale = cmk<T>(0, 0);
    double beta = 0.0;
    if (i + 1 < n) {
        C2 al;
        al.x = __ldcg(&col[i + 1].x);
        al.y = __ldcg(&col[i + 1].y);
        T xnorm = sqrt(xn2);
        if (xnorm == T(0) && al.y == T(0)) {
            beta = (double)al.x;
        } else {
            T bb = sqrt(al.x * al.x + al.y * al.y + xnorm * xnorm);
            bb = (al.x >= T(0)) ? -bb : bb;
            tau = cmk<T>((bb - al.x) / bb, -al.y / bb);
            C2 den = cmk<T>(al.x - bb, al.y);         // 1 / (alpha - beta)
            T dd = den.x * den.x + den.y * den.y;
            scale = cmk<T>(den.x / dd, -den.y / dd);
            beta = (double)bb;
        }
        w.e[(long)b * n + i] = beta;
    }
    w.tau[(long)b * n + i] = tau;
    w.sc[b * 4 + 0] = scale;
    w.counter[b] = 0;
}

// KB: v = scaled column; p1 = W^H v, p2 = V^H v over the panel's previous columns.
template <typename T>
__global__ void __launch_bounds__(EIG_ROWS) k_tri_vdots(EigWork<T> w, int i, int j0, int ncta)
{
    typedef typename cplx<T>::t C2;
    __shared__ C2 sv[EIG_ROWS];
    __shared__ unsigned ticket;
    const int b = blockIdx.y, n = w.n, c = i - j0, tid = threadIdx.x;
    const long ld = w.ld;
    C2 *V = w.V + b * w.mstride, *Wp = w.Wp + (long)b * w.wps, *col = w.col + (long)b * n;
    const C2 scale = w.sc[b * 4 + 0];
    const int r = i + 1 + blockIdx.x * EIG_ROWS + tid;
    C2 v = cmk<T>(0, 0);
    if (r < n) {
        v = (r == i + 1) ? cmk<T>(1, 0) : cmul(col[r], scale);
        V[r + (long)i * ld] = v;
    }
    if (blockIdx.x == 0)
        for (int q = tid; q <= i; q += EIG_ROWS) V[q + (long)i * ld] = cmk<T>(0, 0);
    sv[tid] = v;
    __syncthreads();
    // partial dots: thread j < c sums W[:, j]^H v, thread EIG_NB + j sums V[:, j0+j]^H v
    C2 *part = w.part + ((long)b * ncta + blockIdx.x) * (2 * EIG_NB + 2);
    if (tid < 2 * EIG_NB) {
        int j = tid % EIG_NB;
        bool isV = tid >= EIG_NB;
        C2 s = cmk<T>(0, 0);
        if (j < c) {
            int r0 = i + 1 + blockIdx.x * EIG_ROWS;
            for (int q = 0; q < EIG_ROWS && r0 + q < n; ++q) {
                C2 m = isV ? V[r0 + q + (long)(j0 + j) * ld] : Wp[r0 + q + (long)j * n];
                cfmac(s, m, sv[q]);
            }
        }
        part[tid] = s;
        __threadfence();
    }
    __syncthreads();
    if (tid == 0) {
        ticket = atomicAdd(&w.counter[b], 1u);
    }
    __syncthreads();
    if (ticket != (unsigned)(ncta - 1)) return;
    __threadfence();
    if (tid < 2 * EIG_NB) {
        C2 s = cmk<T>(0, 0);
        for (int q = 0; q < ncta; ++q) {
            const C2 *p = w.part + ((long)b * ncta + q) * (2 * EIG_NB + 2) + tid;
            s.x += __ldcg(&p->x);
            s.y += __ldcg(&p->y);
        }
        w.pp[b * 2 * EIG_NB + tid] = s;
    }
    __syncthreads();
    if (tid == 0) w.counter[b] = 0;
}

// KC: y = A[i+1:, i+1:] v with A stored in its lower triangle.  32-row blocks,
// 32 x 32 tiles through shared memory, 8 column slices per row.
template <typename T>
__global__ void __launch_bounds__(256) k_tri_hemv(EigWork<T> w, int i)
{
    typedef typename cplx<T>::t C2;
    __shared__ C2 tile[32][33];
    __shared__ C2 vs[32];
    __shared__ C2 red[8][33];
    const int b = blockIdx.y, n = w.n, tid = threadIdx.x;
    const long ld = w.ld;
    const C2 *A = w.A + b * w.mstride, *V = w.V + b * w.mstride;
    const int base = i + 1, m = n - base;
    const int rb = blockIdx.x, r0 = base + 32 * rb;
    const int tr = tid & 31, tc = tid >> 5;
    C2 acc = cmk<T>(0, 0);
    const int ntile = cdiv(m, 32);
    for (int t = 0; t < ntile; ++t) {
        const int s0 = base + 32 * t;
        __syncthreads();
        if (tid < 32) vs[tid] = (s0 + tid < n) ? V[s0 + tid + (long)i * ld] : cmk<T>(0, 0);
        if (t <= rb) {
            // tile[rr][ss] = A[r0+rr, s0+ss], coalesced along rr
            for (int e = tid; e < 1024; e += 256) {
                int rr = e & 31, ss = e >> 5;
                int rg = r0 + rr, sg = s0 + ss;
                tile[rr][ss] = (rg < n && sg < n && sg <= rg) ? A[rg + (long)sg * ld] : cmk<T>(0, 0);
            }
        } else {
            // tile[rr][ss] = conj(A[s0+ss, r0+rr]), coalesced along ss
            for (int e = tid; e < 1024; e += 256) {
                int ss = e & 31, rr = e >> 5;
                int rg = r0 + rr, sg = s0 + ss;
                tile[rr][ss] = (rg < n && sg < n) ? cconj(A[sg + (long)rg * ld]) : cmk<T>(0, 0);
            }
        }
        __syncthreads();
        if (t == rb) {
            // diagonal tile: only the lower half was loaded; mirror it
            for (int e = tid; e < 1024; e += 256) {
                int rr = e & 31, ss = e >> 5;
                if (ss > rr) tile[rr][ss] = cconj(tile[ss][rr]);
            }
            __syncthreads();
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            int ss = tc + 8 * q;
            cfma(acc, tile[tr][ss], vs[ss]);
        }
    }
    red[tc][tr] = acc;
    __syncthreads();
    if (tid < 32) {
        C2 s = red[0][tid];
        for (int q = 1; q < 8; ++q) s = cadd(s, red[q][tid]);
        int rg = r0 + tid;
        if (rg < n) w.col[(long)b * n + rg] = s;
    }
}

// KD: w' = tau (y - V p1 - W p2); alpha = -tau/2 (w'^H v) (last CTA).
template <typename T>
__global__ void __launch_bounds__(EIG_ROWS) k_tri_wupd(EigWork<T> w, int i, int j0, int ncta)
{
    typedef typename cplx<T>::t C2;
    __shared__ C2 p1[EIG_NB], p2[EIG_NB];
    __shared__ T red[EIG_ROWS / 32];
    __shared__ unsigned ticket;
    const int b = blockIdx.y, n = w.n, c = i - j0, tid = threadIdx.x;
    const long ld = w.ld;
    const C2 *V = w.V + b * w.mstride, *Wp = w.Wp + (long)b * w.wps;
    C2 *wq = w.wq + (long)b * n;
    const C2 *y = w.col + (long)b * n;
    const C2 tau = w.tau[(long)b * n + i];
    if (tid < c) {
        p1[tid] = w.pp[b * 2 * EIG_NB + tid];
        p2[tid] = w.pp[b * 2 * EIG_NB + EIG_NB + tid];
    }
    __syncthreads();
    const int r = i + 1 + blockIdx.x * EIG_ROWS + tid;
    T dre = T(0), dim = T(0);
    if (r < n) {
        C2 s = y[r];
        for (int j = 0; j < c; ++j) {
            s = csub(s, cmul(V[r + (long)(j0 + j) * ld], p1[j]));
            s = csub(s, cmul(Wp[r + (long)j * n], p2[j]));
        }
        s = cmul(tau, s);
        wq[r] = s;
        C2 v = V[r + (long)i * ld];
        dre = s.x * v.x + s.y * v.y;      // conj(w') v
        dim = s.x * v.y - s.y * v.x;
    }
    if (blockIdx.x == 0)
        for (int q = tid; q <= i; q += EIG_ROWS) wq[q] = cmk<T>(0, 0);
    dre = block_sum(dre, red);
    dim = block_sum(dim, red);
    if (tid == 0) {
        C2 p; p.x = dre; p.y = dim;
        w.part[((long)b * ncta + blockIdx.x) * (2 * EIG_NB + 2) + 2 * EIG_NB] = p;
        __threadfence();
        ticket = atomicAdd(&w.counter[b], 1u);
    }
    __syncthreads();
    if (ticket != (unsigned)(ncta - 1) || tid != 0) return;
    __threadfence();
    C2 dot = cmk<T>(0, 0);
    for (int q = 0; q < ncta; ++q) {
        const C2 *p = w.part + ((long)b * ncta + q) * (2 * EIG_NB + 2) + 2 * EIG_NB;
        dot.x += __ldcg(&p->x);
        dot.y += __ldcg(&p->y);
    }
    w.sc[b * 4 + 1] = cscale(cmul(tau, dot), T(-0.5));
    w.counter[b] = 0;
}

// W[:, c] = w' + alpha v for the panel's last column.
template <typename T>
__global__ void k_tri_wfinal(EigWork<T> w, int i, int c)
{
    typedef typename cplx<T>::t C2;
    const int b = blockIdx.y, n = w.n;
    const C2 alpha = w.sc[b * 4 + 1];
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        C2 v = (r > i) ? w.V[b * w.mstride + r + (long)i * w.ld] : cmk<T>(0, 0);
        C2 q = (r > i) ? w.wq[(long)b * n + r] : cmk<T>(0, 0);
        w.Wp[(long)b * w.wps + r + (long)c * n] = cadd(q, cmul(alpha, v));
    }
}

// ---------------------------------------------------------------------------
// Tridiagonal eigenvalues: Sturm-count bisection inside each unreduced block.
// the same from per-row split flags (split after row k) in shared memory
__device__ inline void find_block_flags(const unsigned char *sp, int n, int r, int &b0, int &b1)
{
    b0 = r;
    while (b0 > 0 && !sp[b0 - 1]) --b0;
    b1 = r;
    while (b1 < n - 1 && !sp[b1]) ++b1;
}

__device__ inline void find_block(const double *d, const double *e, int n, int r, int &b0, int &b1)
{
    const double ulp = DBL_EPSILON;
    auto split = [&](int k) {   // negligible e[k]: split between rows k and k+1
        return fabs(d[k] * d[k + 1]) * ulp * ulp + DBL_MIN >= e[k] * e[k];
    };
    b0 = r;
    while (b0 > 0 && !split(b0 - 1)) --b0;
    b1 = r;
    while (b1 < n - 1 && !split(b1)) ++b1;
}

template <typename TB> __device__ inline TB tiny_of();
template <> __device__ inline float tiny_of<float>() { return FLT_MIN; }
template <> __device__ inline double tiny_of<double>() { return DBL_MIN; }
// Quotient in the tridiagonal recurrences: FP32 takes the reciprocal-based
// quotient (2 ulp; |b| stays below 2^126 there), FP64 the IEEE one.  The FP32
// eigenpairs are refined to FP64 accuracy afterwards.
__device__ inline float tri_div(float a, float b) { return __fdividef(a, b); }
__device__ inline double tri_div(double a, double b) { return a / b; }

// Bounds of an unreduced block [b0, b1] of T: Gershgorin interval [lo, hi],
// max row sum tnorm and max e^2.  When every valid thread of the CTA is in
// the same block (the usual case: one block per matrix) the CTA computes them
// together, each thread a strided part, then min / max over the CTA (exact in
// any order, so the values equal the one-thread loop's); otherwise each
// thread loops over its own block.  Every thread of the CTA must call it.
__device__ void block_bounds(const double *d, const double *e, bool valid, int b0, int b1, double &lo, double &hi,
                             double &tnorm, double &emax2)
{
    __shared__ int sblk[2];
    __shared__ double sred[4][32];
    if (threadIdx.x == 0) { sblk[0] = b0; sblk[1] = b1; }
    __syncthreads();
    const int c0 = sblk[0], c1 = sblk[1];
    const bool all = __syncthreads_and(!valid || (b0 == c0 && b1 == c1));
    auto part = [&](int k0, int k1, int step, int kb0, int kb1) {
        for (int k = k0; k <= k1; k += step) {
            const double off = (k > kb0 ? fabs(e[k - 1]) : 0.0) + (k < kb1 ? fabs(e[k]) : 0.0);
            lo = fmin(lo, d[k] - off);
            hi = fmax(hi, d[k] + off);
            tnorm = fmax(tnorm, fabs(d[k]) + off);
            if (k < kb1) emax2 = fmax(emax2, e[k] * e[k]);
        }
    };
    if (!all) {
        if (valid) part(b0, b1, 1, b0, b1);
        return;
    }
    part(c0 + (int)threadIdx.x, c1, (int)blockDim.x, c0, c1);
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        tnorm = fmax(tnorm, __shfl_xor_sync(0xffffffffu, tnorm, o));
        emax2 = fmax(emax2, __shfl_xor_sync(0xffffffffu, emax2, o));
    }
    const int wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) { sred[0][wid] = lo; sred[1][wid] = hi; sred[2][wid] = tnorm; sred[3][wid] = emax2; }
    __syncthreads();
    for (int q = 0; q < nw; ++q) {
        lo = fmin(lo, sred[0][q]);
        hi = fmax(hi, sred[1][q]);
        tnorm = fmax(tnorm, sred[2][q]);
        emax2 = fmax(emax2, sred[3][q]);
    }
}

// One thread per (matrix, row r): eigenvalue number r - b0 of r's block.
// FP32: the matrix's d and e^2 in FP32 and the split flags of find_block are
// staged once per CTA in shared memory (2 n floats + n bytes of dynamic shared
// memory), so the Sturm chains read them without a conversion from FP64 per
// step and the block search needs no FP64 work (the values are the same).
template <typename TB>
__global__ void k_tri_bisect(const double *dd, const double *ee, double *lamloc, int *blk, int n)
{
    extern __shared__ float bis_s[];
    const int b = blockIdx.y;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const double *d = dd + (long)b * n, *e = ee + (long)b * n;
    float *sd = bis_s, *se2 = bis_s + n;
    unsigned char *ssp = (unsigned char *)(bis_s + 2 * n);
    if (sizeof(TB) == 4) {
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            sd[k] = d2f_rn(d[k]);
            const float ek = d2f_rn(e[k]);
            se2[k] = ek * ek;
            // find_block's split test, once per row
            ssp[k] = k < n - 1 && fabs(d[k] * d[k + 1]) * DBL_EPSILON * DBL_EPSILON + DBL_MIN >= e[k] * e[k];
        }
        __syncthreads();
    }
    const bool valid = r < n;
    int b0 = 0, b1 = -1;
    if (valid) {
        if (sizeof(TB) == 4) find_block_flags(ssp, n, r, b0, b1);
        else find_block(d, e, n, r, b0, b1);
    }
    double tnorm = 0, lo = 1e300, hi = -1e300, emax2 = 0;
    block_bounds(d, e, valid, b0, b1, lo, hi, tnorm, emax2);
    if (!valid) return;
    const TB eps = eps_of<TB>();
    const TB pivmin = tiny_of<TB>() * TB(fmax(1.0, emax2));
    const TB atol = eps * TB(tnorm);
    const int j = r - b0;
    TB a = TB(lo) - TB(2) * atol - pivmin, z = TB(hi) + TB(2) * atol + pivmin;
    // Sturm count: eigenvalues of the block below x (FP32: from the shared
    // copies, the same values as converting d and e here)
    auto count = [&](TB x) {
        int cnt = 0;
        TB q = (sizeof(TB) == 4 ? TB(sd[b0]) : TB(d[b0])) - x;
        if (fabs(q) < pivmin) q = -pivmin;
        cnt += (q < TB(0));
        for (int k = b0 + 1; k <= b1; ++k) {
            TB e2;
            if (sizeof(TB) == 4) {
                e2 = TB(se2[k - 1]);
            } else {
                const TB ek = TB(e[k - 1]);
                e2 = ek * ek;
            }
            q = (sizeof(TB) == 4 ? TB(sd[k]) : TB(d[k])) - x - e2 / q;
            if (fabs(q) < pivmin) q = -pivmin;
            cnt += (q < TB(0));
        }
        return cnt;
    };
    if (sizeof(TB) == 4) {
        // FP32 (latency bound): octasection, seven independent Sturm chains per
        // pass; the new interval lies between the last point counting <= j
        // eigenvalues below it and the first counting more
        constexpr int NP = 7;
        for (int it = 0; it < 64; ++it) {
            const TB h = TB(1.0 / (NP + 1)) * (z - a);
            const TB tol = fmax(atol, TB(2) * eps * fmax(fabs(a), fabs(z))) + pivmin;
            TB m[NP];
            bool ok = z - a > tol;
#pragma unroll
            for (int i = 0; i < NP; ++i) m[i] = a + TB(i + 1) * h;
            ok = ok && m[0] > a && m[NP - 1] < z;
#pragma unroll
            for (int i = 0; i + 1 < NP; ++i) ok = ok && m[i] < m[i + 1];
            if (!ok) break;
            TB q[NP];
            int c[NP];
            const TB d0 = TB(sd[b0]);
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                q[i] = d0 - m[i];
                if (fabs(q[i]) < pivmin) q[i] = -pivmin;
                c[i] = q[i] < TB(0);
            }
            for (int k = b0 + 1; k <= b1; ++k) {
                const TB dk = TB(sd[k]), e2 = TB(se2[k - 1]);
#pragma unroll
                for (int i = 0; i < NP; ++i) {
                    q[i] = dk - m[i] - tri_div(e2, q[i]);
                    if (fabs(q[i]) < pivmin) q[i] = -pivmin;
                    c[i] += q[i] < TB(0);
                }
            }
            TB na = a, nz = z;
            bool found = false;
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                if (!found) {
                    if (c[i] <= j) na = m[i];
                    else { nz = m[i]; found = true; }
                }
            }
            a = na;
            z = nz;
        }
    }
    for (int it = 0; it < 256; ++it) {   // bisection (FP64; FP32 finishes here)
        const TB mid = TB(0.5) * (a + z);
        const TB tol = fmax(atol, TB(2) * eps * fmax(fabs(a), fabs(z))) + pivmin;
        if (!(z - a > tol) || mid == a || mid == z) break;
        if (count(mid) <= j) a = mid; else z = mid;
    }
    lamloc[(long)b * n + r] = (double)(TB(0.5) * (a + z));
    blk[((long)b * n + r) * 2 + 0] = b0;
    blk[((long)b * n + r) * 2 + 1] = b1;
}

// Global ascending order: rank of (lamloc[r], r).
__global__ void k_tri_rank(const double *lamloc, int *rank, double *lam, int n, int keys)
{
    extern __shared__ unsigned long long trk_keys[];
    const int b = blockIdx.y;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const double *L = lamloc + (long)b * n;
    const int cnt = rank_of(L, n, r, keys ? trk_keys : nullptr);
    if (r >= n) return;
    rank[(long)b * n + r] = cnt;
    lam[(long)b * n + cnt] = L[r];
}

__device__ inline unsigned hash_bits(unsigned a, unsigned b)
{
    unsigned h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u;
    h ^= h >> 15; h *= 0x2C1B3C6Du; h ^= h >> 12; h *= 0x297A2D39u; h ^= h >> 15;
    return h & 0xFFFFFFu;
}
// m 2^-23 - 1 in [-1, 1) for a 24-bit m: exact in FP32 as in FP64, so the FP32
// form gives the same values without the FP64 pipe
template <typename TB> __device__ inline TB hash_unit(unsigned a, unsigned b);
template <> __device__ inline double hash_unit<double>(unsigned a, unsigned b)
{
    return (double)hash_bits(a, b) / (double)0x800000 - 1.0;
}
template <> __device__ inline float hash_unit<float>(unsigned a, unsigned b)
{
    return (float)hash_bits(a, b) * (1.0f / 8388608.0f) - 1.0f;
}

// An array of one thread whose elements are `st` apart (thread-interleaved
// scratch: a warp's accesses to the same element index are coalesced).
template <typename TB> struct Strided {
    TB *p;
    long st;
    __device__ Strided(TB *p_, long st_) : p(p_), st(st_) {}
    __device__ TB &operator[](long k) const { return p[k * st]; }
    __device__ Strided operator+(long k) const { return Strided(p + k * st, st); }
};

// Tridiagonal eigenvectors by inverse iteration in TB arithmetic (FP64 for
// the FP64 form, FP32 for the FP32 solve of the mixed form), one thread per
// eigenvalue (dstein's dgttrf/dgtts2 steps, 3 iterations from a pseudo-random
// start in FP64, 2 in FP32), written to the eigenvalue's column of Y.  Members of a cluster of
// close eigenvalues iterate independently; k_tri_cluster_orth then
// orthonormalises each cluster.  An exactly degenerate cluster's iterates are
// independent random combinations inside its invariant subspace, and a member
// separated by g from the others keeps only ~eps ||T|| / g of their
// directions, so orthonormalising after the iteration spans the same subspace
// as re-orthogonalising during it.
//
// Each iteration is two sweeps.  The forward sweep factors T_block - lam I =
// P L U (dgttrf, the running row in registers) and applies P and L at the
// same time; the multipliers are used as they are made and never stored, and
// U's three diagonals are stored in the first iteration only (every
// iteration recomputes the same factor).  The backward sweep solves with U
// and accumulates the norm and the largest component; the normalisation is
// applied as the next sweep reads the vector.  Scratch: 4 arrays of n TB per
// thread, interleaved across the launch's threads (a warp's accesses to one
// element index are one coalesced line); the backward sweep loads INV_BLK
// steps' operands at once so that their latencies overlap.
constexpr int INV_BLK = 8;

template <typename TB>
__global__ void k_tri_invit(const double *dd, const double *ee, const double *lamloc, const int *blk,
                            const int *rank, double *yvec, TB *scratch, int n)
{
    const int b = blockIdx.y;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = r < n;
    const double *d = dd + (long)b * n, *e = ee + (long)b * n, *L = lamloc + (long)b * n;
    const int b0 = valid ? blk[((long)b * n + r) * 2] : 0, b1 = valid ? blk[((long)b * n + r) * 2 + 1] : -1;
    const int len = b1 - b0 + 1;
    // the block's max row sum: by the whole CTA when its threads share one
    // block (max is exact in any order), else per thread
    double tnorm = 0;
    {
        __shared__ int iblk[2];
        __shared__ double ired[32];
        if (threadIdx.x == 0) { iblk[0] = b0; iblk[1] = b1; }
        __syncthreads();
        const int c0 = iblk[0], c1 = iblk[1];
        const bool all = __syncthreads_and(!valid || (b0 == c0 && b1 == c1));
        const int k0 = all ? c0 + (int)threadIdx.x : b0, step = all ? (int)blockDim.x : 1;
        if (all || valid)
            for (int k = k0; k <= (all ? c1 : b1); k += step)
                tnorm = fmax(tnorm, fabs(d[k]) + (k > (all ? c0 : b0) ? fabs(e[k - 1]) : 0.0) +
                                        (k < (all ? c1 : b1) ? fabs(e[k]) : 0.0));
        if (all) {
            for (int o = 16; o > 0; o >>= 1) tnorm = fmax(tnorm, __shfl_xor_sync(0xffffffffu, tnorm, o));
            if ((threadIdx.x & 31) == 0) ired[threadIdx.x >> 5] = tnorm;
            __syncthreads();
            for (int q = 0; q < (int)((blockDim.x + 31) >> 5); ++q) tnorm = fmax(tnorm, ired[q]);
        }
    }
    // FP32: the matrix's d and e rounded once per CTA into shared memory (the
    // same values as converting at each step, without the FP64 pipe)
    extern __shared__ float invit_s[];
    const float *sdf = invit_s, *sef = invit_s + n;
    if (sizeof(TB) == 4) {
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            invit_s[k] = d2f_rn(d[k]);
            invit_s[n + k] = d2f_rn(e[k]);
        }
        __syncthreads();
    }
    auto Dk = [&](int k) { return sizeof(TB) == 4 ? TB(sdf[k]) : TB(d[k]); };
    auto Ek = [&](int k) { return sizeof(TB) == 4 ? TB(sef[k]) : TB(e[k]); };
    if (!valid) return;
    const long NT = (long)gridDim.y * gridDim.x * blockDim.x;
    Strided<TB> S(scratch + ((long)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x, NT);
    // 1 / pivots, first and second super-diagonals of U, iterate
    Strided<TB> RG = S, DU = S + n, DU2 = S + 2 * n, v = S + 3 * n;
    const TB tiny = eps_of<TB>() * TB(2) * TB(fmax(tnorm, (double)tiny_of<TB>()));
    const TB lam = TB(L[r]);
    auto pivot = [&](TB g) { return (fabs(g) < tiny) ? ((g < TB(0)) ? -tiny : tiny) : g; };
    const unsigned seed = (unsigned)(b * 7919 + r);
    // dstein's one converging solve and two extra (FP64); the FP32 solve of the
    // mixed form is refined afterwards, so one extra suffices there
    const int iters = sizeof(TB) == 8 ? 3 : 2;
    TB inv = TB(1);
    int kmax = 0;
    TB vmax = TB(-1), vkmax = TB(0);
    for (int it = 0; it < iters; ++it) {
        // forward: factor (dgttrf) and apply P, L; element k + 1 of the
        // right-hand side is the previous iterate scaled by inv (the random
        // start in the first iteration)
        auto rhs = [&](int k) { return it == 0 ? hash_unit<TB>(seed, (unsigned)k) : v[k] * inv; };
        TB dcur = Dk(b0) - lam, ducur = (len > 1) ? Ek(b0) : TB(0);
        TB vc = rhs(0);
        for (int kb = 0; kb < len - 1; kb += INV_BLK) {
            TB vn[INV_BLK];
#pragma unroll
            for (int u = 0; u < INV_BLK; ++u)
                if (kb + u < len - 1) vn[u] = rhs(kb + u + 1);
#pragma unroll
            for (int u = 0; u < INV_BLK; ++u) {
                const int k = kb + u;
                if (k >= len - 1) break;
                const TB dlk = Ek(b0 + k);
                TB dnext = Dk(b0 + k + 1) - lam;
                TB dunext = (k < len - 2) ? Ek(b0 + k + 1) : TB(0);
                if (fabs(dcur) >= fabs(dlk)) {
                    const TB f = (dcur != TB(0)) ? tri_div(dlk, dcur) : TB(0);
                    if (it == 0) { RG[k] = tri_div(TB(1), pivot(dcur)); DU[k] = ducur; DU2[k] = TB(0); }
                    dnext -= f * ducur;
                    v[k] = vc;
                    vc = vn[u] - f * vc;
                } else {
                    const TB f = tri_div(dcur, dlk);
                    if (it == 0) { RG[k] = tri_div(TB(1), pivot(dlk)); DU[k] = dnext; DU2[k] = dunext; }
                    dnext = ducur - f * dnext;
                    dunext = -f * dunext;
                    v[k] = vn[u];
                    vc = vc - f * vn[u];
                }
                dcur = dnext;
                ducur = dunext;
            }
        }
        if (it == 0) RG[len - 1] = tri_div(TB(1), pivot(dcur));
        // backward: U solve (the two following elements in registers), the
        // norm and the largest component (first in increasing k on ties)
        TB x1 = vc * RG[len - 1], x2 = TB(0);
        v[len - 1] = x1;
        TB nrm = x1 * x1;
        vmax = fabs(x1); kmax = len - 1; vkmax = x1;
        for (int kb = len - 2; kb >= 0; kb -= INV_BLK) {
            TB du[INV_BLK], du2[INV_BLK], rg[INV_BLK], vv[INV_BLK];
#pragma unroll
            for (int u = 0; u < INV_BLK; ++u) {
                const int k = kb - u;
                if (k >= 0) { du[u] = DU[k]; du2[u] = DU2[k]; rg[u] = RG[k]; vv[u] = v[k]; }
            }
#pragma unroll
            for (int u = 0; u < INV_BLK; ++u) {
                const int k = kb - u;
                if (k >= 0) {
                    const TB xk = (vv[u] - du[u] * x1 - du2[u] * x2) * rg[u];
                    v[k] = xk;
                    nrm += xk * xk;
                    if (fabs(xk) >= vmax) { vmax = fabs(xk); kmax = k; vkmax = xk; }
                    x2 = x1;
                    x1 = xk;
                }
            }
        }
        nrm = sqrt(nrm);
        inv = (nrm > TB(0)) ? TB(1) / nrm : TB(0);
    }
    // sign convention: largest component positive
    (void)kmax;
    // (widening and the sign with integer operations: the same values as
    // sg * (double) x, off the FP64 pipe)
    const long long sgbit = (vkmax < TB(0)) ? (long long)0x8000000000000000ull : 0ll;
    double *z = yvec + (long)b * n * n + (long)rank[(long)b * n + r] * n;
    // eight elements' loads before their stores (a load after a store to z
    // could alias it and would wait for it)
    for (int k8 = 0; k8 < n; k8 += 8) {
        TB vv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int k = k8 + u;
            vv[u] = (k < n && k >= b0 && k <= b1) ? v[k - b0] : TB(0);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int k = k8 + u;
            if (k >= n) break;
            double x = 0.0;
            if (k >= b0 && k <= b1) {
                if constexpr (sizeof(TB) == 4) x = f2d_exact(vv[u] * inv);
                else x = (double)(vv[u] * inv);
                x = __longlong_as_double(__double_as_longlong(x) ^ sgbit);
            }
            z[k] = x;
        }
    }
}

// Orthonormalise each cluster of eigenvalues closer than ctol ||T|| (within
// an unreduced block) by modified Gram-Schmidt, twice; one warp per
// eigenvalue, the warp of a cluster's first member does the work.
__global__ void __launch_bounds__(256) k_tri_cluster_orth(const double *dd, const double *ee, const double *lamloc,
                                                          const int *blk, const int *rank, double *yvec, int n,
                                                          double ctol)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b = blockIdx.y, r = blockIdx.x * 8 + warp;
    if (r >= n) return;   // warp-uniform
    const double *d = dd + (long)b * n, *e = ee + (long)b * n, *L = lamloc + (long)b * n;
    const int b0 = blk[((long)b * n + r) * 2], b1 = blk[((long)b * n + r) * 2 + 1];
    const int len = b1 - b0 + 1;
    double tnorm = 0;
    for (int k = b0 + lane; k <= b1; k += 32)
        tnorm = fmax(tnorm, fabs(d[k]) + (k > b0 ? fabs(e[k - 1]) : 0.0) + (k < b1 ? fabs(e[k]) : 0.0));
    for (int o = 16; o > 0; o >>= 1) tnorm = fmax(tnorm, __shfl_xor_sync(0xffffffffu, tnorm, o));
    const double gap = ctol * fmax(tnorm, DBL_MIN);
    if (r > b0 && L[r] - L[r - 1] < gap) return;   // not the first member
    int rend = r;
    while (rend < b1 && L[rend + 1] - L[rend] < gap) ++rend;
    if (rend == r) return;
    double *Y = yvec + (long)b * n * n;
    for (int m = r; m <= rend; ++m) {
        double *v = Y + (long)rank[(long)b * n + m] * n + b0;
        for (int pass = 0; pass < 2; ++pass) {
            for (int p = r; p < m; ++p) {
                const double *zp = Y + (long)rank[(long)b * n + p] * n + b0;
                double sdot = 0;
                for (int k = lane; k < len; k += 32) sdot += zp[k] * v[k];
                sdot = warp_sum(sdot);
                for (int k = lane; k < len; k += 32) v[k] -= sdot * zp[k];
                __syncwarp();
            }
        }
        double nrm = 0;
        for (int k = lane; k < len; k += 32) nrm += v[k] * v[k];
        nrm = sqrt(warp_sum(nrm));
        const double inv = (nrm > 0) ? 1.0 / nrm : 0.0;
        // sign convention: the first largest component positive
        double vmax = -1.0;
        int kmax = 0;
        for (int k = lane; k < len; k += 32) {
            const double a = fabs(v[k]);
            if (a > vmax) { vmax = a; kmax = k; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, vmax, o);
            const int ok = __shfl_xor_sync(0xffffffffu, kmax, o);
            if (ov > vmax || (ov == vmax && ok < kmax)) { vmax = ov; kmax = ok; }
        }
        const double sg = (v[kmax] < 0) ? -inv : inv;
        __syncwarp();
        for (int k = lane; k < len; k += 32) v[k] *= sg;
        __syncwarp();
    }
}

// real eigenvector matrix -> complex working precision
template <typename C2>
__global__ void k_real_to_cplx(const double *y, C2 *z, long count)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < count; i += (long)gridDim.x * blockDim.x) {
        C2 o;
        if constexpr (sizeof(o.x) == 4) o.x = d2f_rn(y[i]);
        else o.x = y[i];
        o.y = 0;
        z[i] = o;
    }
}

// compact-WY T factor of a block of jb <= EIG_WY reflectors (G = Vb^H Vb and T
// column-major nbw x nbw per matrix): column by column,
// T[0:c, c] = -tau_c T[0:c, 0:c] G[0:c, c], T[c, c] = tau_c (LAPACK's larft,
// forward columnwise).  One CTA of EIG_WY threads per matrix, thread = row;
// T is built in shared memory when it fits (FP32: 128 x 129 complex = 132 KB,
// dynamic), else in global memory.  Row r of T depends only on row r and on
// G, so the threads need no barrier between columns: the columns of G (and
// the taus) come in groups of LARFT_GC through shared memory, with a barrier
// per group.  The lanes of a warp walk k together from the warp's first row,
// so that their reads of T are consecutive and G[k, c] is one broadcast; row r
// adds its terms k >= r in order of k (the one-row-at-a-time sums).
constexpr int LARFT_GC = 8;
template <typename T, bool SMEM>
__global__ void __launch_bounds__(EIG_WY) k_larft_wy(const typename cplx<T>::t *G, typename cplx<T>::t *Tm,
                                                     const typename cplx<T>::t *tau, int n, int j0, int jb, int nbw)
{
    typedef typename cplx<T>::t C2;
    __shared__ C2 g[LARFT_GC][EIG_WY];
    __shared__ C2 tg[LARFT_GC];
    extern __shared__ __align__(16) unsigned char larft_smem[];
    const int b = blockIdx.x, r = threadIdx.x, kw = r & ~31;
    const C2 *Gb = G + (long)b * nbw * nbw;
    C2 *Tb = Tm + (long)b * nbw * nbw;
    const int lt = SMEM ? EIG_WY + 1 : nbw;   // column stride of the working T
    C2 *Tw = SMEM ? (C2 *)larft_smem : Tb;
    for (int c0 = 0; c0 < jb; c0 += LARFT_GC) {
        const int cn = min(LARFT_GC, jb - c0);
        __syncthreads();   // every thread is done with the previous group's columns
        for (int q = 0; q < cn; ++q)
            if (r < c0 + q) g[q][r] = Gb[r + (long)(c0 + q) * nbw];
        if (r < cn) tg[r] = tau[(long)b * n + j0 + c0 + r];
        __syncthreads();
        for (int q = 0; q < cn; ++q) {
            const int c = c0 + q;
            const C2 tc = tg[q];
            if (kw < c) {   // warp-uniform
                C2 acc = cmk<T>(0, 0);
                int k = kw;
                for (; k + 8 <= c; k += 8) {
                    C2 tv[8], gv[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        tv[u] = Tw[r + (k + u) * lt];
                        gv[u] = g[q][k + u];
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u)
                        if (k + u >= r) cfma(acc, tv[u], gv[u]);
                }
                for (; k < c; ++k)
                    if (k >= r) cfma(acc, Tw[r + k * lt], g[q][k]);
                if (r < c) Tw[r + (long)c * lt] = cscale(cmul(tc, acc), T(-1));
            }
            if (r == c) Tw[c + (long)c * lt] = tc;
        }
    }
    __syncthreads();
    if (SMEM)
        for (int c = 0; c < jb; ++c)
            if (r <= c) Tb[r + (long)c * nbw] = Tw[r + (long)c * lt];
}

// Join the inverted 32 x 32 diagonal blocks of L pairwise: for the 64-block at
// j0 = 64 t, W(j0+32.., j0..) = -W11 L10 W00 (W00, W11 the blocks' inverses,
// lower triangular; L10 the 32 x 32 block of L below W00).  One CTA per
// (pair, matrix); the three 32 x 32 blocks in shared memory.
template <typename T>
__global__ void __launch_bounds__(256) k_inv_pair(EigWork<T> w)
{
    typedef typename cplx<T>::t C2;
    __shared__ C2 a0[32][32], b1[32][32], lt[32][32];   // [col][row]
    const int b = blockIdx.y, n = w.n, tid = threadIdx.x;
    const int j0 = 2 * EIG_NB * blockIdx.x, j1 = j0 + EIG_NB;
    if (j1 >= n) return;
    const int m1 = min(EIG_NB, n - j1);
    const long ld = w.ld;
    const C2 *Wi = w.Wi + b * w.mstride, *L = w.L + b * w.mstride;
    C2 *Wo = w.Wi + b * w.mstride;
    const C2 z = cmk<T>(0, 0);
    for (int e = tid; e < 1024; e += 256) {
        const int r = e & 31, c = e >> 5;
        a0[c][r] = (r >= c) ? Wi[(j0 + r) + (long)(j0 + c) * ld] : z;
        b1[c][r] = (r >= c && r < m1) ? Wi[(j1 + r) + (long)(j1 + c) * ld] : z;
        lt[c][r] = (r < m1) ? L[(j1 + r) + (long)(j0 + c) * ld] : z;
    }
    __syncthreads();
    // T1 = W11 L10 (W11 lower: k <= r), four entries per thread
    C2 t1[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int e = tid + 256 * u, r = e & 31, c = e >> 5;
        C2 acc = z;
        for (int k = 0; k <= r; ++k) cfma(acc, b1[k][r], lt[c][k]);
        t1[u] = acc;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int e = tid + 256 * u;
        lt[e >> 5][e & 31] = t1[u];
    }
    __syncthreads();
    // W10 = -T1 W00 (W00 lower: k >= c)
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int e = tid + 256 * u, r = e & 31, c = e >> 5;
        C2 acc = z;
        for (int k = c; k < 32; ++k) cfma(acc, lt[k][r], a0[c][k]);
        if (r < m1) Wo[(j1 + r) + (long)(j0 + c) * ld] = cscale(acc, T(-1));
    }
}

// Rows t0.. of the panel's V columns j0..j0+jb into columns 0..jb and
// 2 EIG_NB.. of VW (W sits in between), for the merged trailing update
template <typename C2>
__global__ void k_copy_vpanel(const C2 *V, long ld, long ms, C2 *VW, long ldw, long wps, int t0, int j0, int jb,
                              int rem)
{
    const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= (long)rem * jb) return;
    const int b = blockIdx.y, r = (int)(e % rem), c = (int)(e / rem);
    const C2 v = V[b * ms + t0 + r + (long)(j0 + c) * ld];
    C2 *o = VW + b * wps + t0 + r;
    o[(long)c * ldw] = v;
    o[(long)(2 * EIG_NB + c) * ldw] = v;
}

__global__ void k_fill_int(int *p, int v, int count)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) p[i] = v;
}

// ---------------------------------------------------------------------------
template <typename T>
void eig_solve(cudaStream_t s, EigWork<T> &w, const double2 *H, const double2 *S, double *eig,
               typename cplx<T>::t *X, bool vectors, cudaEvent_t tri_start, const EigAux *ax)
{
    typedef typename cplx<T>::t C2;
    const int n = w.n, B = w.batch;
    const long ld = w.ld, ms = w.mstride;
    const C2 one = cmk<T>(1, 0), mone = cmk<T>(-1, 0), zero = cmk<T>(0, 0);
    const long cnt = (long)n * n * B;
    cudaMemsetAsync(w.status, 0, sizeof(int) * B, s);
    cudaMemsetAsync(w.counter, 0, sizeof(unsigned) * B, s);
    cudaMemsetAsync(w.sc, 0, sizeof(C2) * 4 * B, s);
    // 0. inputs in working precision: S -> L, H -> A (A is free until step 3)
    NRLTB_LAUNCH(k_convert_h<C2>, 1184, 256, 0, s, S, w.L, cnt);
    NRLTB_LAUNCH(k_convert_h<C2>, 1184, 256, 0, s, H, w.A, cnt);
    // 1. Cholesky S = L L^H
    for (int j0 = 0; j0 < n; j0 += EIG_NB) {
        const int jb = std::min(EIG_NB, n - j0), rem = n - j0 - jb;
        NRLTB_LAUNCH(k_potrf_diag<T>, B, 256, 0, s, w, j0, jb);
        if (rem > 0) {
            C2 *P = w.L + (j0 + jb) + (long)j0 * ld;
            zgemm<T>(s, rem, jb, jb, B, one, P, ld, ms, 0, w.Wi + j0 + (long)j0 * ld, ld, ms, 1, zero, P, ld, ms,
                     0, 1, 0);
            zgemm<T>(s, rem, rem, jb, B, mone, P, ld, ms, 0, P, ld, ms, 1, one,
                     w.L + (j0 + jb) + (long)(j0 + jb) * ld, ld, ms, 0, 0, 1);
        }
    }
    // 2. Wi = L^{-1}, bottom-up blocked: the 32 x 32 diagonal blocks are already
    //    inverted; pairs of them are joined into 64 x 64 diagonal inverses, then
    //    the 64-wide block columns are filled from the bottom (GEMMs with n = 64,
    //    wide enough for the tensor-core tile)
    {
        const int npair = cdiv(n, 2 * EIG_NB);
        NRLTB_LAUNCH(k_inv_pair<T>, dim3(npair, B), 256, 0, s, w);
        constexpr int NB2 = 2 * EIG_NB;
        int jlast = ((n - 1) / NB2) * NB2;
        for (int j0 = jlast; j0 >= 0; j0 -= NB2) {
            const int jb = std::min(NB2, n - j0), rem = n - j0 - jb;
            if (rem <= 0) continue;
            const long ldx = n;
            zgemm<T>(s, rem, jb, rem, B, one, w.Wi + (long)(j0 + jb) * (ld + 1), ld, ms, 0,
                     w.L + (j0 + jb) + (long)j0 * ld, ld, ms, 0, zero, w.Xt, ldx, (long)NB2 * n, 1, 0, 0);
            zgemm<T>(s, rem, jb, jb, B, mone, w.Xt, ldx, (long)NB2 * n, 0, w.Wi + (long)j0 * (ld + 1), ld, ms, 0,
                     zero, w.Wi + (j0 + jb) + (long)j0 * ld, ld, ms, 0, 2, 0);
        }
    }
    // 3. A = Wi H Wi^H (lower tiles); FP32: Wi^H formed explicitly in L (free
    //    after step 2) so that both tensor-core GEMMs stream stored operands
    if (sizeof(T) == 4) {
        conj_transpose<T>(s, w.Wi, w.L, n, B);
        zgemm<T>(s, n, n, n, B, one, w.A, ld, ms, 0, w.L, ld, ms, 0, zero, w.Y, ld, ms, 0, 1, 0);
    } else {
        zgemm<T>(s, n, n, n, B, one, w.A, ld, ms, 0, w.Wi, ld, ms, 1, zero, w.Y, ld, ms, 0, 1, 0);
    }
    zgemm<T>(s, n, n, n, B, one, w.Wi, ld, ms, 0, w.Y, ld, ms, 0, zero, w.A, ld, ms, 1, 0, 1);
    if (tri_start) cudaEventRecord(tri_start, s);
    // 4. tridiagonalisation: one cluster launch per panel (tri_panel.cuh); the
    //    per-column launch chain below is the path for devices or sizes where
    //    such a cluster cannot be scheduled
    bool clusters = true;
    for (int j0 = 0; j0 < n; j0 += EIG_NB) {
        const int jb = std::min(EIG_NB, n - j0);
        if (clusters) clusters = tri_panel_launch<T>(s, w, j0, jb);
        if (!clusters) {
            for (int c = 0; c < jb; ++c) {
                const int i = j0 + c;
                const int nA = cdiv(n - i, EIG_ROWS);
                NRLTB_LAUNCH(k_tri_colupd<T>, dim3(nA, B), EIG_ROWS, 0, s, w, i, j0, nA);
                if (i == n - 1) break;
                const int nB = cdiv(n - i - 1, EIG_ROWS);
                NRLTB_LAUNCH(k_tri_vdots<T>, dim3(nB, B), EIG_ROWS, 0, s, w, i, j0, nB);
                NRLTB_LAUNCH(k_tri_hemv<T>, dim3(cdiv(n - i - 1, 32), B), 256, 0, s, w, i);
                NRLTB_LAUNCH(k_tri_wupd<T>, dim3(nB, B), EIG_ROWS, 0, s, w, i, j0, nB);
            }
            const int last = std::min(j0 + jb - 1, n - 2);
            if (last >= j0) NRLTB_LAUNCH(k_tri_wfinal<T>, dim3(cdiv(n, 256), B), 256, 0, s, w, last, last - j0);
        }
        if (std::min(j0 + jb - 1, n - 2) < j0) break;
        const int t0 = j0 + jb, rem = n - t0;
        if (rem > 0) {
            C2 *Vp = w.V + t0 + (long)j0 * ld, *Wpp = w.Wp + t0;
            C2 *At = w.A + (long)t0 * (ld + 1);
            if (jb == EIG_NB) {
                // A -= [Vp Wp] [Wp Vp]^H in one rank-64 update: Vp copied on both sides of W
                NRLTB_LAUNCH(k_copy_vpanel<C2>, dim3(cdiv((long)rem * jb, 256), B), 256, 0, s, w.V, ld, ms, w.VW,
                             (long)n, w.wps, t0, j0, jb, rem);
                zgemm<T>(s, rem, rem, 2 * EIG_NB, B, mone, w.VW + t0, n, w.wps, 0, w.VW + t0 + (long)n * EIG_NB, n,
                         w.wps, 1, one, At, ld, ms, 0, 0, 1);
            } else {
                zgemm<T>(s, rem, rem, jb, B, mone, Vp, ld, ms, 0, Wpp, n, w.wps, 1, one, At, ld, ms, 0, 0, 1);
                zgemm<T>(s, rem, rem, jb, B, mone, Wpp, n, w.wps, 0, Vp, ld, ms, 1, one, At, ld, ms, 0, 0, 1);
            }
        }
    }
    // the back-transform's WY factors need only V and tau: with the auxiliary
    // streams they are formed there, a block on each in turn, while this one
    // solves the tridiagonal problem
    const int nbw = std::min(EIG_WY, n), nref = n - 1;
    const long sG = (long)nbw * nbw;
    auto Tf_of = [&](int j0) { return w.Tt + (long)(EIG_NAUX + j0 / nbw) * sG * B; };
    // block j0's G and T on stream st, with G buffer g
    auto wy_block = [&](cudaStream_t st, int g, int j0) {
        C2 *const G = w.Tt + (long)g * sG * B;
        const int jb = std::min(nbw, nref - j0), mb = n - j0 - 1;
        const C2 *Vb = w.V + (j0 + 1) + (long)j0 * ld;
        zgemm<T>(st, jb, jb, mb, B, one, Vb, ld, ms, 1, Vb, ld, ms, 0, zero, G, nbw, sG);
        if (sizeof(T) == 4) {
            const int sm = (int)(sizeof(C2) * EIG_WY * (EIG_WY + 1));
            smem_attr_at_least((const void *)k_larft_wy<T, true>, sm);
            NRLTB_LAUNCH((k_larft_wy<T, true>), B, EIG_WY, sm, st, G, Tf_of(j0), w.tau, n, j0, jb, nbw);
        } else {
            NRLTB_LAUNCH((k_larft_wy<T, false>), B, EIG_WY, 0, st, G, Tf_of(j0), w.tau, n, j0, jb, nbw);
        }
    };
    const int j0last = nref >= 1 ? ((nref - 1) / nbw) * nbw : -1;
    bool on_aux = vectors && ax && ax->tri_done;
    for (int q = 0; q < EIG_NAUX; ++q) on_aux = on_aux && ax->aux[q] && ax->wy_done[q];
    if (on_aux) {
        cudaEventRecord(ax->tri_done, s);
        for (int q = 0; q < EIG_NAUX; ++q) cudaStreamWaitEvent(ax->aux[q], ax->tri_done, 0);
        for (int j0 = j0last, q = 0; j0 >= 0; j0 -= nbw, q = (q + 1) % EIG_NAUX) wy_block(ax->aux[q], q, j0);
        for (int q = 0; q < EIG_NAUX; ++q) cudaEventRecord(ax->wy_done[q], ax->aux[q]);
    }
    // 5. tridiagonal eigenproblem (FP64 inverse iteration; bisection in T)
    double *lamloc = (double *)w.Xt;   // free at this point: n doubles per matrix fit
    int *blk = w.perm, *rank = w.perm + 2 * (long)n * B;
    {
        dim3 g(cdiv(n, 128), B);
        const size_t bsm = sizeof(T) == 4 ? 2 * sizeof(float) * n + n : 0;
        if (bsm > 48 * 1024)
            smem_attr_at_least((const void *)k_tri_bisect<T>, (int)bsm);
        NRLTB_LAUNCH(k_tri_bisect<T>, g, 128, bsm, s, w.d, w.e, lamloc, blk, n);
        const size_t rsm = rank_keys_bytes(n);
        if (rsm > 48 * 1024) smem_attr_at_least((const void *)k_tri_rank, (int)rsm);
        NRLTB_LAUNCH(k_tri_rank, g, 128, rsm, s, lamloc, rank, w.lam, n, rsm > 0 ? 1 : 0);
        cudaMemcpyAsync(eig, w.lam, sizeof(double) * n * B, cudaMemcpyDeviceToDevice, s);
    }
    if (!vectors) return;
    {
        // eigenvalues closer than ctol ||T|| are orthonormalised as one cluster
        // (LAPACK's dstein uses 1e-3 ||T||; outside a cluster the vectors'
        // overlap is ~ eps ||T|| / gap <= 1e-11 for FP64)
        const double ctol = 1e-5;
        // 64 threads per CTA: cdiv(n, 64) * 64 * B thread slots <= the scratch carve's 64 cdiv(n, 64) n B
        const size_t ism = sizeof(T) == 4 ? 2 * sizeof(float) * n : 0;
        if (ism > 48 * 1024)
            smem_attr_at_least((const void *)k_tri_invit<T>, (int)ism);
        NRLTB_LAUNCH(k_tri_invit<T>, dim3(cdiv(n, 64), B), 64, ism, s, w.d, w.e, lamloc, blk, rank, w.yvec,
                     (T *)w.ylu, n);
        NRLTB_LAUNCH(k_tri_cluster_orth, dim3(cdiv(n, 8), B), 256, 0, s, w.d, w.e, lamloc, blk, rank, w.yvec, n,
                     ctol);
        NRLTB_LAUNCH(k_real_to_cplx<C2>, 1184, 256, 0, s, w.yvec, w.Y, cnt);
    }
    // 6. Z = Q Y: blocks of EIG_WY reflectors applied last to first as
    //    Y[j0+1:, :] -= Vb (Tb (Vb^H Y[j0+1:, :])), Vb = V[j0+1:, j0:j0+jb] (the
    //    reflectors of the block vanish above row j0+1); then X = Wi^H Z.
    //    A (free after step 4) holds Vb^H Y, L (free after step 2) holds Tb Vb^H Y.
    {
        if (on_aux)
            for (int q = 0; q < EIG_NAUX; ++q) cudaStreamWaitEvent(s, ax->wy_done[q], 0);
        else
            for (int j0 = j0last; j0 >= 0; j0 -= nbw) wy_block(s, 0, j0);
        const long sX = (long)nbw * n;
        for (int j0 = (nref >= 1 ? ((nref - 1) / nbw) * nbw : -1); j0 >= 0; j0 -= nbw) {
            const int jb = std::min(nbw, nref - j0), mb = n - j0 - 1;
            const C2 *Vb = w.V + (j0 + 1) + (long)j0 * ld;
            C2 *Yb = w.Y + (j0 + 1);
            const C2 *Tf = Tf_of(j0);
            if (sizeof(T) == 4) {
                // Vb^H formed explicitly in Xt: the tensor-core GEMM streams an A
                // operand in its stored orientation twice as fast
                conj_transpose<T>(s, Vb, ld, ms, w.Xt, nbw, sX, mb, jb, B);
                zgemm<T>(s, jb, n, mb, B, one, w.Xt, nbw, sX, 0, Yb, ld, ms, 0, zero, w.A, nbw, sX);
            } else {
                zgemm<T>(s, jb, n, mb, B, one, Vb, ld, ms, 1, Yb, ld, ms, 0, zero, w.A, nbw, sX);
            }
            zgemm<T>(s, jb, n, jb, B, one, Tf, nbw, sG, 0, w.A, nbw, sX, 0, zero, w.L, nbw, sX, 2, 0, 0);
            zgemm<T>(s, mb, n, jb, B, mone, Vb, ld, ms, 0, w.L, nbw, sX, 0, one, Yb, ld, ms);
        }
        if (sizeof(T) == 4) {
            // Wi^H formed explicitly in L (free again): the tensor-core GEMM
            // streams an A operand in its stored orientation twice as fast
            conj_transpose<T>(s, w.Wi, w.L, n, B);
            zgemm<T>(s, n, n, n, B, one, w.L, ld, ms, 0, w.Y, ld, ms, 0, zero, X, ld, ms, 2, 0, 0);
        } else {
            zgemm<T>(s, n, n, n, B, one, w.Wi, ld, ms, 1, w.Y, ld, ms, 0, zero, X, ld, ms, 2, 0, 0);
        }
    }
}

template size_t eig_work_bytes<double>(int, int);
template size_t eig_work_bytes<float>(int, int);
template void eig_work_carve<double>(EigWork<double> &, void *, int, int);
template void eig_work_carve<float>(EigWork<float> &, void *, int, int);
template void eig_solve<double>(cudaStream_t, EigWork<double> &, const double2 *, const double2 *, double *,
                                double2 *, bool, cudaEvent_t, const EigAux *);
template void eig_solve<float>(cudaStream_t, EigWork<float> &, const double2 *, const double2 *, double *,
                               float2 *, bool, cudaEvent_t, const EigAux *);

}  // namespace nrltb
