// tri_panel.cuh -- one panel (up to EIG_NB columns) of the blocked Householder
// tridiagonalisation A = Q T Q^H, with one thread-block cluster per matrix.
//
// The per-column chain of zhetrd/zlatrd (column update, reflector, Hermitian
// mat-vec y = A v of the trailing matrix, w = tau (y - V p1 - W p2),
// alpha = -tau/2 w^H v) is latency bound when each step is its own launch.
// Here the CL CTAs of a cluster own the matrix rows in 32-row tiles (tile t
// belongs to CTA t mod CL) and run every column of the panel in one launch,
// with three cluster barriers per column.  The cluster-wide sums (|x|^2 of
// the reflector, W^H v / V^H v, w^H v) are per-CTA partials in shared memory,
// read by every CTA through distributed shared memory in rank order, so all
// CTAs derive identical scalars without a further barrier and the result does
// not depend on scheduling.
//
// The mat-vec reads only A's lower triangle: for an own row tile R and a
// column tile S > R, the lower tile (S, R) is read (coalesced) and its
// conjugate transpose applied with a warp butterfly (transpose-reduce), so a
// CTA forms the whole y of its own rows without cross-CTA traffic.
//
// The CTA keeps its own rows of the panel's V and W columns (and of w') in
// shared memory, so the per-column updates read no global memory but the
// current column of A, row i and the mat-vec tiles.
//
// Every CTA executes the same sequence of barriers: control flow that
// encloses a barrier depends only on kernel arguments.
#pragma once
#include <cooperative_groups.h>
#include "eig.cuh"

namespace nrltb {

constexpr int TP_THREADS = 256, TP_WARPS = TP_THREADS / 32;
constexpr int TP_CL = 8;   // CTAs per cluster (portable size)

// values per lane of one butterfly (16: two CTAs of 256 threads fit an SM)
template <typename T> struct TpNV { static constexpr int v = 16; };

// Transpose-reduce over the warp: lane l holds x[0..NV); afterwards x[0] of
// lane l is sum over all lanes of x[u] with u = l >> (5 - log2 NV) (lanes that
// share u hold the same total).
template <int NV, typename C2>
__device__ __forceinline__ void tp_butterfly(C2 (&x)[NV], int lane)
{
    int o = 16;
#pragma unroll
    for (int m = NV; m > 1; m >>= 1, o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int u = 0; u < m / 2; ++u) {
            C2 send = up ? x[u] : x[u + m / 2];
            C2 keep = up ? x[u + m / 2] : x[u];
            keep.x += __shfl_xor_sync(0xffffffffu, send.x, o);
            keep.y += __shfl_xor_sync(0xffffffffu, send.y, o);
            x[u] = keep;
        }
    }
    for (; o > 0; o >>= 1) {
        x[0].x += __shfl_xor_sync(0xffffffffu, x[0].x, o);
        x[0].y += __shfl_xor_sync(0xffffffffu, x[0].y, o);
    }
}

template <typename T> struct TpSmem {
    typedef typename cplx<T>::t C2;
    C2 *vfull;      // v of the current column, all rows (32 T_)
    C2 *acol;       // own rows: updated column, then v (32 nown)
    C2 *ypart;      // per warp: partial y of the own rows (TP_WARPS x 32 nown)
    C2 *Vs, *Ws;    // own rows of the panel's V and W columns (EIG_NB x 32 nown each)
    C2 *wqs;        // own rows of w' of the previous column (32 nown)
    C2 *wi, *vi;    // row i of the panel's W and V
    C2 *p1, *p2;    // W^H v, V^H v (cluster sums)
    C2 *pw;         // per-warp partials of W^H v | V^H v (TP_WARPS x 64)
    C2 *p12part;    // this CTA's W^H v | V^H v (64)
    C2 *a0;         // element i+1 of the updated column (owner CTA)
    C2 *dotpart;    // this CTA's w^H v
    T *normpart;    // this CTA's |x|^2
    T *red;         // block_sum scratch
};

inline size_t tp_smem_bytes(int n, int csize, size_t c2)
{
    const int T_ = cdiv(n, 32), nown = cdiv(T_, TP_CL);
    (void)csize;
    return c2 * (32 * (size_t)T_ + 32 * (size_t)nown * (2 + TP_WARPS + 2 * EIG_NB) + 4 * 32 + TP_WARPS * 64 + 64 +
                 2) +
           2 * 16 * (TP_WARPS + 1) + 64;
}

template <typename T>
__device__ __forceinline__ TpSmem<T> tp_carve(unsigned char *base, int n)
{
    typedef typename cplx<T>::t C2;
    const int T_ = cdiv(n, 32), nown = cdiv(T_, TP_CL);
    TpSmem<T> s;
    C2 *p = (C2 *)base;
    s.vfull = p; p += 32 * T_;
    s.acol = p; p += 32 * nown;
    s.ypart = p; p += 32 * nown * TP_WARPS;
    s.Vs = p; p += 32 * nown * EIG_NB;
    s.Ws = p; p += 32 * nown * EIG_NB;
    s.wqs = p; p += 32 * nown;
    s.wi = p; p += 32;
    s.vi = p; p += 32;
    s.p1 = p; p += 32;
    s.p2 = p; p += 32;
    s.pw = p; p += TP_WARPS * 64;
    s.p12part = p; p += 64;
    s.a0 = p; p += 1;
    s.dotpart = p; p += 1;
    T *q = (T *)p;
    s.normpart = q; q += 2;
    s.red = q;
    return s;
}

// The trailing mat-vec for own row tile R over column tiles [s_lo, s_hi), one
// warp: y_R += A_RS v_S for S < R (lane = row), for S > R the lower tile (S, R)
// is read by rows and its conjugate transpose applied: the lanes' products are
// summed over all S of the strip in registers and reduced across lanes once per
// half tile (butterfly), and the diagonal tile combines both.  Tiles inside
// [lo, n) in both directions take an unmasked path.  Contributions are added to
// this warp's ypart slots of tile R.
template <typename T>
__device__ __forceinline__ void tp_strip(const typename cplx<T>::t *A, long ld, int n, int lo, int R, int s_lo,
                                         int s_hi, const typename cplx<T>::t *vfull, typename cplx<T>::t *yp,
                                         int lane)
{
    typedef typename cplx<T>::t C2;
    constexpr int NV = TpNV<T>::v;
    C2 yr = cmk<T>(0, 0);
    const bool has_upper = s_hi - 1 >= R;   // trans or diagonal tiles in the strip (warp-uniform)
#pragma unroll 1
    for (int h = 0; h < 32 / NV; ++h) {
        C2 x[NV];
#pragma unroll
        for (int u = 0; u < NV; ++u) x[u] = cmk<T>(0, 0);
#pragma unroll 1
        for (int S = s_lo; S < s_hi; ++S) {
            const bool trans = S > R, diag = S == R;
            const int rowt = trans ? S : R, colt = trans ? R : S;
            const int r = 32 * rowt + lane, c0 = 32 * colt + h * NV;
            const C2 vr = vfull[r];
            const bool interior = !diag && 32 * rowt >= lo && 32 * rowt + 31 < n && c0 >= lo && c0 + NV <= n;
            C2 a[NV];
            if (interior) {
#pragma unroll
                for (int u = 0; u < NV; ++u) a[u] = A[r + (long)(c0 + u) * ld];
            } else {
                const bool rv = r >= lo && r < n;
#pragma unroll
                for (int u = 0; u < NV; ++u) {
                    const int sc = c0 + u;
                    a[u] = cmk<T>(0, 0);
                    if (rv && sc >= lo && sc < n && (!diag || sc <= r)) a[u] = A[r + (long)sc * ld];
                }
            }
            if (!trans) {
#pragma unroll
                for (int u = 0; u < NV; ++u) cfma(yr, a[u], vfull[c0 + u]);
            }
            if (trans) {
#pragma unroll
                for (int u = 0; u < NV; ++u) cfmac(x[u], a[u], vr);   // conj(a) v_r
            } else if (diag) {
#pragma unroll
                for (int u = 0; u < NV; ++u)
                    if (c0 + u < r) cfmac(x[u], a[u], vr);
            }
        }
        if (has_upper) {
            tp_butterfly<NV>(x, lane);
            constexpr int sh = (NV == 32) ? 0 : (NV == 16 ? 1 : 2);
            if ((lane & ((1 << sh) - 1)) == 0) {
                C2 &dst = yp[h * NV + (lane >> sh)];
                dst = cadd(dst, x[0]);
            }
        }
    }
    yp[lane] = cadd(yp[lane], yr);
}

template <typename T>
__global__ void __launch_bounds__(TP_THREADS, 2) k_tri_panel(EigWork<T> w, int j0, int jb)
{
    typedef typename cplx<T>::t C2;
    namespace cg = cooperative_groups;
    constexpr int CL = TP_CL, NV = TpNV<T>::v;
    extern __shared__ __align__(16) unsigned char tp_raw[];
    cg::cluster_group cluster = cg::this_cluster();
    const int q = (int)cluster.block_rank();
    const int b = blockIdx.y, n = w.n, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long ld = w.ld;
    const C2 *A = w.A + b * w.mstride;
    C2 *V = w.V + b * w.mstride;
    C2 *Wp = w.Wp + (long)b * w.wps, *wq = w.wq + (long)b * n;
    const int T_ = cdiv(n, 32);
    const int nown = (q < T_) ? (T_ - 1 - q) / CL + 1 : 0;
    TpSmem<T> sm = tp_carve<T>(tp_raw, n);
    const int ns = 32 * cdiv(T_, CL);   // row stride of Vs, Ws
    const C2 zero = cmk<T>(0, 0);

    C2 tau = zero, alpha = zero;
    int c = 0;
    for (; c < jb; ++c) {
        const int i = j0 + c;
        // ---- A: alpha of the previous column; row i of V, W; update column i ----
        if (c > 0) {
            C2 dot = zero;
            for (int rk = 0; rk < CL; ++rk) dot = cadd(dot, *cluster.map_shared_rank(sm.dotpart, rk));
            alpha = cscale(cmul(tau, dot), T(-0.5));
        }
        if (tid < c) {
            sm.vi[tid] = V[i + (long)(j0 + tid) * ld];
            sm.wi[tid] = (tid < c - 1) ? Wp[i + (long)tid * n] : cadd(wq[i], cmul(alpha, V[i + (long)(i - 1) * ld]));
        }
        __syncthreads();
        T nrm2 = T(0);
        for (int k = warp; k < nown; k += TP_WARPS) {
            const int r = 32 * (q + CL * k) + lane;
            if (r < i || r >= n) continue;
            C2 a = A[r + (long)i * ld];   // before the store to Wp, which it could alias
            C2 wl = zero;
            const int slot = 32 * k + lane;
            if (c > 0) {
                wl = cadd(sm.wqs[slot], cmul(alpha, sm.Vs[(c - 1) * ns + slot]));
                Wp[r + (long)(c - 1) * n] = wl;
                sm.Ws[(c - 1) * ns + slot] = wl;
            }
            // eight panel columns per round: their loads are issued together
            for (int j8 = 0; j8 < c; j8 += 8) {
                C2 vv[8], ww[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int j = j8 + u;
                    vv[u] = zero;
                    ww[u] = zero;
                    if (j < c) {
                        vv[u] = sm.Vs[j * ns + slot];
                        ww[u] = sm.Ws[j * ns + slot];
                    }
                }
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (j8 + u < c) {
                        a = csub(a, cmul(vv[u], cconj(sm.wi[j8 + u])));
                        a = csub(a, cmul(ww[u], cconj(sm.vi[j8 + u])));
                    }
            }
            sm.acol[32 * k + lane] = a;
            if (r == i) w.d[(long)b * n + i] = (double)a.x;
            if (r == i + 1) *sm.a0 = a;
            if (r >= i + 2) nrm2 += a.x * a.x + a.y * a.y;
        }
        // CTA sum with one barrier: warp sums, then thread 0 adds them in warp order
        nrm2 = warp_sum(nrm2);
        if (lane == 0) sm.red[warp] = nrm2;
        __syncthreads();
        if (tid == 0) {
            T t = T(0);
            for (int ww = 0; ww < TP_WARPS; ++ww) t += sm.red[ww];
            *sm.normpart = t;
        }
        if (i == n - 1) break;   // last column of the matrix: d only (uniform)
        cluster.sync();   // #1

        // ---- B: reflector (every CTA, same order); v; partial W^H v, V^H v ----
        T xn2 = T(0);
        for (int rk = 0; rk < CL; ++rk) xn2 += *cluster.map_shared_rank(sm.normpart, rk);
        const C2 al = *cluster.map_shared_rank(sm.a0, ((i + 1) / 32) % CL);
        C2 scale = zero;
        double beta;
        tau = zero;
        {
            const T xnorm = sqrt(xn2);
            if (xnorm == T(0) && al.y == T(0)) {
                beta = (double)al.x;
            } else {
                T bb = sqrt(al.x * al.x + al.y * al.y + xnorm * xnorm);
                bb = (al.x >= T(0)) ? -bb : bb;
                tau = cmk<T>((bb - al.x) / bb, -al.y / bb);
                const C2 den = cmk<T>(al.x - bb, al.y);   // 1 / (alpha - beta)
                const T dd = den.x * den.x + den.y * den.y;
                scale = cmk<T>(den.x / dd, -den.y / dd);
                beta = (double)bb;
            }
        }
        if (q == 0 && tid == 0) {
            w.e[(long)b * n + i] = beta;
            w.tau[(long)b * n + i] = tau;
        }
        if (q == 0)
            for (int qq = tid; qq <= i; qq += TP_THREADS) V[qq + (long)i * ld] = zero;
        // this warp's W^H v | V^H v slots: cleared by the warp itself
        for (int e = lane; e < 64; e += 32) sm.pw[warp * 64 + e] = zero;
        __syncwarp();
        for (int k = warp; k < nown; k += TP_WARPS) {
            const int r = 32 * (q + CL * k) + lane;
            const bool valid = r >= i + 1 && r < n;
            C2 v = zero;
            if (valid) {
                v = (r == i + 1) ? cmk<T>(1, 0) : cmul(sm.acol[32 * k + lane], scale);
                V[r + (long)i * ld] = v;
            }
            sm.acol[32 * k + lane] = v;
            sm.Vs[c * ns + 32 * k + lane] = v;
            // W^H v and V^H v over this warp's rows: column j in butterfly slot j
#pragma unroll 1
            for (int part = 0; part < 2; ++part) {
#pragma unroll 1
                for (int h = 0; h < 32 / NV; ++h) {
                    C2 x[NV];
#pragma unroll
                    for (int u = 0; u < NV; ++u) {
                        const int j = h * NV + u;
                        x[u] = zero;
                        if (valid && j < c) {
                            const C2 m = part ? sm.Vs[j * ns + 32 * k + lane] : sm.Ws[j * ns + 32 * k + lane];
                            cfmac(x[u], m, v);
                        }
                    }
                    tp_butterfly<NV>(x, lane);
                    constexpr int sh = (NV == 32) ? 0 : 1;
                    if ((lane & ((1 << sh) - 1)) == 0) {
                        C2 &dst = sm.pw[warp * 64 + part * 32 + h * NV + (lane >> sh)];
                        dst = cadd(dst, x[0]);
                    }
                }
            }
        }
        __syncthreads();
        if (tid < 64) {
            C2 s = zero;
            for (int ww = 0; ww < TP_WARPS; ++ww) s = cadd(s, sm.pw[ww * 64 + tid]);
            sm.p12part[tid] = s;
        }
        cluster.sync();   // #2

        // ---- C: cluster sums p1, p2; full v; trailing mat-vec for own rows ----
        if (tid < 64) {
            C2 s = zero;
            for (int rk = 0; rk < CL; ++rk) s = cadd(s, cluster.map_shared_rank(sm.p12part, rk)[tid]);
            if (tid < 32) sm.p1[tid] = s; else sm.p2[tid - 32] = s;
        }
        for (int s = tid; s < 32 * T_; s += TP_THREADS)
            sm.vfull[s] = (s >= i + 1 && s < n) ? V[s + (long)i * ld] : zero;
        for (int e = tid; e < 32 * nown * TP_WARPS; e += TP_THREADS) sm.ypart[e] = zero;
        __syncthreads();
        {
            // each own row tile's column tiles are cut into TP_WARPS contiguous strips
            const int tb = (i + 1) / 32, ncol = T_ - tb;
            C2 *yw = sm.ypart + warp * 32 * nown;
            const int s_lo = tb + (warp * ncol) / TP_WARPS, s_hi = tb + ((warp + 1) * ncol) / TP_WARPS;
            for (int k = 0; k < nown; ++k) {
                const int R = q + CL * k;
                if (R < tb || s_lo >= s_hi) continue;
                tp_strip<T>(A, ld, n, i + 1, R, s_lo, s_hi, sm.vfull, yw + 32 * k, lane);
            }
        }
        __syncthreads();

        // ---- D: w' = tau (y - V p1 - W p2) for own rows; partial w'^H v ----
        C2 dot = zero;
        for (int k = warp; k < nown; k += TP_WARPS) {
            const int r = 32 * (q + CL * k) + lane;
            if (r < i + 1 || r >= n) continue;
            C2 y = zero;
            for (int ww = 0; ww < TP_WARPS; ++ww) y = cadd(y, sm.ypart[ww * 32 * nown + 32 * k + lane]);
            for (int j8 = 0; j8 < c; j8 += 8) {
                C2 vv[8], ww[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int j = j8 + u;
                    vv[u] = zero;
                    ww[u] = zero;
                    if (j < c) {
                        vv[u] = sm.Vs[j * ns + 32 * k + lane];
                        ww[u] = sm.Ws[j * ns + 32 * k + lane];
                    }
                }
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (j8 + u < c) {
                        y = csub(y, cmul(vv[u], sm.p1[j8 + u]));
                        y = csub(y, cmul(ww[u], sm.p2[j8 + u]));
                    }
            }
            y = cmul(tau, y);
            wq[r] = y;
            sm.wqs[32 * k + lane] = y;
            cfmac(dot, y, sm.acol[32 * k + lane]);   // conj(w') v
        }
        if (q == 0)
            for (int qq = tid; qq <= i; qq += TP_THREADS) wq[qq] = zero;
        dot.x = warp_sum(dot.x);
        dot.y = warp_sum(dot.y);
        if (lane == 0) { sm.red[2 * warp] = dot.x; sm.red[2 * warp + 1] = dot.y; }
        __syncthreads();
        if (tid == 0) {
            C2 t = zero;
            for (int ww = 0; ww < TP_WARPS; ++ww) { t.x += sm.red[2 * ww]; t.y += sm.red[2 * ww + 1]; }
            *sm.dotpart = t;
        }
        cluster.sync();   // #3
    }
    // W[:, last] = w' + alpha v of the panel's last reflected column
    if (c == jb) {
        const int i = j0 + jb - 1;
        C2 dot = zero;
        for (int rk = 0; rk < CL; ++rk) dot = cadd(dot, *cluster.map_shared_rank(sm.dotpart, rk));
        alpha = cscale(cmul(tau, dot), T(-0.5));
        for (int k = warp; k < nown; k += TP_WARPS) {
            const int r = 32 * (q + CL * k) + lane;
            if (r >= n) continue;
            const C2 v = (r > i) ? sm.Vs[(jb - 1) * ns + 32 * k + lane] : zero;
            const C2 qv = (r > i) ? sm.wqs[32 * k + lane] : zero;
            Wp[r + (long)(jb - 1) * n] = cadd(qv, cmul(alpha, v));
        }
    }
    cluster.sync();   // no CTA leaves while others may read its shared memory
}

// Launches the panel kernel with cluster dimension TP_CL; returns false if a
// cluster of this size and shared memory cannot be scheduled on the device.
template <typename T>
bool tri_panel_launch(cudaStream_t s, const EigWork<T> &w, int j0, int jb)
{
    // FP64: the mat-vec is bound by the FP64 pipe, which the per-column launch
    // chain (every SM on every column) uses better than 8 CTAs per matrix
    if (sizeof(T) == 8) return false;
    const size_t smem = tp_smem_bytes(w.n, 0, sizeof(typename cplx<T>::t));
    if (smem > 200 * 1024) return false;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = TP_CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(TP_CL, w.batch, 1);
    cfg.blockDim = dim3(TP_THREADS, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (smem_attr_at_least((const void *)k_tri_panel<T>, (int)smem) != cudaSuccess) {
        cudaGetLastError();   // not sticky: the per-column path takes over
        return false;
    }
    {
        // whether a cluster of this shared-memory size can be scheduled, once per
        // (device, size) for the whole process (the answer does not depend on
        // which thread asks or on what ran before)
        static std::mutex mu;
        static std::map<std::pair<int, size_t>, bool> fits;
        std::lock_guard<std::mutex> g(mu);
        auto it = fits.find(std::make_pair(dev, smem));
        if (it == fits.end()) {
            int nclusters = 0;
            const bool ok = cudaOccupancyMaxActiveClusters(&nclusters, k_tri_panel<T>, &cfg) == cudaSuccess &&
                            nclusters > 0;
            cudaGetLastError();
            it = fits.emplace(std::make_pair(dev, smem), ok).first;
        }
        if (!it->second) return false;
    }
    cudaEvent_t ev = kt_begin(s);
    if (cudaLaunchKernelEx(&cfg, k_tri_panel<T>, w, j0, jb) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (g_launch_counter) ++*g_launch_counter;
    // algorithmic bytes: the lower triangle of each column's trailing matrix, read once
    double bytes = 0;
    for (int c = 0; c < jb; ++c) {
        const double m = w.n - (j0 + c) - 1;
        bytes += 0.5 * m * (m + 1) * sizeof(typename cplx<T>::t);
    }
    kt_end(ev, s, KC_TRI_PANEL, bytes * w.batch);
    return true;
}

}  // namespace nrltb
