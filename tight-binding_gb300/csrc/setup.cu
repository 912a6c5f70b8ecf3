// setup.cu -- per-structure k-independent stage and the Bloch sums.
//
//   search2.f:95-223   neighbour list: one thread per (iat, jat, image) candidate,
//                      then an order-preserving compaction, so the pair list is
//                      the reference's, integer for integer.  Distances use the
//                      reference's operation order with no fused multiply-add.
//   setpar.f:399-884   SK integrals per pair; on-site densities summed per atom
//   setparv.f:426-886  in the reference's pair order; on-site polynomials.
//   rotate.f:131-258   9x9 Slater-Koster blocks per pair (k independent), for H,
//                      S and, in pressure mode, dH/dV and dS/dV.
//   setham.f, rotate.f:260-326, sethamv.f
//                      dense Hermitian H(k), S(k) (and dH, dS): one thread per
//                      matrix element and per k chunk, summing the few pairs of
//                      its atom block with Bloch phases e^{2 pi i k.(dlv - q_j + q_i)}.
#include <cfloat>
#include "setup.cuh"
#include "noncol_math.h"

namespace nrltb {

// ---- parameter index arithmetic (setpar.f:461, 567-578, 654-667, 852-856) ----
__host__ __device__ inline int ip_density(int kind) { return (kind - 1) * 17 + 1; }
__host__ __device__ inline int ip_hop(int kinds, int jk1, int jk2)
{
    int base = kinds * (1 + 4 * (3 * kinds + 1));
    if (jk1 == jk2) return base + 40 * (jk1 - 1);
    return base + 40 * kinds + 56 * ((jk2 - 1) * (jk2 - 2) / 2 + jk1 - 1);
}
__host__ __device__ inline int ip_over(int kinds, int jk1, int jk2)
{
    int base = kinds * (1 + 4 * (3 * kinds + 1));
    if (jk1 == jk2) return base + 40 * kinds + 56 * (kinds * (kinds - 1) / 2) + 40 * (jk1 - 1);
    return base + 80 * kinds + 56 * (kinds * (kinds - 1) / 2) + 56 * ((jk2 - 1) * (jk2 - 2) / 2 + jk1 - 1);
}
__host__ __device__ inline int ip_cross_onsite(int kinds, int jk1, int jk2)
{
    int jkx = jk1 > jk2 ? jk1 : jk2, jkm = jk1 < jk2 ? jk1 : jk2;
    int ip = kinds * 17 + 24 * ((jkx - 1) * (jkx - 2) / 2 + jkm - 1);
    if (jk2 < jkx) ip += 12;
    return ip;
}
__host__ __device__ inline int interaction_type(int kinds, int k1, int k2)
{
    if (k1 == k2) return k1;
    int jk1 = k1 < k2 ? k1 : k2, jk2 = k1 < k2 ? k2 : k1;
    return kinds + (jk2 - 1) * (jk2 - 2) / 2 + jk1;
}
__constant__ double c_ovlnull[10] = {1, 0, 1, 1, 0, 0, 0, 1, 1, 1};
__constant__ double c_harsign[9] = {-1, 1, 1, -1, -1, -1, 1, -1, 1};

// ---------------------------------------------------------------------------
// search2: candidate evaluation.  code: 0 sets kneigh=0, 1 sets kneigh=1 (kept),
// 2 rejected (beyond cutoff or jat < iat), 3 exact tie dd == dnnsq (kneigh kept).
__device__ inline void candidate(const DevStructure &S, const DevParams &P, long c, int &iat, int &jat,
                                 int im[3], double T[3], double &dsq, int &t)
{
    const int box = (2 * S.nd[0] + 1) * (2 * S.nd[1] + 1) * (2 * S.nd[2] + 1);
    const long ap = c / box;
    int img = (int)(c - ap * box);
    iat = (int)(ap / S.natoms);
    jat = (int)(ap - (long)iat * S.natoms);
    const int kz = 2 * S.nd[2] + 1, ky = 2 * S.nd[1] + 1;
    int iz = img % kz, iy = (img / kz) % ky, ix = img / (kz * ky);
    im[0] = ix - S.nd[0]; im[1] = iy - S.nd[1]; im[2] = iz - S.nd[2];
    dsq = 0.0;
    for (int i = 0; i < 3; ++i) {
        double rlv = 0.0;
        for (int j = 0; j < 3; ++j) rlv = __dadd_rn(rlv, __dmul_rn(S.plv[j][i], (double)im[j]));
        T[i] = __dsub_rn(__dadd_rn(S.posn[3 * jat + i], rlv), S.posn[3 * iat + i]);
        dsq = __dadd_rn(dsq, __dmul_rn(T[i], T[i]));
    }
    t = interaction_type(P.kinds, S.kkind[iat], S.kkind[jat]) - 1;
}

__global__ void k_search_eval(DevStructure S, DevParams P, long ncand, unsigned char *code, int *tie_count,
                              unsigned long long *dismin_bits)
{
    const double eps = 1e-3;
    unsigned long long best = 0x7FF0000000000000ull;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < ncand; c += (long)gridDim.x * blockDim.x) {
        int iat, jat, im[3], t;
        double T[3], dsq;
        candidate(S, P, c, iat, jat, im, T, dsq, t);
        unsigned char cd = 2;
        if (jat >= iat) {
            const double dnnsq = __dmul_rn(P.dnn[t], P.dnn[t]);
            const double dd = __dsub_rn(dsq, eps);
            if (dd > dnnsq) cd = 2;
            else if (dd < eps) cd = 0;
            else if (dd < dnnsq) cd = 1;
            else { cd = 3; atomicAdd(tie_count, 1); }
            if (dd > eps) {
                unsigned long long bits = (unsigned long long)__double_as_longlong(dsq);
                best = bits < best ? bits : best;
            }
        }
        code[c] = cd;
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
        best = other < best ? other : best;
    }
    if ((threadIdx.x & 31) == 0) atomicMin(dismin_bits, best);
}

// Ties (dd == dnnsq exactly) take search2's carried kneigh flag: resolved in
// candidate order by one thread, only when any tie exists.  Also returns the
// final flag.
__global__ void k_search_ties(unsigned char *code, long ncand, int kneigh_in, int *kneigh_out, int resolve)
{
    if (threadIdx.x || blockIdx.x) return;
    int kn = kneigh_in;
    if (resolve) {
        for (long c = 0; c < ncand; ++c) {
            unsigned char cd = code[c];
            if (cd == 0) kn = 0;
            else if (cd == 1) kn = 1;
            else if (cd == 3) code[c] = kn ? 1 : 2;
        }
    } else {
        for (long c = ncand - 1; c >= 0; --c) {
            unsigned char cd = code[c];
            if (cd == 0 || cd == 1) { kn = cd; break; }
        }
    }
    *kneigh_out = kn;
}

// Order-preserving compaction: per-block counts, scan, scatter.
constexpr int SCAN_BLOCK = 1024;
__global__ void k_search_count(const unsigned char *code, long ncand, int *blockcnt)
{
    __shared__ int red[32];
    long base = (long)blockIdx.x * SCAN_BLOCK;
    int v = 0;
    long c = base + threadIdx.x;
    if (c < ncand) v = (code[c] == 1);
    int s = block_sum(v, red);
    if (threadIdx.x == 0) blockcnt[blockIdx.x] = s;
}

__global__ void k_scan_small(int *cnt, int nblk, int *total)
{
    // exclusive scan of up to a few hundred thousand block counts by one CTA
    __shared__ int sums[1024];
    const int per = (nblk + 1023) / 1024;
    const int t = threadIdx.x;
    int s = 0;
    for (int q = 0; q < per; ++q) { int i = t * per + q; if (i < nblk) s += cnt[i]; }
    sums[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        int v = (t >= o) ? sums[t - o] : 0;
        __syncthreads();
        sums[t] += v;
        __syncthreads();
    }
    int run = (t > 0) ? sums[t - 1] : 0;
    for (int q = 0; q < per; ++q) {
        int i = t * per + q;
        if (i < nblk) { int v = cnt[i]; cnt[i] = run; run += v; }
    }
    if (t == 1023) *total = sums[1023];
}

__global__ void k_search_scatter(DevStructure S, DevParams P, const unsigned char *code, long ncand,
                                 const int *blockoff, DevPairs out, int capacity)
{
    __shared__ int wsum[32];
    const long c = (long)blockIdx.x * SCAN_BLOCK + threadIdx.x;
    const int keep = (c < ncand) ? (code[c] == 1) : 0;
    // block-exclusive scan of keep flags
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned m = __ballot_sync(0xffffffffu, keep);
    int pre = __popc(m & ((1u << lane) - 1));
    if (lane == 31) wsum[wid] = pre + keep;
    __syncthreads();
    if (wid == 0) {
        int v = wsum[lane];
        for (int o = 1; o < 32; o <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        wsum[lane] = v;
    }
    __syncthreads();
    if (!keep) return;
    const int pos = blockoff[blockIdx.x] + (wid ? wsum[wid - 1] : 0) + pre;
    if (pos >= capacity) return;
    int iat, jat, im[3], t;
    double T[3], dsq;
    candidate(S, P, c, iat, jat, im, T, dsq, t);
    const double scrninv = 1.0 / P.screenl[t];
    const double screenr = P.dnn[t] - 5.0 * P.screenl[t];
    const double dist = sqrt(dsq), tinv = 1.0 / dist;
    const double expdl = exp((dist - screenr) * scrninv);
    const double screen = 1.0 / (expdl + 1.0);
    for (int j = 0; j < 3; ++j) {
        out.tt[3 * (long)pos + j] = __dmul_rn(T[j], tinv);
        out.dlv[3 * (long)pos + j] = im[j];
    }
    out.dist[pos] = dist;
    out.screen[pos] = screen;
    out.dscrn[pos] = -expdl * screen * scrninv;
    out.jkind[2 * (long)pos] = S.kkind[iat];
    out.jkind[2 * (long)pos + 1] = S.kkind[jat];
    out.jatm[2 * (long)pos] = iat + 1;
    out.jatm[2 * (long)pos + 1] = jat + 1;
}

// ---------------------------------------------------------------------------
// setpar / setparv, per pair: hop, over (and dhop, dover); the density terms of
// both atoms are stored per pair and summed per atom afterwards.
__global__ void k_setpar_pairs(DevStructure S, DevParams P, DevPairs pr, int npairs, DevSK sk, int deriv)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const double *Pm = P.param - 1;
    const int realov = (P.nltype == 1 || P.nltype == 3), harrison = (P.nltype == 2 || P.nltype == 3);
    const int k1 = pr.jkind[2 * p], k2 = pr.jkind[2 * p + 1];
    const double dist = pr.dist[p], scr = pr.screen[p], dsc = pr.dscrn[p];
    const double vdist = (1.0 / 3.0) * dist / S.volume;
    // density contributions (setpar.f:500-536, setparv.f:510-535); the
    // receiving atom's spin picks the parameter set
    const double *Pi = atom_params(S, P, pr.jatm[2 * p] - 1), *Pj = atom_params(S, P, pr.jatm[2 * p + 1] - 1);
    double b2 = Pi[ip_density(k2)] * Pi[ip_density(k2)];
    double dent = exp(-b2 * dist) * scr;
    sk.dent[2 * (long)p] = dent;
    sk.vdent[2 * (long)p] = (dsc - b2) * dent * vdist;
    double b1 = Pj[ip_density(k1)] * Pj[ip_density(k1)];
    double dent1 = exp(-b1 * dist) * scr;
    sk.dent[2 * (long)p + 1] = dent1;
    sk.vdent[2 * (long)p + 1] = (dsc - b1) * dent1 * vdist;
    const int jk1 = k1 < k2 ? k1 : k2, jk2 = k1 < k2 ? k2 : k1;
    const int npk = (jk1 == jk2) ? 10 : 14;
    double h[14], o[14], dh[14], dov[14];
    for (int j = 0; j < 14; ++j) { h[j] = 0; o[j] = 0; dh[j] = 0; dov[j] = 0; }
    const int ip = ip_hop(P.kinds, jk1, jk2);
    const bool like = (jk1 == jk2);
    if (P.nltype != 90000) {
        for (int j = 1; j <= npk; ++j) {
            double abr = Pm[ip + 4 * j - 3] + dist * (Pm[ip + 4 * j - 2] + dist * Pm[ip + 4 * j - 1]);
            double p32m = -(Pm[ip + 4 * j] * Pm[ip + 4 * j]);
            double ex = exp(p32m * dist);
            double par21 = abr * ex * scr;
            h[j - 1] = par21;
            dh[j - 1] = vdist * (((Pm[ip + 4 * j - 2] + 2.0 * dist * Pm[ip + 4 * j - 1]) + p32m * abr) * ex * scr + dsc * par21);
            if (harrison && like && j < npk) dh[j - 1] = c_harsign[j - 1] * dh[j - 1] * (abr >= 0 ? 1.0 : -1.0);
        }
        if (harrison && like)
            for (int j = 0; j < 9; ++j) h[j] = c_harsign[j] * fabs(h[j]);
    } else {
        const int j = 1;
        double abr = Pm[ip + 4 * j - 3] + dist * (Pm[ip + 4 * j - 2] + dist * (Pm[ip + 4 * j - 1] +
                     dist * (Pm[ip + 4 * j + 1] + dist * Pm[ip + 4 * j + 2])));
        double p32m = -(Pm[ip + 4 * j] * Pm[ip + 4 * j]);
        double ex = exp(p32m * dist);
        h[0] = abr * ex * scr;
        dh[0] = vdist * (((Pm[ip + 4 * j - 2] + dist * (2.0 * Pm[ip + 4 * j - 1] + dist * (3.0 * Pm[ip + 4 * j + 1] +
                 dist * (4.0 * Pm[ip + 4 * j + 2])))) + p32m * abr) * ex * scr + dsc * h[0]);
    }
    if (P.jsover) {
        const int usenew = realov && like;
        const int iop = ip_over(P.kinds, jk1, jk2);
        if (P.nltype != 90000) {
            for (int j = 1; j <= npk; ++j) {
                double abr = Pm[iop + 4 * j - 3] + dist * (Pm[iop + 4 * j - 2] + dist * Pm[iop + 4 * j - 1]);
                double p32m = -(Pm[iop + 4 * j] * Pm[iop + 4 * j]);
                if (usenew) abr = c_ovlnull[j - 1] + dist * abr;
                o[j - 1] = abr * exp(p32m * dist) * scr;
            }
            if (harrison && like)
                for (int j = 0; j < 9; ++j) o[j] = -c_harsign[j] * fabs(o[j]);
        } else {
            const int j = 1;
            double abr = Pm[iop + 4 * j - 3] + dist * (Pm[iop + 4 * j - 2] + dist * (Pm[iop + 4 * j - 1] +
                         dist * (Pm[iop + 4 * j + 1] + dist * Pm[iop + 4 * j + 2])));
            double p32m = -(Pm[iop + 4 * j] * Pm[iop + 4 * j]);
            o[0] = abr * exp(p32m * dist) * scr;
        }
        // dover: setparv.f:640 compares nltype with 9000, never true after input.f,
        // so the polynomial forms are always used
        for (int j = 1; j <= npk; ++j) {
            double abr, d1;
            double p32m = -(Pm[iop + 4 * j] * Pm[iop + 4 * j]);
            if (usenew) {
                abr = c_ovlnull[j - 1] + dist * (Pm[iop + 4 * j - 3] + dist * (Pm[iop + 4 * j - 2] + dist * Pm[iop + 4 * j - 1]));
                d1 = Pm[iop + 4 * j - 3] + 2.0 * dist * Pm[iop + 4 * j - 2] + 3.0 * dist * dist * Pm[iop + 4 * j - 1];
            } else {
                abr = Pm[iop + 4 * j - 3] + dist * (Pm[iop + 4 * j - 2] + dist * Pm[iop + 4 * j - 1]);
                d1 = Pm[iop + 4 * j - 2] + 2.0 * dist * Pm[iop + 4 * j - 1];
            }
            double ex = exp(p32m * dist);
            double ovl21 = abr * ex * scr;
            dov[j - 1] = vdist * ((d1 + p32m * abr) * ex * scr + dsc * ovl21);
            if (harrison && like && j < npk) dov[j - 1] = -c_harsign[j - 1] * dov[j - 1] * (abr >= 0 ? 1.0 : -1.0);
        }
    }
    for (int j = 0; j < 14; ++j) {
        sk.hop[14 * (long)p + j] = h[j];
        sk.over[14 * (long)p + j] = o[j];
        if (deriv) { sk.dhop[14 * (long)p + j] = dh[j]; sk.dover[14 * (long)p + j] = dov[j]; }
    }
}

// Per-atom densities in pair order, then the on-site polynomials (setpar.f:735-884)
// and their volume derivatives (setparv.f:730-886).  One warp per atom: the
// lanes scan 32 pairs at a time and the matching pairs are added in pair order
// (the reference's summation order), every lane keeping the same sums.
__global__ void k_setpar_atoms(DevStructure S, DevParams P, DevPairs pr, int npairs, DevSK sk, int deriv)
{
    const int a = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (a >= S.natoms) return;   // warp-uniform
    const int kinds = P.kinds;
    double den[NRLTB_MAX_KINDS], vden[NRLTB_MAX_KINDS];
    for (int k = 0; k < kinds; ++k) { den[k] = 0; vden[k] = 0; }
    for (int p0 = 0; p0 < npairs; p0 += 32) {
        const int p = p0 + lane;
        int iat = -1, jat = -1, kk = 0;
        double d1 = 0, v1 = 0;
        bool m1 = false, m2 = false;
        if (p < npairs) {
            iat = pr.jatm[2 * p] - 1;
            jat = pr.jatm[2 * p + 1] - 1;
            m1 = iat == a;
            m2 = jat == a && iat != a;
            if (m1) { kk = pr.jkind[2 * p + 1]; d1 = sk.dent[2 * (long)p]; v1 = sk.vdent[2 * (long)p]; }
            else if (m2) { kk = pr.jkind[2 * p]; d1 = sk.dent[2 * (long)p + 1]; v1 = sk.vdent[2 * (long)p + 1]; }
        }
        unsigned hits = __ballot_sync(0xffffffffu, m1 || m2);
        while (hits) {   // in pair order
            const int l = __ffs(hits) - 1;
            hits &= hits - 1;
            const int k = __shfl_sync(0xffffffffu, kk, l);
            const double d = __shfl_sync(0xffffffffu, d1, l), v = __shfl_sync(0xffffffffu, v1, l);
            den[k - 1] += d;
            vden[k - 1] += v;
        }
    }
    if (lane != 0) return;
    const double *Pm = atom_params(S, P, a);   // on-site terms from the atom's own spin set
    const int jk1 = S.kkind[a];
    for (int k = 0; k < kinds; ++k) sk.den[(long)a * kinds + k] = den[k];
    if (deriv)
        for (int k = 0; k < kinds; ++k) sk.vden[(long)a * kinds + k] = vden[k];
    double paros[4], dparos[4];
    {
        int ip = ip_density(jk1);
        double vm23 = pow(den[jk1 - 1], 2.0 / 3.0);
        for (int k = 0; k < 4; ++k) {
            paros[k] = Pm[ip + 1] + vm23 * (Pm[ip + 2] + vm23 * (Pm[ip + 3] + vm23 * Pm[ip + 4]));
            ip += 4;
        }
        for (int jk2 = 1; jk2 <= kinds; ++jk2) {
            double d = den[jk2 - 1];
            if (jk2 == jk1 || d == 0.0) continue;
            vm23 = pow(d, 2.0 / 3.0);
            ip = ip_cross_onsite(kinds, jk1, jk2);
            for (int k = 0; k < 4; ++k) {
                paros[k] = paros[k] + vm23 * (Pm[ip + 1] + vm23 * (Pm[ip + 2] + vm23 * Pm[ip + 3]));
                ip += 3;
            }
        }
    }
    if (deriv) {
        int ip = ip_density(jk1);
        double vm13 = pow(den[jk1 - 1], 1.0 / 3.0);
        double vm23 = vm13 * vm13, vm2t = 2.0 * vm23, vm3t = 1.5 * vm23;
        double drho = (2.0 / 3.0) * vden[jk1 - 1] / vm13;
        for (int k = 0; k < 4; ++k) {
            dparos[k] = drho * (Pm[ip + 2] + vm2t * (Pm[ip + 3] + vm3t * Pm[ip + 4]));
            ip += 4;
        }
        for (int jk2 = 1; jk2 <= kinds; ++jk2) {
            double d = den[jk2 - 1];
            if (jk2 == jk1 || d == 0.0) continue;
            vm13 = pow(d, 1.0 / 3.0);
            vm23 = vm13 * vm13; vm2t = 2.0 * vm23; vm3t = 1.5 * vm23;
            drho = (2.0 / 3.0) * vden[jk2 - 1] / vm13;
            ip = ip_cross_onsite(kinds, jk1, jk2);
            for (int k = 0; k < 4; ++k) {
                dparos[k] = dparos[k] + drho * (Pm[ip + 1] + vm2t * (Pm[ip + 2] + vm3t * Pm[ip + 3]));
                ip += 3;
            }
        }
    }
    for (int k = 0; k < 4; ++k) {
        sk.paros[4 * (long)a + k] = paros[k];
        if (deriv) sk.dparos[4 * (long)a + k] = dparos[k];
    }
}

// ---------------------------------------------------------------------------
// Slater-Koster 9x9 blocks (rotate.f:131-258) for every pair, k independent.
__device__ void sk_params(const double *v, int k1, int k2, double p[14])
{
    for (int j = 0; j < 14; ++j) p[j] = v[j];
    if (k1 == k2) {
        p[10] = -v[1]; p[11] = v[4]; p[12] = -v[5]; p[13] = -v[6];
    } else if (k1 > k2) {   // setham.f:329-344: the mirrored parameter slot
        p[1] = -v[10]; p[4] = v[11]; p[5] = -v[12]; p[6] = -v[13];
        p[10] = -v[1]; p[11] = v[4]; p[12] = -v[5]; p[13] = -v[6];
    }
}

__device__ void sk_table(double l, double m, double n, const double p[14], int unlike, double *e /*[81] e[i*9+j]*/)
{
    const double rt3 = 1.732050807568877, half = 0.5;
    const double rt3h = half * rt3, rt3q = half * rt3h, rt32 = 2.0 * rt3;
    const double parity[9] = {1, -1, -1, -1, 1, 1, 1, 1, 1};
    const double ll = l * l, mm = m * m, nn = n * n, lm = l * m, mn = m * n, nl = n * l, lmn = lm * n;
    const double P1 = p[0], P2 = p[1], P3 = p[2], P4 = p[3], P5 = p[4], P6 = p[5], P7 = p[6], P8 = p[7], P9 = p[8], P10 = p[9];
#define E(i, j) e[(i) * 9 + (j)]
    E(0, 0) = P1;
    E(0, 1) = l * P2; E(0, 2) = m * P2; E(0, 3) = n * P2;
    const double rp5 = rt3 * P5;
    E(0, 4) = mn * rp5; E(0, 5) = nl * rp5; E(0, 6) = lm * rp5;
    E(0, 7) = half * rp5 * (ll - mm);
    E(0, 8) = (nn - half * (ll + mm)) * P5;
    const double p34 = P3 - P4;
    E(1, 1) = P4 + ll * p34; E(2, 2) = P4 + mm * p34; E(3, 3) = P4 + nn * p34;
    E(1, 2) = lm * p34; E(1, 3) = nl * p34; E(2, 3) = mn * p34;
    const double p67 = rt3 * P6 - 2.0 * P7;
    E(1, 4) = lmn * p67;
    E(1, 5) = n * (ll * p67 + P7);
    E(1, 6) = m * (ll * p67 + P7);
    E(2, 4) = n * (mm * p67 + P7);
    E(2, 5) = E(1, 4);
    E(2, 6) = l * (mm * p67 + P7);
    E(3, 4) = m * (nn * p67 + P7);
    E(3, 5) = l * (nn * p67 + P7);
    E(3, 6) = E(1, 4);
    E(1, 7) = l * (half * (ll - mm) * p67 + P7);
    const double p67a = P6 - rt3 * P7;
    E(1, 8) = l * (nn * p67a - (half * (ll + mm)) * P6);
    E(2, 7) = m * (half * (ll - mm) * p67 - P7);
    E(2, 8) = m * (nn * p67a - (half * (ll + mm)) * P6);
    E(3, 7) = n * (half * (ll - mm) * p67);
    E(3, 8) = n * (nn * P6 - half * (ll + mm) * (P6 - rt32 * P7));
    const double p8910 = (3.0 * P8 + P10) - 4.0 * P9;
    E(4, 4) = ll * P10 + mm * (nn * p8910) + (mm + nn) * P9;
    const double p910m = P9 - P10;
    E(4, 5) = lm * (p910m + nn * p8910);
    E(4, 6) = nl * (p910m + mm * p8910);
    E(5, 5) = mm * P10 + ll * (nn * p8910) + (ll + nn) * P9;
    E(5, 6) = mn * (p910m + ll * p8910);
    E(6, 6) = nn * P10 + ll * (mm * p8910) + (ll + mm) * P9;
    E(4, 7) = mn * ((half * (ll - mm)) * p8910 - p910m);
    E(5, 7) = nl * ((half * (ll - mm)) * p8910 + p910m);
    E(6, 7) = lm * (half * (ll - mm)) * p8910;
    const double p89 = P8 - 2.0 * P9, p8910a = p89 + P10, p8910b = p8910a + p89, p89m = P8 - P9;
    E(4, 8) = rt3 * mn * (nn * p89m - (half * (ll + mm)) * p8910a);
    E(5, 8) = rt3 * nl * (nn * p89m - (half * (ll + mm)) * p8910a);
    E(6, 8) = rt3h * lm * (P10 - (ll + mm) * P8 + nn * p8910b);
    E(7, 7) = (ll + mm) * P9 + nn * P10 + ((half * (ll - mm)) * (half * (ll - mm))) * p8910;
    E(7, 8) = rt3q * (ll - mm) * (P10 - (ll + mm) * P8 + nn * p8910b);
    E(8, 8) = nn * nn * P8 + (ll + mm) * (0.25 * (ll + mm) * (3.0 * P10 + P8) - nn * (P8 - 3.0 * P9));
    for (int i = 1; i < 9; ++i)
        for (int j = 0; j < i; ++j) E(i, j) = parity[i] * (E(j, i) * parity[j]);
    if (unlike) {
        const double P11 = p[10], P12 = p[11], P13 = p[12], P14 = p[13];
        E(1, 0) = l * P11; E(2, 0) = m * P11; E(3, 0) = n * P11;
        const double rp12 = rt3 * P12;
        E(4, 0) = mn * rp12; E(5, 0) = nl * rp12; E(6, 0) = lm * rp12;
        E(7, 0) = half * rp12 * (ll - mm);
        E(8, 0) = (nn - half * (ll + mm)) * P12;
        const double p134 = rt3 * P13 - 2.0 * P14;
        E(4, 1) = lmn * p134;
        E(5, 1) = n * (ll * p134 + P14);
        E(6, 1) = m * (ll * p134 + P14);
        E(4, 2) = n * (mm * p134 + P14);
        E(5, 2) = E(4, 1);
        E(6, 2) = l * (mm * p134 + P14);
        E(4, 3) = m * (nn * p134 + P14);
        E(5, 3) = l * (nn * p134 + P14);
        E(6, 3) = E(4, 1);
        E(7, 1) = l * (half * (ll - mm) * p134 + P14);
        const double p134a = P13 - rt3 * P14;
        E(8, 1) = l * (nn * p134a - (half * (ll + mm)) * P13);
        E(7, 2) = m * (half * (ll - mm) * p134 - P14);
        E(8, 2) = m * (nn * p134a - (half * (ll + mm)) * P13);
        E(7, 3) = n * (half * (ll - mm) * p134);
        E(8, 3) = n * (nn * P13 - half * (ll + mm) * (P13 - rt32 * P14));
    }
#undef E
}

// which: 0 H, 1 S, 2 dH, 3 dS
__global__ void k_sk_blocks(DevPairs pr, int npairs, DevSK sk, int nwhich)
{
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= (long)npairs * nwhich) return;
    const int p = (int)(t % npairs), which = (int)(t / npairs);
    const double *src = which == 0 ? sk.hop : which == 1 ? sk.over : which == 2 ? sk.dhop : sk.dover;
    const int k1 = pr.jkind[2 * p], k2 = pr.jkind[2 * p + 1];
    double pv[14], e[81];
    sk_params(src + 14 * (long)p, k1, k2, pv);
    sk_table(pr.tt[3 * (long)p], pr.tt[3 * (long)p + 1], pr.tt[3 * (long)p + 2], pv, k1 != k2, e);
    double *dst = sk.E + ((long)which * npairs + p) * 81;
    for (int q = 0; q < 81; ++q) dst[q] = e[q];
}

// Atom-pair segments of the (iat, jat)-ordered pair list.
__global__ void k_segments(DevPairs pr, int npairs, int natoms, int2 *seg)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const int a = pr.jatm[2 * p] - 1, b = pr.jatm[2 * p + 1] - 1;
    const bool first = (p == 0) || pr.jatm[2 * p - 2] != pr.jatm[2 * p] || pr.jatm[2 * p - 1] != pr.jatm[2 * p + 1];
    const bool last = (p == npairs - 1) || pr.jatm[2 * p + 2] != pr.jatm[2 * p] || pr.jatm[2 * p + 3] != pr.jatm[2 * p + 1];
    if (first) seg[(long)a * natoms + b].x = p;
    if (last) seg[(long)a * natoms + b].y = p + 1;
}

// Bloch phases for a chunk of k points: ph[kk][p] = e^{2 pi i k.(dlv - q_j + q_i)}
__global__ void k_phases(DevStructure S, DevPairs pr, int npairs, const double *kq, int nk, double2 *ph)
{
    const double tpi = 6.283185307179586;
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= (long)npairs * nk) return;
    const int p = (int)(t % npairs), kk = (int)(t / npairs);
    const int a1 = pr.jatm[2 * p] - 1, a2 = pr.jatm[2 * p + 1] - 1;
    double q[3];
    for (int c = 0; c < 3; ++c)
        q[c] = (double)pr.dlv[3 * (long)p + c] - S.posq[3 * a2 + c] + S.posq[3 * a1 + c];
    const double dot = kq[3 * kk] * q[0] + kq[3 * kk + 1] * q[1] + kq[3 * kk + 2] * q[2];
    double sn, cs;
    sincos(tpi * dot, &sn, &cs);
    ph[(long)kk * npairs + p] = make_double2(cs, sn);
}

// Dense Hermitian matrices for a chunk of k points; `which0` selects H/S (0) or
// dH/dS (2).  Column-major, leading dimension nv.  One CTA per pair of 32 x 32
// tiles (R, C), R <= C: thread (row tr, column tc) forms elements (32 R + tr,
// 32 C + tc + 8 q), q < 4.  Element (r, c) is the sum over the images of its
// atom pair taken in the reference's upper storage (min-atom row, max-atom
// column) and conjugated when (r, c) is the lower one, so the two elements of
// a mirrored pair are conjugates of one sum: off the diagonal tiles each sum is
// formed once and its conjugate written to (c, r) through a shared-memory
// transpose (coalesced both ways), halving the FP64 work; diagonal tiles form
// every element.  The values are those of one thread per element.
__device__ __forceinline__ void bloch_elem(const DevStructure &S, const DevSK &sk, int npairs, const int2 *seg,
                                           const int *orb_atom, const int *ksk, int r, int c, int which0,
                                           int &a1, int &a2, int &oi, int &oj, bool &conjg, int2 &sg, double &on1,
                                           double &on2)
{
    const int ar = orb_atom[r], ac = orb_atom[c];
    const int i = r - ksk[ar], j = c - ksk[ac];
    // element (r, c): upper storage of the reference is (min-atom row, max-atom col)
    if (ar < ac || (ar == ac && i <= j)) { a1 = ar; a2 = ac; oi = i; oj = j; conjg = false; }
    else { a1 = ac; a2 = ar; oi = j; oj = i; conjg = true; }
    sg = seg[(long)a1 * S.natoms + a2];
    on1 = 0.0;
    on2 = 0.0;
    if (r == c) {
        const int cls = (i == 0) ? 0 : (i <= 3) ? 1 : (i <= 6) ? 2 : 3;
        on1 = (which0 == 0 ? sk.paros : sk.dparos)[4 * (long)ar + cls];
        on2 = (which0 == 0) ? 1.0 : 0.0;
    }
}

__global__ void __launch_bounds__(256)
k_bloch_build(DevStructure S, DevParams P, DevPairs pr, int npairs, DevSK sk, const int2 *seg,
              const int *orb_atom, const int *ksk, const double2 *ph, int nk, int nv, int which0,
              double2 *M1, double2 *M2, int jsover)
{
    __shared__ double2 t1[32][33], t2[32][33];   // [row in R][column in C]
    // tile pair of this CTA: blockIdx.x = C (C + 1) / 2 + R
    const int u = blockIdx.x;
    int C = (int)((sqrtf(8.f * u + 1.f) - 1.f) * 0.5f);
    while ((C + 1) * (C + 2) / 2 <= u) ++C;
    while (C * (C + 1) / 2 > u) --C;
    const int R = u - C * (C + 1) / 2;
    const bool diag = R == C;
    const int tr = threadIdx.x & 31, tc = threadIdx.x >> 5;
    const int r = 32 * R + tr;
    const double *E1 = sk.E + (long)which0 * npairs * 81;
    const double *E2 = sk.E + (long)(which0 + 1) * npairs * 81;
    int a1[4], a2[4], oi[4], oj[4];
    bool conjg[4], ok[4];
    int2 sg[4];
    double on1[4], on2[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int c = 32 * C + tc + 8 * q;
        ok[q] = r < nv && c < nv;
        if (ok[q]) bloch_elem(S, sk, npairs, seg, orb_atom, ksk, r, c, which0, a1[q], a2[q], oi[q], oj[q], conjg[q],
                              sg[q], on1[q], on2[q]);
    }
    for (int kk = 0; kk < nk; ++kk) {
        const double2 *phk = ph + (long)kk * npairs;
        double2 *m1 = M1 + (long)kk * nv * nv, *m2 = M2 + (long)kk * nv * nv;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (!ok[q]) continue;
            const int c = 32 * C + tc + 8 * q;
            double h_re = 0, h_im = 0, s_re = 0, s_im = 0;
            for (int p = sg[q].x; p < sg[q].y; ++p) {
                const double2 z = phk[p];
                const double e1 = E1[(long)p * 81 + oi[q] * 9 + oj[q]];
                h_re += e1 * z.x;
                h_im += e1 * z.y;
                if (jsover) {
                    const double e2 = E2[(long)p * 81 + oi[q] * 9 + oj[q]];
                    s_re += e2 * z.x;
                    s_im += e2 * z.y;
                }
            }
            h_re += on1[q];
            if (jsover) s_re += on2[q];
            else s_re = (r == c && which0 == 0) ? 1.0 : 0.0;
            if (conjg[q]) { h_im = -h_im; s_im = -s_im; }
            const long off = r + (long)c * nv;
            m1[off] = make_double2(h_re, h_im);
            m2[off] = make_double2(s_re, s_im);
            if (!diag) {
                t1[tr][tc + 8 * q] = make_double2(h_re, -h_im);
                t2[tr][tc + 8 * q] = make_double2(s_re, -s_im);
            }
        }
        if (!diag) {
            // (c, r) = conj (r, c): rows 32 C + tr, columns 32 R + tc + 8 q
            __syncthreads();
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int rr = 32 * C + tr, cc = 32 * R + tc + 8 * q;
                if (rr < nv && cc < nv) {
                    const long off = rr + (long)cc * nv;
                    m1[off] = t1[tc + 8 * q][tr];
                    m2[off] = t2[tc + 8 * q][tr];
                }
            }
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------------------
// Non-collinear spins.  One thread per atom: the on-site average and splitting
// of the two parameter sets (setpar.f:746-796, setparv.f:723-795); P1, P2 are
// the two sets (0-based pointers).
__global__ void k_noncol_onsite(int natoms, int kinds, const int *kkind, const double *den1, const double *den2,
                                const double *vden1, const double *vden2, const double *P1, const double *P2,
                                int deriv, double *paros, double *spinos, double *dparos, double *dspnos)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natoms) return;
    const long o = (long)a * kinds;
    nc_onsite_atom(kinds, kkind[a], den1 + o, den2 + o, vden1 + o, vden2 + o, P1 - 1, P2 - 1, deriv,
                   paros + 4 * (long)a, spinos + 4 * (long)a, dparos + 4 * (long)a, dspnos + 4 * (long)a);
}

// One thread per orbital: spinham.f's diagonal and mixing terms
__global__ void k_noncol_spin_terms(int nv, const int *orb_atom, const int *ksk, const double *spinos,
                                    const double *spinat, double *diag, double *mix_re, double *mix_im)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int a = orb_atom[i];
    nc_spin_terms(i - ksk[a], spinos + 4 * (long)a, spinat + 3 * (long)a, diag + i, mix_re + i, mix_im + i);
}

// One thread per element of the doubled matrices (addspins.f:77-110); Hn holds
// batch column-major N x N matrices, H2 receives the 2N x 2N ones.  diag = NULL
// doubles an overlap block-diagonally.
__global__ void k_noncol_expand(int nv, int batch, const double2 *Hn, const double *diag, const double *mix_re,
                                const double *mix_im, double2 *H2)
{
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const long n2 = 2L * nv, nn2 = n2 * n2, nn = (long)nv * nv;
    if (t >= nn2 * batch) return;
    const long b = t / nn2, e = t - b * nn2;
    const int r = (int)(e % n2), c = (int)(e / n2);
    const double *hb = (const double *)(Hn + b * nn);
    double re, im;
    nc_expand(nv, r, c, hb, hb + 1, 2, diag, mix_re, mix_im, &re, &im);
    H2[t] = make_double2(re, im);
}

}  // namespace nrltb
