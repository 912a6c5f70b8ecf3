// sums.cu -- Fermi level, band energy, pressure (fermi.f, bande.f sums) and the
// Hellmann-Feynman eigenvalue derivatives (perturb.f).
//
// k_fermi_sums: one CTA per structure.  The MPI_ALLREDUCE of every Newton step
// (fermi.f:365-376) and the final MPI_REDUCEs (bande.f:1255-1331) become block
// reductions; the iteration itself is the reference's: start at the middle of
// the band-nfill / nfill+1 edges, Newton steps clamped to the bracket, bisection
// when dN/dmu is small, stop when |N - zfill| < tol or the bracket closes.
// Occupations are exactly 1 below mu - 20 kT and 0 above mu + 20 kT.  With
// lentro (modes 1, 2) the same window also gives Gillan's entropy S(T) and its
// two volume-derivative sums (bande.f:1189-1242).
//
// Every sum (the occupation and its derivative in each Newton step, E(T), the
// pressure partials, the entropy terms, the spin populations) is compensated:
// each thread keeps a (sum, error) pair updated by Knuth's two-sum, and the
// block reduction merges the pairs in a fixed tree order, so the result is
// what an exact summation of the rounded terms would give to within a few
// units in the last place of the result, however much the terms cancel, and
// the same from run to run.
#include "sums.cuh"

namespace nrltb {

// compensated accumulator: the exact sum of the terms added is hi + lo up to
// the rounding of lo (Knuth's two-sum, no ordering assumption)
struct DD {
    double hi = 0.0, lo = 0.0;
    __device__ __forceinline__ void add(double b)
    {
        // _rn intrinsics: a term's product is never contracted into the sum
        const double s = __dadd_rn(hi, b), bp = __dsub_rn(s, hi);
        lo += __dadd_rn(__dsub_rn(hi, __dsub_rn(s, bp)), __dsub_rn(b, bp));
        hi = s;
    }
    __device__ __forceinline__ void merge(double bhi, double blo)
    {
        lo += blo;
        add(bhi);
    }
};

// block-wide compensated sum; every thread gets hi + lo of the total.  `sh`
// needs 2 * blockDim.x / 32 entries.
__device__ double block_sum_dd(DD v, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) {
        const double h = __shfl_xor_sync(0xffffffffu, v.hi, o), l = __shfl_xor_sync(0xffffffffu, v.lo, o);
        v.merge(h, l);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) { sh[wid] = v.hi; sh[32 + wid] = v.lo; }
    __syncthreads();
    if (wid == 0) {
        DD t;
        if (lane < nw) { t.hi = sh[lane]; t.lo = sh[32 + lane]; }
        for (int o = 16; o > 0; o >>= 1) {
            const double h = __shfl_xor_sync(0xffffffffu, t.hi, o), l = __shfl_xor_sync(0xffffffffu, t.lo, o);
            t.merge(h, l);
        }
        if (lane == 0) sh[0] = t.hi + t.lo;
    }
    __syncthreads();
    const double r = sh[0];
    __syncthreads();
    return r;
}

__device__ inline double block_sum_d(double v, double *sh) { return block_sum<double>(v, sh); }
__device__ inline double block_max_d(double v, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double t = (threadIdx.x < nw) ? sh[threadIdx.x] : -1e308;
    if (wid == 0) for (int o = 16; o > 0; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
    if (threadIdx.x == 0) sh[0] = t;
    __syncthreads();
    double r = sh[0];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(1024) k_fermi_sums(FermiJob *jobs)
{
    __shared__ double sh[64];
    FermiJob J = jobs[blockIdx.x];
    const int nv = J.nv, nk = J.nk, tid = threadIdx.x, nt = blockDim.x;
    const long tot = (long)nv * nk;
    const double el = J.el, nearz = 1e-5, tkb = J.tkb, zfill = J.zfill, tol = J.tol;
    const double beta = (tkb < nearz) ? 1.0 / nearz : 1.0 / tkb;
    const int nfill = (int)(zfill / el + nearz);
    const bool linst = fabs(zfill / el - (double)nfill) < tol;
    // bounds (fermi.f:197-261) from bands nfill and nfill+1; where those lie
    // outside the nv computed bands (nfill >= nv happens with one electron per
    // band) the reference reads past them: here the band indices are clamped
    // and the insulator shortcut is not taken, which moves only the start
    const int ilo = max(min(nfill, nv) - 1, 0), ihi = min(nfill, nv - 1);
    const bool inrange = nfill >= 1 && nfill < nv;
    double stl = -1e308, sth = 1e308, mul = 1e308, muh = -1e308;
    for (long q = tid; q < tot; q += nt) {
        const int k = (int)(q / nv), i = (int)(q % nv);
        const double e = J.eig[(long)k * J.ldk + i];
        if (i == ilo) stl = fmax(stl, e);
        if (i == ihi) sth = fmin(sth, e);
        muh = fmax(muh, e);
        mul = fmin(mul, e);
    }
    double stlow = block_max_d(stl, sh), sthigh = -block_max_d(-sth, sh);
    double muhigh = block_max_d(muh, sh), mulow = -block_max_d(-mul, sh);
    double mu;
    int it = 0;
    if (linst && inrange && (sthigh - stlow > 20.0 * tkb)) {
        mu = 0.5 * (stlow + sthigh);
    } else {
        mu = 0.5 * (stlow + sthigh);
        for (it = 1; it <= 10000; ++it) {
            const double mum20 = mu - tkb * 20.0, mup20 = mu + tkb * 20.0, btmu = -beta * mu;
            DD ns, dns;
            for (long q = tid; q < tot; q += nt) {
                const int k = (int)(q / nv), i = (int)(q % nv);
                const double e = J.eig[(long)k * J.ldk + i];
                const double wk = J.w[k];
                if (e < mum20) ns.add(wk);
                else if (e < mup20) {
                    const double ex = exp(beta * e + btmu);
                    const double f = 1.0 / (1.0 + ex);
                    ns.add(wk * f);
                    dns.add(wk * (ex * f * f));
                }
            }
            double nsum = el * block_sum_dd(ns, sh);
            double dnsum = beta * el * block_sum_dd(dns, sh);
            if (fabs(nsum - zfill) < tol) break;
            if (nsum < zfill) mulow = mu; else muhigh = mu;
            double mu1;
            if (dnsum < tol) mu1 = 0.5 * (mulow + muhigh);
            else {
                mu1 = mu + (zfill - nsum) / dnsum;
                if (mu1 > muhigh) mu1 = 0.5 * (mu + muhigh);
                else if (mu1 < mulow) mu1 = 0.5 * (mu + mulow);
            }
            if (muhigh - mulow > tol) mu = mu1;
            else break;
        }
    }
    // energy and pressure sums (bande.f:1162-1330)
    const double tkbi = (tkb < 1e-5) ? 1e5 : 1.0 / tkb;
    const double efp = mu + 20.0 * tkb, efm = mu - 20.0 * tkb;
    DD es, d1, d2, d3, dfb, dfe, ent, dn1, dn2, sup, sdn;
    for (long q = tid; q < tot; q += nt) {
        const int k = (int)(q / nv), i = (int)(q % nv);
        const double e = J.eig[(long)k * J.ldk + i];
        // spin populations over all nv states (bande.f:1336-1395), weight w(k)
        if (J.nks > 0 && e < efp) {
            const double occ = (e < efm) ? J.w[k] : J.w[k] * (1.0 / (1.0 + exp(tkbi * (e - mu))));
            if (k < J.nks) sup.add(occ);
            else sdn.add(occ);
        }
        const int lim = J.lpress ? J.ncut[k] : nv;
        if (i >= lim) continue;
        if (!(e < efp)) continue;
        const double wt = J.el * J.w[k], ewt = wt * e;
        const double de = J.lpress ? J.deig[(long)k * J.ldk + i] : 0.0;
        if (e < efm) {
            es.add(ewt);
            d1.add(wt * de);
        } else {
            const double x = e - mu;
            const double fbe = 1.0 / (1.0 + exp(tkbi * x));
            es.add(ewt * fbe);
            // Gillan entropy of the window states (bande.f:1233-1242, 1313)
            if (J.lentro) ent.add(-(wt * (fbe * log(fbe) + (1.0 - fbe) * log(1.0 - fbe))));
            if (J.lpress) {
                const double dfbe = -tkbi * fbe * (1.0 / (1.0 + exp(tkbi * (-x))));
                dfb.add(dfbe * wt);
                d3.add(dfbe * ewt);
                const double dewt = wt * de;
                d1.add(dewt * fbe);
                dfe.add(dfbe * dewt);
                d2.add(dfbe * ewt * de);
                if (J.lentro) {
                    const double con1 = dfbe * wt * x;
                    dn1.add(con1 * de);
                    dn2.add(con1);
                }
            }
        }
    }
    const double es_ = block_sum_dd(es, sh), d1_ = block_sum_dd(d1, sh), d2_ = block_sum_dd(d2, sh);
    const double d3_ = block_sum_dd(d3, sh), dfb_ = block_sum_dd(dfb, sh), dfe_ = block_sum_dd(dfe, sh);
    double ent_ = 0, dn1_ = 0, dn2_ = 0, sup_ = 0, sdn_ = 0;
    if (J.lentro) {
        ent_ = block_sum_dd(ent, sh);
        dn1_ = block_sum_dd(dn1, sh);
        dn2_ = block_sum_dd(dn2, sh);
    }
    if (J.nks > 0) {
        sup_ = block_sum_dd(sup, sh);
        sdn_ = block_sum_dd(sdn, sh);
    }
    if (tid == 0) {
        FermiOut o;
        o.efermi = mu;
        o.e_total = es_;
        o.fermi_shift = 0;
        o.pressure = 0;
        if (J.lpress) {
            const double dfermi = (fabs(dfb_) > 1e-10) ? dfe_ / dfb_ : 0.0;
            o.fermi_shift = dfermi;
            o.pressure = -(d1_ + (d2_ - dfermi * d3_));
        }
        o.entropy = ent_;
        o.dent1 = dn1_;
        o.dent2 = dn2_;
        o.spin_up = sup_;
        o.spin_dn = sdn_;
        o.iterations = it;
        o.pad = 0;
        J.out[0] = o;
    }
}

// One thread per (k, state, atom).  Z: batch column-major n2 x n2 eigenvectors
// (n2 = 2N, the up half first); ksk: first orbital of each atom.  The spin
// vector of diag.f:486-513 as written there: x = -2 Re(u* d), y = 2 Im(u* d),
// z = |d|^2 - |u|^2 summed over the atom's orbitals, without the overlap.
__global__ void k_spin_expect(const double2 *Z, int n2, int batch, int natoms, const int *ksk, double *spev)
{
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= (long)batch * n2 * natoms) return;
    const int a = (int)(t % natoms);
    const long q = t / natoms;
    const int ie = (int)(q % n2);
    const long b = q / n2;
    const int nh = n2 / 2, i0 = ksk[a], i1 = (a + 1 < natoms) ? ksk[a + 1] : nh;
    const double2 *z = Z + b * (long)n2 * n2 + (long)ie * n2;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int ib = i0; ib < i1; ++ib) {
        const double2 u = z[ib], d = z[ib + nh];
        const double re_ud = u.x * d.x + u.y * d.y, im_ud = u.x * d.y - u.y * d.x;   // conj(u) d
        const double re_du = d.x * u.x + d.y * u.y, im_du = d.x * u.y - d.y * u.x;   // conj(d) u
        sx = (sx - re_ud) - re_du;
        sy = sy + (im_ud - im_du);
        sz = (sz + (d.x * d.x + d.y * d.y)) - (u.x * u.x + u.y * u.y);
    }
    double *o = spev + 3 * t;
    o[0] = sx;
    o[1] = sy;
    o[2] = sz;
}

// One block per atom and component: the occupation-weighted sum over every
// row and state, weight el w(k) below E_F - 20 kT and el w(k) f inside the
// window (bande.f:1505-1516); E_F from the Fermi kernel's output
__global__ void __launch_bounds__(256) k_spin_dir_sum(const double *eig, const double *w, const double *spev,
                                                      const FermiOut *fo, double tkb, double el, int nrow, int n2,
                                                      int natoms, double *spdir)
{
    __shared__ double sh[32];
    const int j = blockIdx.x;   // 3 * atom + component
    const double mu = fo->efermi, tkbi = (tkb < 1e-5) ? 1e5 : 1.0 / tkb;
    const double efp = mu + 20.0 * tkb, efm = mu - 20.0 * tkb;
    double acc = 0.0;
    for (long q = threadIdx.x; q < (long)nrow * n2; q += blockDim.x) {
        const double e = eig[q];
        if (!(e < efp)) continue;
        const double wt = el * w[q / n2];
        double fbe = wt;
        if (e > efm) fbe = wt * (1.0 / (1.0 + exp(tkbi * (e - mu))));
        acc += fbe * spev[q * 3L * natoms + j];
    }
    acc = block_sum_d(acc, sh);
    if (threadIdx.x == 0) spdir[j] = acc;
}

// ncut[k] = number of eigenvalues <= eigcut (perturb.f:87-95)
__global__ void k_ncut(const double *eig, int ldk, int nv, int nk, double eigcut, int *ncut)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    int c = 0;
    while (c < nv && !(eig[(long)k * ldk + c] > eigcut)) ++c;
    ncut[k] = c;
}

// Hellmann-Feynman shifts from P = triu(dH) Z and Q = triu(dS) Z:
//   z^H M z = 2 Re(z^H triu(M) z) - sum_i M_ii |z_i|^2
//   deig_n = z_n^H dH z_n - e_n z_n^H dS z_n
// or, FULL, from the full products P = dH Z, Q = dS Z (deig_n = Re z_n^H P_n -
// e_n Re z_n^H Q_n).  One warp per (column n, matrix).
template <typename C2, bool FULL = false>
__global__ void k_hf_dots(const C2 *Z, const C2 *Pm, const C2 *Qm, const double2 *dH, const double2 *dS,
                          const double *eig, double *deig, int n, int batch)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n * batch) return;
    const int b = warp / n, col = warp % n;
    const long off = (long)b * n * n + (long)col * n;
    double sp = 0, sq = 0, dh = 0, ds = 0;
    for (int i = lane; i < n; i += 32) {
        const C2 z = Z[off + i], p = Pm[off + i], q = Qm[off + i];
        sp += (double)z.x * p.x + (double)z.y * p.y;
        sq += (double)z.x * q.x + (double)z.y * q.y;
        if (!FULL) {
            const double a2 = (double)z.x * z.x + (double)z.y * z.y;
            dh += dH[(long)b * n * n + (long)i * (n + 1)].x * a2;
            ds += dS[(long)b * n * n + (long)i * (n + 1)].x * a2;
        }
    }
    sp = warp_sum(sp); sq = warp_sum(sq);
    if (!FULL) { dh = warp_sum(dh); ds = warp_sum(ds); }
    if (lane == 0) {
        const double e = eig[(long)b * n + col];
        deig[(long)b * n + col] = FULL ? sp - e * sq : (2.0 * sp - dh) - e * (2.0 * sq - ds);
    }
}

void launch_hf_dots(cudaStream_t s, const double2 *Z, const double2 *P, const double2 *Q, const double2 *dH,
                    const double2 *dS, const double *eig, double *deig, int n, int batch)
{
    const long warps = (long)n * batch;
    NRLTB_LAUNCH(k_hf_dots<double2>, cdiv(warps * 32, 256), 256, 0, s, Z, P, Q, dH, dS, eig, deig, n, batch);
}

void launch_hf_dots_full(cudaStream_t s, const double2 *Z, const double2 *P, const double2 *Q, const double *eig,
                         double *deig, int n, int batch)
{
    const long warps = (long)n * batch;
    NRLTB_LAUNCH((k_hf_dots<double2, true>), cdiv(warps * 32, 256), 256, 0, s, Z, P, Q, nullptr, nullptr, eig,
                 deig, n, batch);
}

}  // namespace nrltb
