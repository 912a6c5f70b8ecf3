// sums.cu -- Fermi level, band energy, pressure (fermi.f, bande.f sums) and the
// Hellmann-Feynman eigenvalue derivatives (perturb.f).
//
// launch_fermi_sums: k_fermi_level finds E_F in one CTA, k_band_sums and
// k_band_finish form the sums over the whole GPU.  The MPI_ALLREDUCE of every
// Newton step (fermi.f:365-376) and the final MPI_REDUCEs (bande.f:1255-1331)
// become block and grid reductions; the iteration itself is the reference's: start at the middle of
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

// number of entries of the ascending row e[0..m) below x
__device__ __forceinline__ int count_below(const double *e, int m, double x)
{
    int lo = 0, hi = m;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (e[mid] < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// E_F (fermi.f:162-425).  When every row is ascending (the eigensolver's
// output always is) the band edges are row ends and each Newton step's
// occupation needs only the states inside the +-20 kT window: a row's fully
// occupied states below it are counted by a binary search (their w_k add up
// to count x w_k), a warp per row takes the window.  Rows that are not
// ascending (caller eigenvalues) fall back to a scan of every state.
__global__ void __launch_bounds__(1024) k_fermi_level(FermiJob *jobs)
{
    __shared__ double sh[64];
    __shared__ int s_sorted;
    FermiJob J = jobs[blockIdx.x];
    const int nv = J.nv, nk = J.nk, tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = nt >> 5;
    const long tot = (long)nv * nk;
    const double el = J.el, nearz = 1e-5, tkb = J.tkb, zfill = J.zfill, tol = J.tol;
    const double beta = (tkb < nearz) ? 1.0 / nearz : 1.0 / tkb;
    const int nfill = (int)(zfill / el + nearz);
    const bool linst = fabs(zfill / el - (double)nfill) < tol;
    if (tid == 0) s_sorted = 1;
    __syncthreads();
    {
        int uns = 0;
        for (int k = warp; k < nk; k += nwarps) {   // a warp per row
            const double *e = J.eig + (long)k * J.ldk;
            for (int i = lane; i + 1 < nv; i += 32)
                if (e[i + 1] < e[i]) uns = 1;
        }
        if (__syncthreads_or(uns) && tid == 0) s_sorted = 0;
        __syncthreads();
    }
    const bool sorted = s_sorted != 0;
    // bounds (fermi.f:197-261) from bands nfill and nfill+1; where those lie
    // outside the nv computed bands (nfill >= nv happens with one electron per
    // band) the reference reads past them: here the band indices are clamped
    // and the insulator shortcut is not taken, which moves only the start
    const int ilo = max(min(nfill, nv) - 1, 0), ihi = min(nfill, nv - 1);
    const bool inrange = nfill >= 1 && nfill < nv;
    double stl = -1e308, sth = 1e308, mul = 1e308, muh = -1e308;
    if (sorted) {
        for (int k = tid; k < nk; k += nt) {
            const double *e = J.eig + (long)k * J.ldk;
            stl = fmax(stl, e[ilo]);
            sth = fmin(sth, e[ihi]);
            muh = fmax(muh, e[nv - 1]);
            mul = fmin(mul, e[0]);
        }
    } else {
        for (long q = tid; q < tot; q += nt) {
            const int k = (int)(q / nv), i = (int)(q % nv);
            const double e = J.eig[(long)k * J.ldk + i];
            if (i == ilo) stl = fmax(stl, e);
            if (i == ihi) sth = fmin(sth, e);
            muh = fmax(muh, e);
            mul = fmin(mul, e);
        }
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
            if (sorted) {
                for (int k = warp; k < nk; k += nwarps) {
                    const double *e = J.eig + (long)k * J.ldk;
                    const double wk = J.w[k];
                    const int lo = count_below(e, nv, mum20), hi = count_below(e, nv, mup20);
                    if (lane == 0) ns.add(wk * (double)lo);
                    for (int i = lo + lane; i < hi; i += 32) {
                        const double ex = exp(beta * e[i] + btmu);
                        const double f = 1.0 / (1.0 + ex);
                        ns.add(wk * f);
                        dns.add(wk * (ex * f * f));
                    }
                }
            } else {
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
    if (tid == 0) {
        J.out->efermi = mu;
        J.out->iterations = it;
    }
}

// The sums after E_F (bande.f:1162-1330), spread over the GPU: each CTA
// forms compensated partial sums over a stride of the states and stores
// them (hi, lo) in part[blockIdx.x][2 x FERMI_NSUM]; k_band_finish merges the
// CTAs' partials in CTA order.
constexpr int FERMI_NSUM = 11;
__global__ void __launch_bounds__(256) k_band_sums(FermiJob *jobs, double *part)
{
    __shared__ double sh[64];
    FermiJob J = jobs[0];
    const int nv = J.nv, nk = J.nk, tid = threadIdx.x;
    const long tot = (long)nv * nk, stride = (long)gridDim.x * blockDim.x;
    const double tkb = J.tkb, mu = J.out->efermi;
    const double tkbi = (tkb < 1e-5) ? 1e5 : 1.0 / tkb;
    const double efp = mu + 20.0 * tkb, efm = mu - 20.0 * tkb;
    DD acc[FERMI_NSUM];   // es, d1, d2, d3, dfb, dfe, ent, dn1, dn2, sup, sdn
    for (long q = blockIdx.x * (long)blockDim.x + tid; q < tot; q += stride) {
        const int k = (int)(q / nv), i = (int)(q % nv);
        const double e = J.eig[(long)k * J.ldk + i];
        // spin populations over all nv states (bande.f:1336-1395), weight w(k)
        if (J.nks > 0 && e < efp) {
            const double occ = (e < efm) ? J.w[k] : J.w[k] * (1.0 / (1.0 + exp(tkbi * (e - mu))));
            if (k < J.nks) acc[9].add(occ);
            else acc[10].add(occ);
        }
        const int lim = J.lpress ? J.ncut[k] : nv;
        if (i >= lim) continue;
        if (!(e < efp)) continue;
        const double wt = J.el * J.w[k], ewt = wt * e;
        const double de = J.lpress ? J.deig[(long)k * J.ldk + i] : 0.0;
        if (e < efm) {
            acc[0].add(ewt);
            acc[1].add(wt * de);
        } else {
            const double x = e - mu;
            const double fbe = 1.0 / (1.0 + exp(tkbi * x));
            acc[0].add(ewt * fbe);
            // Gillan entropy of the window states (bande.f:1233-1242, 1313)
            if (J.lentro) acc[6].add(-(wt * (fbe * log(fbe) + (1.0 - fbe) * log(1.0 - fbe))));
            if (J.lpress) {
                const double dfbe = -tkbi * fbe * (1.0 / (1.0 + exp(tkbi * (-x))));
                acc[4].add(dfbe * wt);
                acc[3].add(dfbe * ewt);
                const double dewt = wt * de;
                acc[1].add(dewt * fbe);
                acc[5].add(dfbe * dewt);
                acc[2].add(dfbe * ewt * de);
                if (J.lentro) {
                    const double con1 = dfbe * wt * x;
                    acc[7].add(con1 * de);
                    acc[8].add(con1);
                }
            }
        }
    }
    // CTA-wide merge of each pair (fixed tree order), then one store per sum
#pragma unroll
    for (int s = 0; s < FERMI_NSUM; ++s) {
        DD v = acc[s];
        for (int o = 16; o > 0; o >>= 1) {
            const double h = __shfl_xor_sync(0xffffffffu, v.hi, o), l = __shfl_xor_sync(0xffffffffu, v.lo, o);
            v.merge(h, l);
        }
        const int lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
        __syncthreads();
        if (lane == 0) { sh[wid] = v.hi; sh[32 + wid] = v.lo; }
        __syncthreads();
        if (tid == 0) {
            DD t;
            for (int q2 = 0; q2 < nw; ++q2) t.merge(sh[q2], sh[32 + q2]);
            part[(long)blockIdx.x * 2 * FERMI_NSUM + 2 * s] = t.hi;
            part[(long)blockIdx.x * 2 * FERMI_NSUM + 2 * s + 1] = t.lo;
        }
    }
}

__global__ void k_band_finish(FermiJob *jobs, const double *part, int nblk)
{
    FermiJob J = jobs[0];
    const int s = threadIdx.x;
    __shared__ double tot[FERMI_NSUM];
    if (s < FERMI_NSUM) {
        DD t;
        for (int b = 0; b < nblk; ++b) t.merge(part[(long)b * 2 * FERMI_NSUM + 2 * s], part[(long)b * 2 * FERMI_NSUM + 2 * s + 1]);
        tot[s] = t.hi + t.lo;
    }
    __syncthreads();
    if (s == 0) {
        FermiOut o = *J.out;
        o.e_total = tot[0];
        o.fermi_shift = 0;
        o.pressure = 0;
        if (J.lpress) {
            const double dfermi = (fabs(tot[4]) > 1e-10) ? tot[5] / tot[4] : 0.0;
            o.fermi_shift = dfermi;
            o.pressure = -(tot[1] + (tot[2] - dfermi * tot[3]));
        }
        o.entropy = J.lentro ? tot[6] : 0.0;
        o.dent1 = J.lentro ? tot[7] : 0.0;
        o.dent2 = J.lentro ? tot[8] : 0.0;
        o.spin_up = J.nks > 0 ? tot[9] : 0.0;
        o.spin_dn = J.nks > 0 ? tot[10] : 0.0;
        o.pad = 0;
        *J.out = o;
    }
}

size_t fermi_part_bytes() { return sizeof(double) * 2 * FERMI_NSUM * FERMI_BLOCKS; }

void launch_fermi_sums(cudaStream_t s, FermiJob *djob, double *part)
{
    NRLTB_LAUNCH(k_fermi_level, 1, 1024, 0, s, djob);
    NRLTB_LAUNCH(k_band_sums, FERMI_BLOCKS, 256, 0, s, djob, part);
    NRLTB_LAUNCH(k_band_finish, 1, 32, 0, s, djob, part, FERMI_BLOCKS);
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
// ncut[k] = the first band whose eigenvalue exceeds eigcut (nv if none); one
// warp per row, 32 bands per step
__global__ void k_ncut(const double *eig, int ldk, int nv, int nk, double eigcut, int *ncut)
{
    const int k = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (k >= nk) return;   // warp-uniform
    int c = nv;
    for (int c0 = 0; c0 < nv; c0 += 32) {
        const int q = c0 + lane;
        const unsigned above = __ballot_sync(0xffffffffu, q < nv && eig[(long)k * ldk + q] > eigcut);
        if (above) { c = c0 + __ffs(above) - 1; break; }
    }
    if (lane == 0) ncut[k] = c;
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
