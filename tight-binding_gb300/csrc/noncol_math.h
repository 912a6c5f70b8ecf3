/*
 * noncol_math.h -- non-collinear spins, the per-atom and per-element formulas.
 *
 * Plain C functions used by the CUDA kernels (as __host__ __device__) and by a
 * host-compiled check.  Parameters are passed as 1-based views (P[1] is the
 * first parameter of a set), as the reference indexes them.
 *
 *   nc_onsite_atom   setpar.f:746-796 and setparv.f:723-795, lnoncol branches:
 *                    the average and half difference of the two parameter
 *                    sets' on-site polynomials.  The cross-species terms are
 *                    the reference's own: they replace (not add to) the
 *                    average, setpar reads 4 coefficients with stride 4 and a
 *                    full difference, setparv takes the first set's density
 *                    derivative for both spins and a stride of 3.
 *   nc_spin_terms    spinham.f:122-158: a spin splitting s along direction m
 *                    gives s m_z on the diagonal and s (m_x + i m_y) between
 *                    the spin blocks.
 *   nc_expand        addspins.f:77-110: element (r, c) of the 2N x 2N matrix
 *                    [H + D, M; M^H, H - D] (or [S, 0; 0, S]) from the N x N
 *                    column-major H, D = diag(diag), M = diag(mix).
 */
#ifndef NRLTB_NONCOL_MATH_H
#define NRLTB_NONCOL_MATH_H
#include <math.h>

#ifdef __CUDACC__
#define NC_HD __host__ __device__ inline
#else
#define NC_HD static inline
#endif

/* kinds(29 + 68 kinds) layout: density and on-site block of a species, and the
 * cross-species on-site block of (jk1, jk2) (setpar.f:456, 806-812) */
NC_HD int nc_ip_density(int kind) { return (kind - 1) * 17 + 1; }
NC_HD int nc_ip_cross(int kinds, int jk1, int jk2)
{
    int jkx = jk1 > jk2 ? jk1 : jk2, jkm = jk1 < jk2 ? jk1 : jk2;
    int ip = kinds * 17 + 24 * ((jkx - 1) * (jkx - 2) / 2 + jkm - 1);
    if (jk2 < jkx) ip += 12;
    return ip;
}

/* d1, d2: the atom's densities from each set, [kinds]; v1, v2 their volume
 * derivatives (used when deriv).  Outputs [4] per orbital class. */
NC_HD void nc_onsite_atom(int kinds, int jk1, const double *d1, const double *d2, const double *v1,
                          const double *v2, const double *P1, const double *P2, int deriv, double *paros,
                          double *spinos, double *dparos, double *dspnos)
{
    const double third = 1.0 / 3.0, twtrd = 2.0 / 3.0, threeh = 1.5, half = 0.5;
    int ip = nc_ip_density(jk1);
    double vm23up = pow(d1[jk1 - 1], twtrd), vm23dn = pow(d2[jk1 - 1], twtrd);
    for (int k = 0; k < 4; ++k) {
        double pup = P1[ip + 1] + vm23up * (P1[ip + 2] + vm23up * (P1[ip + 3] + vm23up * P1[ip + 4]));
        double pdn = P2[ip + 1] + vm23dn * (P2[ip + 2] + vm23dn * (P2[ip + 3] + vm23dn * P2[ip + 4]));
        paros[k] = half * (pup + pdn);
        spinos[k] = half * (pup - pdn);
        ip += 4;
    }
    for (int jk2 = 1; jk2 <= kinds; ++jk2) {
        double dmax = d1[jk2 - 1] > d2[jk2 - 1] ? d1[jk2 - 1] : d2[jk2 - 1];
        if (jk2 == jk1 || !(dmax > 0.0)) continue;
        vm23up = pow(d1[jk2 - 1], twtrd);
        vm23dn = pow(d2[jk2 - 1], twtrd);
        ip = nc_ip_cross(kinds, jk1, jk2);
        for (int k = 0; k < 4; ++k) {
            double pup = P1[ip + 1] + vm23up * (P1[ip + 2] + vm23up * (P1[ip + 3] + vm23up * P1[ip + 4]));
            double pdn = P2[ip + 1] + vm23dn * (P2[ip + 2] + vm23dn * (P2[ip + 3] + vm23dn * P2[ip + 4]));
            paros[k] = half * (pup + pdn);
            spinos[k] = pup - pdn;
            ip += 4;
        }
    }
    if (!deriv) return;
    ip = nc_ip_density(jk1);
    double vm13up = pow(d1[jk1 - 1], third), vm13dn = pow(d2[jk1 - 1], third);
    vm23up = vm13up * vm13up;
    vm23dn = vm13dn * vm13dn;
    double vm2tup = 2.0 * vm23up, vm3tup = threeh * vm23up, vm2tdn = 2.0 * vm23dn, vm3tdn = threeh * vm23dn;
    double drhoup = twtrd * v1[jk1 - 1] / vm13up, drhodn = twtrd * v2[jk1 - 1] / vm13dn;
    for (int k = 0; k < 4; ++k) {
        double dpup = drhoup * (P1[ip + 2] + vm2tup * (P1[ip + 3] + vm3tup * P1[ip + 4]));
        double dpdn = drhodn * (P2[ip + 2] + vm2tdn * (P2[ip + 3] + vm3tdn * P2[ip + 4]));
        dparos[k] = half * (dpup + dpdn);
        dspnos[k] = half * (dpup - dpdn);
        ip += 4;
    }
    for (int jk2 = 1; jk2 <= kinds; ++jk2) {
        if (jk2 == jk1 || d1[jk2 - 1] == 0.0) continue;
        vm13up = pow(d1[jk2 - 1], third);
        vm23up = vm13up * vm13up;
        vm2tup = 2.0 * vm23up;
        vm3tup = threeh * vm23up;
        drhoup = twtrd * v1[jk2 - 1] / vm13up;
        vm13dn = pow(d2[jk2 - 1], third);
        vm23dn = vm13dn * vm13dn;
        vm2tdn = 2.0 * vm23dn;
        vm3tdn = threeh * vm23dn;
        drhodn = twtrd * v1[jk2 - 1] / vm13dn;
        ip = nc_ip_cross(kinds, jk1, jk2);
        for (int k = 0; k < 4; ++k) {
            double dpup = drhoup * (P1[ip + 2] + vm2tup * (P1[ip + 3] + vm3tup * P1[ip + 4]));
            double dpdn = drhodn * (P2[ip + 2] + vm2tdn * (P2[ip + 3] + vm3tdn * P2[ip + 4]));
            dparos[k] = half * (dpup + dpdn);
            dspnos[k] = half * (dpup - dpdn);
            ip += 3;
        }
    }
}

/* orbital kloc (0-based within its atom): class s, p, t2g, eg (spinham.f:141-149) */
NC_HD void nc_spin_terms(int kloc, const double *spinos, const double *m, double *diag, double *mix_re,
                         double *mix_im)
{
    const int q = (kloc == 0) ? 0 : (kloc < 4) ? 1 : (kloc < 7) ? 2 : 3;
    const double so = spinos[q];
    *diag = so * m[2];
    *mix_re = so * m[0];
    *mix_im = so * m[1];
}

/* element (r, c) of the doubled matrix; h_re/h_im point at the N x N
 * column-major matrix, diag/mix at the per-orbital spin terms (NULL for S) */
NC_HD void nc_expand(int nv, int r, int c, const double *h_re, const double *h_im, int hstride,
                     const double *diag, const double *mix_re, const double *mix_im, double *out_re, double *out_im)
{
    const int r0 = r < nv ? r : r - nv, c0 = c < nv ? c : c - nv;
    const int rb = r >= nv, cb = c >= nv;
    if (rb == cb) {   /* diagonal spin block: H (+ D above, - D below) */
        const long e = (long)hstride * (r0 + (long)c0 * nv);
        double re = h_re[e], im = h_im[e];
        if (diag && r0 == c0) re = rb ? re - diag[r0] : re + diag[r0];
        *out_re = re;
        *out_im = im;
    } else if (diag && r0 == c0) {   /* the mixing term, M above and M^H below */
        *out_re = mix_re[r0];
        *out_im = rb ? -mix_im[r0] : mix_im[r0];
    } else {
        *out_re = 0.0;
        *out_im = 0.0;
    }
}

#endif
