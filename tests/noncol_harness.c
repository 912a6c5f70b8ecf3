/*
 * Host build of the non-collinear formulas that the CUDA kernels evaluate
 * (tight-binding_gb300/csrc/noncol_math.h), for the CPU test that compares
 * them with the oracle.  Test infrastructure only.
 */
#include "noncol_math.h"

void h_onsite(int natoms, int kinds, const int *kkind, const double *den1, const double *den2, const double *vden1,
              const double *vden2, const double *P1, const double *P2, int deriv, double *paros, double *spinos,
              double *dparos, double *dspnos)
{
    for (int a = 0; a < natoms; ++a) {
        const int o = a * kinds;
        nc_onsite_atom(kinds, kkind[a], den1 + o, den2 + o, vden1 + o, vden2 + o, P1 - 1, P2 - 1, deriv,
                       paros + 4 * a, spinos + 4 * a, dparos + 4 * a, dspnos + 4 * a);
    }
}

void h_spin_terms(int natoms, const int *nbas, const double *spinos, const double *spinat, double *diag, double *mre,
                  double *mim)
{
    int i = 0;
    for (int a = 0; a < natoms; ++a)
        for (int k = 0; k < nbas[a]; ++k, ++i)
            nc_spin_terms(k, spinos + 4 * a, spinat + 3 * a, diag + i, mre + i, mim + i);
}

/* Hn: batch interleaved complex column-major N x N; H2 receives 2N x 2N */
void h_expand(int nv, int batch, const double *Hn, const double *diag, const double *mre, const double *mim,
              double *H2)
{
    const long n2 = 2L * nv, nn = (long)nv * nv;
    for (int b = 0; b < batch; ++b)
        for (int c = 0; c < n2; ++c)
            for (int r = 0; r < n2; ++r) {
                const double *hb = Hn + 2 * b * nn;
                double *o = H2 + 2 * (b * n2 * n2 + r + c * n2);
                nc_expand(nv, r, c, hb, hb + 1, 2, diag, mre, mim, o, o + 1);
            }
}
