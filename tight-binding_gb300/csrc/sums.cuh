// sums.cuh -- Fermi level / energy / pressure reduction and Hellmann-Feynman dots.
#pragma once
#include "common.cuh"

namespace nrltb {

struct FermiOut {
    double efermi, e_total, pressure, fermi_shift;
    double entropy, dent1, dent2;   // Gillan sums (lentro), else 0
    int iterations, pad;
};

struct FermiJob {
    const double *eig;      // [nk][ldk]
    const double *deig;     // [nk][ldk] (mode 4)
    const double *w;        // [nk]
    const int *ncut;        // [nk] (mode 4)
    int nv, nk, ldk, lpress;
    int lentro, pad;        // entropy sums (modes 1, 2)
    double tkb, zfill, tol;
    FermiOut *out;
};

__global__ void k_fermi_sums(FermiJob *jobs);
__global__ void k_ncut(const double *eig, int ldk, int nv, int nk, double eigcut, int *ncut);
void launch_hf_dots(cudaStream_t s, const double2 *Z, const double2 *P, const double2 *Q, const double2 *dH,
                    const double2 *dS, const double *eig, double *deig, int n, int batch);
// the same from the full products P = dH Z, Q = dS Z
void launch_hf_dots_full(cudaStream_t s, const double2 *Z, const double2 *P, const double2 *Q, const double *eig,
                         double *deig, int n, int batch);

}  // namespace nrltb
