// sums.cuh -- Fermi level / energy / pressure reduction and Hellmann-Feynman dots.
#pragma once
#include "common.cuh"

namespace nrltb {

struct FermiOut {
    double efermi, e_total, pressure, fermi_shift;
    double entropy, dent1, dent2;   // Gillan sums (lentro), else 0
    double spin_up, spin_dn;        // spin populations (nks > 0), else 0
    int iterations, pad;
};

struct FermiJob {
    const double *eig;      // [nk][ldk]
    const double *deig;     // [nk][ldk] (modes 2, 4)
    const double *w;        // [nk] weight of each row
    const int *ncut;        // [nk] (modes 2, 4)
    int nv, nk, ldk, lpress;   // nk rows: all spin channels' k points, spin 1 first
    int lentro;             // entropy sums (modes 1, 2)
    int nks;                // k points per spin channel when there are two, else 0
    double el;              // electrons per band: 2 spin-restricted, 1 spin-polarized
    double tkb, zfill, tol;
    FermiOut *out;
};

// E_F, then the energy / pressure / entropy / spin sums: three launches on s
// (one CTA for the Newton iteration, FERMI_BLOCKS CTAs for the sums, one to
// merge them); part holds fermi_part_bytes() of device scratch.
constexpr int FERMI_BLOCKS = 152;
size_t fermi_part_bytes();
void launch_fermi_sums(cudaStream_t s, FermiJob *djob, double *part);
// non-collinear spin directions (diag.f:458-524, bande.f:1480-1537): per k,
// state and atom the spin vector of the up and down halves of the
// eigenvector; then its occupied-state sum per atom and component
__global__ void k_spin_expect(const double2 *Z, int n2, int batch, int natoms, const int *ksk, double *spev);
__global__ void k_spin_dir_sum(const double *eig, const double *w, const double *spev, const FermiOut *fo,
                               double tkb, double el, int nrow, int n2, int natoms, double *spdir);
__global__ void k_ncut(const double *eig, int ldk, int nv, int nk, double eigcut, int *ncut);
void launch_hf_dots(cudaStream_t s, const double2 *Z, const double2 *P, const double2 *Q, const double2 *dH,
                    const double2 *dS, const double *eig, double *deig, int n, int batch);
// the same from the full products P = dH Z, Q = dS Z
void launch_hf_dots_full(cudaStream_t s, const double2 *Z, const double2 *P, const double2 *Q, const double *eig,
                         double *deig, int n, int batch);

}  // namespace nrltb
