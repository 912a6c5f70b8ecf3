// setup.cuh -- device views of the structure, parameters, pair list and the
// k-independent Slater-Koster tables, and the kernels of setup.cu.
#pragma once
#include "common.cuh"

#define NRLTB_MAX_KINDS 8

namespace nrltb {

struct DevStructure {
    int natoms;
    const int *kkind;       // device
    const double *posn;     // device [natoms][3]
    const double *posq;     // device [natoms][3]
    double plv[3][3];
    int nd[3];
    double volume;
    const int *flip;        // device [natoms], nonzero = spin flipped; nullptr = none
};

struct DevParams {
    int kinds, jsover, nltype;
    const int *kbas;        // device
    const double *dnn, *screenl, *param;   // device; param = this spin channel's set
    const double *param_alt;               // the set flipped atoms' densities and on-site terms use
};

// parameter set (1-based view) for atom a's density and on-site terms
// (setpar.f:500-536, 806-867: jsfrm = 3 - jspin for a flipped atom)
__device__ __forceinline__ const double *atom_params(const DevStructure &S, const DevParams &P, int a)
{
    return ((S.flip && S.flip[a]) ? P.param_alt : P.param) - 1;
}

struct DevPairs {
    double *tt; int *dlv; double *dist, *screen, *dscrn; int *jkind, *jatm;
};

struct DevSK {
    double *hop, *over, *dhop, *dover;  // [P][14]
    double *dent, *vdent;               // [P][2] density terms of atom 1, atom 2
    double *den;                        // [natoms][kinds]
    double *vden;                       // [natoms][kinds] volume derivatives of den (deriv)
    double *paros, *dparos;             // [natoms][4]
    double *E;                          // [4][P][81] SK blocks: H, S, dH, dS
};

__global__ void k_search_eval(DevStructure S, DevParams P, long ncand, unsigned char *code, int *tie_count,
                              unsigned long long *dismin_bits);
__global__ void k_search_ties(unsigned char *code, long ncand, int kneigh_in, int *kneigh_out, int resolve);
__global__ void k_search_count(const unsigned char *code, long ncand, int *blockcnt);
__global__ void k_scan_small(int *cnt, int nblk, int *total);
__global__ void k_search_scatter(DevStructure S, DevParams P, const unsigned char *code, long ncand,
                                 const int *blockoff, DevPairs out, int capacity);
__global__ void k_setpar_pairs(DevStructure S, DevParams P, DevPairs pr, int npairs, DevSK sk, int deriv);
__global__ void k_setpar_atoms(DevStructure S, DevParams P, DevPairs pr, int npairs, DevSK sk, int deriv);
__global__ void k_sk_blocks(DevPairs pr, int npairs, DevSK sk, int nwhich);
// non-collinear spins (noncol_math.h): on-site terms per atom, spin terms per
// orbital, and the N x N -> 2N x 2N expansion of a batch of matrices
__global__ void k_noncol_onsite(int natoms, int kinds, const int *kkind, const double *den1, const double *den2,
                                const double *vden1, const double *vden2, const double *P1, const double *P2,
                                int deriv, double *paros, double *spinos, double *dparos, double *dspnos);
__global__ void k_noncol_spin_terms(int nv, const int *orb_atom, const int *ksk, const double *spinos,
                                    const double *spinat, double *diag, double *mix_re, double *mix_im);
__global__ void k_noncol_expand(int nv, int batch, const double2 *Hn, const double *diag, const double *mix_re,
                                const double *mix_im, double2 *H2);
__global__ void k_segments(DevPairs pr, int npairs, int natoms, int2 *seg);
__global__ void k_phases(DevStructure S, DevPairs pr, int npairs, const double *kq, int nk, double2 *ph);
__global__ void k_bloch_build(DevStructure S, DevParams P, DevPairs pr, int npairs, DevSK sk, const int2 *seg,
                              const int *orb_atom, const int *ksk, const double2 *ph, int nk, int nv, int which0,
                              double2 *M1, double2 *M2, int jsover);

constexpr int SEARCH_BLOCK = 1024;

}  // namespace nrltb
