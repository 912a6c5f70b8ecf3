// refine.cuh -- mixed-precision form: FP64-accurate refinement of FP32
// eigenpairs, and the Hellmann-Feynman products of both forms.
#pragma once
#include "common.cuh"
#include "ozaki.cuh"

namespace nrltb {

struct RefineWork {
    int n, batch;
    double2 *YH, *YS;       // H X, S X
    double2 *Xd;            // rotated vectors X' = X U (FP64)
    float2 *G;              // X'^H r', r'_j = H x'_j - l_j S x'_j
    double2 *U;             // cluster rotations
    float2 *Ef;             // FP32 update matrix
    float2 *Xr;             // rotated FP32 vectors
    float2 *XE;             // X' E (FP32)
    float2 *Fb;             // second-order Gram terms near the sorted diagonal
    double *lam;            // refined eigenvalues
    int *cl;                // cluster id per eigenvalue
    void *oz;               // digit planes of the tensor-core products (ozaki.cuh)
};

bool refine_available();
size_t refine_work_bytes(int n, int batch);
void refine_work_carve(RefineWork &w, void *base, int n, int batch);
// H, S FP64; X FP32 eigenvectors from the FP32 solve (S-orthonormal to FP32
// accuracy); writes refined eigenvalues (ascending) and, if Z != NULL, FP64
// eigenvectors.  status[k] gets NRLTB_K_NOT_CONVERGED when a cluster exceeds the
// handled size.
// X is rounded in place to the representation the tensor-core products use.
// pre (optional): the 6-digit forms of H and S from ozaki_prepare_a, already
// made (or being made on a stream this one waits for).
// aux (optional): a second stream and two events; the rotated residuals of
// the columns outside clusters, which need no cluster solve, are then formed
// on it beside the cluster Rayleigh-Ritz solves (the same values either way).
struct RefAux {
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;
};
void refine_eigen(cudaStream_t s, RefineWork &w, const double2 *H, const double2 *S, float2 *X,
                  double *eig, double2 *Z, int *status, const OzakiA *pre = nullptr, const RefAux *ra = nullptr);

// Hellmann-Feynman shifts deig = diag(Z^H dH Z) - eig * diag(Z^H dS Z) for nkc
// matrices; scratch must hold hf_scratch_bytes(n, nkc), 256-byte aligned.
// pre (optional, mixed form): the 3-digit forms of dH and dS from
// ozaki_prepare_a (dH, dS are then not read).
int run_hf(cudaStream_t s, int n, int nkc, int prec, const double2 *dH, const double2 *dS, const double2 *Z,
           const double *eig, double *deig, void *scratch, const OzakiA *pre = nullptr);
size_t hf_scratch_bytes(int n, int nkc);

}  // namespace nrltb
