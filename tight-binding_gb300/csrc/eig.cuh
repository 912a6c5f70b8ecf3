// eig.cuh -- batched generalized Hermitian eigensolver H x = lambda S x.
//
// Replaces diag.f:385-455 -> zhpgv(1,'V','U') (Cholesky zpptrf, reduction
// zhpgst, tridiagonalisation zhptrd, tridiagonal solve, back-transform) by a
// blocked GPU design written from the published algorithms:
//
//   1. S = L L^H, right-looking blocked Cholesky; the nb x nb diagonal blocks
//      are factored (and inverted) in shared memory, panels and trailing
//      updates are batched GEMMs.
//   2. W = L^{-1} by the blocked bottom-up triangular inverse (GEMMs).
//   3. A = W H W^H as two triangular GEMMs.
//   4. A = Q T Q^H, blocked Householder tridiagonalisation (lower): per column a
//      column update, reflector, lower-triangle Hermitian mat-vec and w update;
//      per panel a rank-2nb trailing update as two GEMMs.
//   5. T (real symmetric) eigenvalues by Sturm-count bisection per unreduced
//      block; eigenvectors by inverse iteration (dstein's factorisation and
//      solves) in FP64, each cluster of close eigenvalues orthonormalised
//      afterwards.
//   6. X = W^H Q Y: compact-WY application of the reflectors in blocks of
//      EIG_WY (rows above each block skipped) and a triangular GEMM.
// Every stage runs on all matrices of the batch at once (grid.z / grid.y =
// matrix).  Non-positive-definite S is reported per matrix (status 1), as
// diag.f:429-455 does with ioverr, without stopping the batch.
#pragma once
#include "common.cuh"
#include "gemm.cuh"

namespace nrltb {

constexpr int EIG_NB = 32;          // panel width (Cholesky, inverse, tridiagonal)
constexpr int EIG_ROWS = 128;       // rows per CTA in the column kernels
constexpr int EIG_WY = 128;         // reflectors per block of the back-transform

// Device workspace for one batch of `batch` matrices of order n.
template <typename T> struct EigWork {
    typedef typename cplx<T>::t C2;
    int n, batch;
    long ld, mstride;               // leading dimension, matrix stride (elements)
    C2 *L;                          // S -> Cholesky factor (lower)
    C2 *Wi;                         // L^{-1} (lower)
    C2 *A;                          // reduced matrix, overwritten by tridiagonalisation
    C2 *Y;                          // scratch n x n (reduction product, then Q Y)
    C2 *V;                          // Householder vectors, column i in V[:, i]
    C2 *Wp;                         // panel W, n x EIG_NB per matrix (matrix stride wps)
    C2 *VW;                         // [V panel | W | V panel], n x 3 EIG_NB per matrix; Wp is its middle
    long wps;                       // matrix stride of VW and Wp
    C2 *wq;                         // w' of the current column, n per matrix
    C2 *col;                        // current updated column, n per matrix
    C2 *tau;                        // n per matrix
    C2 *pp;                         // p1 | p2, 2*EIG_NB per matrix
    C2 *part;                       // per-CTA partial sums, [batch][ncta][2*EIG_NB+2]
    C2 *sc;                         // per-matrix scalars: [0] scale, [1] alpha
    C2 *Tt;                         // back-transform: G = Vb^H Vb, then the T factor of every block
    C2 *Xt;                         // EIG_NB x n per matrix
    double *d, *e;                  // tridiagonal, n per matrix
    double *lam;                    // eigenvalues, n per matrix (ascending)
    double *ylu;                    // inverse-iteration scratch, 4 n per thread
    double *yvec;                   // real eigenvectors of T, n x n per matrix
    int *perm;                      // eigenvalue -> block bookkeeping, 3 n per matrix
    unsigned *counter;              // per-matrix ticket counters (last-CTA pattern)
    int *status;                    // per-matrix status
};

template <typename T> size_t eig_work_bytes(int n, int batch);
template <typename T> void eig_work_carve(EigWork<T> &w, void *base, int n, int batch);

// Optional streams for the back-transform's WY factors: given them and their
// events, eig_solve forms the blocks' G = Vb^H Vb and T factors on the aux
// streams, block by block in turn (after `tri_done`, recorded on s when the
// tridiagonalisation is queued), while s solves the tridiagonal eigenproblem,
// and s waits for every `wy_done` before the back-transform.  The results are
// the same either way.
constexpr int EIG_NAUX = 3;   // auxiliary streams for the WY factors (blocks dealt round-robin)
struct EigAux {
    cudaStream_t aux[EIG_NAUX] = {};
    cudaEvent_t tri_done = nullptr, wy_done[EIG_NAUX] = {};
};

// Full solve.  H and S (FP64, column-major, leading dimension n, stride n*n)
// are converted to T inside.  eig: n per matrix; X (optional, precision T):
// S-orthonormal eigenvectors, column-major, stride n*n.  tri_start (optional)
// is recorded on s when the tridiagonalisation begins (its latency-bound
// panels leave most of the GPU to work on other streams).
template <typename T>
void eig_solve(cudaStream_t s, EigWork<T> &w, const double2 *H, const double2 *S,
               double *eig, typename cplx<T>::t *X, bool vectors, cudaEvent_t tri_start = nullptr,
               const EigAux *ax = nullptr);

}  // namespace nrltb
