// refine.cu -- mixed-precision refinement and Hellmann-Feynman products.
#include "refine.cuh"
#include "gemm.cuh"
#include "sums.cuh"
#include "nrltb.h"

namespace nrltb {

static inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

bool refine_available() { return false; }

size_t refine_work_bytes(int n, int batch)
{
    RefineWork w;
    refine_work_carve(w, nullptr, n, batch);
    return (size_t)(uintptr_t)w.cl + sizeof(int) * (size_t)n * batch + 256;
}

void refine_work_carve(RefineWork &w, void *base, int n, int batch)
{
    size_t off = 0, nn = (size_t)n * n * batch;
    char *b = (char *)base;
    auto take = [&](size_t bytes) { void *p = b + off; off = al256(off + bytes); return p; };
    w.n = n; w.batch = batch;
    w.YH = (double2 *)take(sizeof(double2) * nn);
    w.YS = (double2 *)take(sizeof(double2) * nn);
    w.T = (double2 *)take(sizeof(double2) * nn);
    w.R = (double2 *)take(sizeof(double2) * nn);
    w.U = (double2 *)take(sizeof(double2) * nn);
    w.Ef = (float2 *)take(sizeof(float2) * nn);
    w.Xr = (float2 *)take(sizeof(float2) * nn);
    w.XE = (float2 *)take(sizeof(float2) * nn);
    w.lam = (double *)take(sizeof(double) * (size_t)n * batch);
    w.cl = (int *)take(sizeof(int) * (size_t)n * batch);
    if (!base) w.cl = (int *)(uintptr_t)off;
}

void refine_eigen(cudaStream_t s, RefineWork &w, const double2 *H, const double2 *S, const float2 *X,
                  double *eig, double2 *Z, int *status)
{
    (void)s; (void)w; (void)H; (void)S; (void)X; (void)eig; (void)Z; (void)status;
}

size_t hf_scratch_bytes(int n, int nkc) { return 2 * sizeof(double2) * (size_t)n * n * nkc + 512; }

int run_hf(cudaStream_t s, int n, int nkc, int prec, const double2 *dH, const double2 *dS, const double2 *Z,
           const double *eig, double *deig, void *scratch, void *unused)
{
    (void)unused; (void)prec;
    const long nn = (long)n * n;
    double2 *P = (double2 *)scratch;
    double2 *Q = (double2 *)((char *)scratch + al256(sizeof(double2) * nn * nkc));
    const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
    // P = triu(dH) Z, Q = triu(dS) Z
    zgemm<double>(s, n, n, n, nkc, one, dH, n, nn, 0, Z, n, nn, 0, zero, P, n, nn, 2, 0, 0);
    zgemm<double>(s, n, n, n, nkc, one, dS, n, nn, 0, Z, n, nn, 0, zero, Q, n, nn, 2, 0, 0);
    launch_hf_dots(s, Z, P, Q, dH, dS, eig, deig, n, nkc);
    return cudaGetLastError() == cudaSuccess ? NRLTB_OK : NRLTB_E_CUDA;
}

}  // namespace nrltb
