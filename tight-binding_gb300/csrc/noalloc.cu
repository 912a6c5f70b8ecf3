// noalloc.cu -- neighbour list (search2.f) for callers that cannot allocate.
//
// Some host codes own all device memory themselves: a framework whose caching
// allocator has reserved the GPU, or a production code that carves every buffer
// out of one arena at start-up.  A cudaMalloc/cudaFree from inside a library
// either fails there or forces a device-wide synchronisation in the middle of
// their pipeline.  nrltb_search2_noalloc gives them the pair list without any
// allocation: inputs and outputs are the caller's device buffers, and the only
// scratch (one code byte per candidate image plus the scan counters) lives in
// the file-scope device array below, which every GPU that loads this library
// keeps until the process exits (NRLTB_NOALLOC_SCRATCH_BYTES, about 16.1 MiB).
//
// The array's host-side name is only a stand-in: its device address is taken
// once per device with cudaGetSymbolAddress, on the first call made with that
// device current (retried by later calls if that lookup failed), and every
// call after that reuses it.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include "nrltb.h"
#include "common.cuh"
#include "setup.cuh"

using namespace nrltb;

namespace {

constexpr long NOALLOC_MAX_CAND = NRLTB_NOALLOC_MAX_CANDIDATES;
constexpr long NOALLOC_BLOCKS = NOALLOC_MAX_CAND / SEARCH_BLOCK + 1;
// layout: [codes: MAX_CAND bytes][block offsets: BLOCKS ints][misc: 64 B][dnn, screenl: 2 x 64 doubles]
constexpr size_t OFF_BLK = (size_t)NOALLOC_MAX_CAND;
constexpr size_t OFF_MISC = OFF_BLK + (((size_t)NOALLOC_BLOCKS * sizeof(int) + 255) & ~size_t(255));
constexpr size_t OFF_CUT = OFF_MISC + 256;
constexpr size_t SCRATCH_BYTES = OFF_CUT + 2 * 64 * sizeof(double);
static_assert(SCRATCH_BYTES == NRLTB_NOALLOC_SCRATCH_BYTES, "header and layout disagree");

__device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
unsigned char *g_scratch_addr[MAX_DEVICES];
std::mutex g_scratch_mutex;

// atom kinds outside 1..kinds would index the cut-off tables out of range:
// count them before the search reads them
__global__ void k_noalloc_kinds(const int *kkind, int natoms, int kinds, int *bad)
{
    int nbad = 0;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < natoms; a += gridDim.x * blockDim.x)
        nbad += (kkind[a] < 1 || kkind[a] > kinds);
    if (nbad) atomicAdd(bad, nbad);
}

}  // namespace

void nrltb_internal_set_error(const char *msg);

extern "C" int nrltb_search2_noalloc(int device, void *stream, int natoms, const int *d_kkind, const double *d_posn,
                                     const double plv[3][3], const int nd[3], int kinds, const double *dnn,
                                     const double *screenl, int kneigh_in, int capacity, double *d_tt, int *d_dlv,
                                     double *d_dist, double *d_screen, double *d_dscrn, int *d_jkind, int *d_jatm,
                                     int *npairs, int *kneigh_out, double *dismin)
{
    if (device < 0 || device >= MAX_DEVICES || natoms < 1 || !d_kkind || !d_posn || !plv || !nd || kinds < 1 ||
        kinds > NRLTB_MAX_KINDS || !dnn || !screenl || capacity < 0 || !npairs)
        return NRLTB_E_ARG;
    if (capacity > 0 && (!d_tt || !d_dlv || !d_dist || !d_screen || !d_dscrn || !d_jkind || !d_jatm))
        return NRLTB_E_ARG;
    for (int i = 0; i < 3; ++i)
        if (nd[i] < 0 || nd[i] > 64) return NRLTB_E_ARG;
    const long box = (long)(2 * nd[0] + 1) * (2 * nd[1] + 1) * (2 * nd[2] + 1);
    const long ncand = (long)natoms * natoms * box;
    if (ncand > NOALLOC_MAX_CAND) {
        char msg[200];
        snprintf(msg, sizeof msg, "search box holds %ld candidate images; the no-allocation path takes at most %ld",
                 ncand, NOALLOC_MAX_CAND);
        nrltb_internal_set_error(msg);
        return NRLTB_E_CAPACITY;
    }
    if (cudaSetDevice(device) != cudaSuccess) return NRLTB_E_CUDA;
    // set-up, once per device, with that device current; a failed lookup is
    // not remembered, so a later call tries again
    unsigned char *base;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_addr[device]) {
            void *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                char msg[200];
                snprintf(msg, sizeof msg, "cudaGetSymbolAddress of the no-allocation scratch array failed: %s",
                         cudaGetErrorString(e));
                nrltb_internal_set_error(msg);
                return NRLTB_E_CUDA;
            }
            g_scratch_addr[device] = (unsigned char *)p;
        }
        base = g_scratch_addr[device];
    }
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *code = base;
    int *blk = (int *)(base + OFF_BLK);
    int *misc = (int *)(base + OFF_MISC);                 // [0] ties [1] total [2] kneigh_out, [4..5] dismin bits
    unsigned long long *dmin = (unsigned long long *)(misc + 4);
    double *ddnn = (double *)(base + OFF_CUT), *dscr = ddnn + 64;
    const int nint = kinds * (kinds + 1) / 2;
    // the array keeps the previous call's contents: counters and cut-offs are reset here
    const unsigned long long inf = 0x7FF0000000000000ull;
    if (cudaMemsetAsync(misc, 0, 16, s) != cudaSuccess ||
        cudaMemcpyAsync(dmin, &inf, 8, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(ddnn, dnn, sizeof(double) * nint, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(dscr, screenl, sizeof(double) * nint, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return NRLTB_E_CUDA;
    DevStructure S;
    S.natoms = natoms;
    S.kkind = d_kkind;
    S.posn = d_posn;
    S.posq = nullptr;
    memcpy(S.plv, plv, sizeof S.plv);
    memcpy(S.nd, nd, sizeof S.nd);
    S.volume = 0.0;
    S.flip = nullptr;
    DevParams P;
    P.kinds = kinds;
    P.jsover = 1;
    P.nltype = 0;
    P.kbas = nullptr;
    P.dnn = ddnn;
    P.screenl = dscr;
    P.param = nullptr;
    P.param_alt = nullptr;
    const int nblk = cdiv(ncand, SEARCH_BLOCK);
    int host_misc[6];
    k_noalloc_kinds<<<cdiv(natoms, 256) < 152 ? cdiv(natoms, 256) : 152, 256, 0, s>>>(d_kkind, natoms, kinds, misc + 3);
    if (cudaMemcpyAsync(host_misc, misc, sizeof host_misc, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return NRLTB_E_CUDA;
    if (host_misc[3] != 0) {
        char msg[200];
        snprintf(msg, sizeof msg, "%d atom kind(s) outside 1..%d", host_misc[3], kinds);
        nrltb_internal_set_error(msg);
        return NRLTB_E_ARG;
    }
    k_search_eval<<<std::min(cdiv(ncand, 256), 152 * 16), 256, 0, s>>>(S, P, ncand, code, misc, dmin);
    if (cudaMemcpyAsync(host_misc, misc, sizeof host_misc, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return NRLTB_E_CUDA;
    k_search_ties<<<1, 1, 0, s>>>(code, ncand, kneigh_in, misc + 2, host_misc[0] > 0);
    k_search_count<<<nblk, SEARCH_BLOCK, 0, s>>>(code, ncand, blk);
    k_scan_small<<<1, 1024, 0, s>>>(blk, nblk, misc + 1);
    if (cudaMemcpyAsync(host_misc, misc, sizeof host_misc, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return NRLTB_E_CUDA;
    const int total = host_misc[1];
    DevPairs out;
    out.tt = d_tt; out.dlv = d_dlv; out.dist = d_dist; out.screen = d_screen; out.dscrn = d_dscrn;
    out.jkind = d_jkind; out.jatm = d_jatm;
    if (capacity > 0)
        k_search_scatter<<<nblk, SEARCH_BLOCK, 0, s>>>(S, P, code, ncand, blk, out, capacity);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) return NRLTB_E_CUDA;
    *npairs = total;
    if (kneigh_out) *kneigh_out = host_misc[2];
    if (dismin) {
        unsigned long long bits;
        memcpy(&bits, host_misc + 4, 8);
        double d2;
        memcpy(&d2, &bits, 8);
        *dismin = (bits == inf) ? sqrt(1e10) : sqrt(d2);
    }
    return total > capacity ? NRLTB_E_CAPACITY : NRLTB_OK;
}
