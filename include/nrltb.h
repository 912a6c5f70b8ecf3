/*
 * nrltb.h -- C ABI of the GB300 (sm_103a) implementation of the NRL tight-binding
 * per-k-point path: neighbour list, Slater-Koster tables, Bloch sums, generalized
 * Hermitian eigensolve, Fermi level, band energy and Hellmann-Feynman pressure.
 *
 * Every entry point takes plain host pointers and sizes, returns NRLTB_OK (0) or a
 * negative NRLTB_E_* code, and never aborts the process.  Per-k failures are
 * reported through the k_status array, not through the return code.
 *
 * Reference paths below are relative to the NRLtb project root of the reference
 * code ("static" version 1.33, Fortran 77).  Indices in the structs are 1-based
 * where the reference's are (species numbers kkind), 0-based everywhere else.
 */
#ifndef NRLTB_H
#define NRLTB_H

#ifdef __cplusplus
extern "C" {
#endif

#define NRLTB_ABI_VERSION 2

/* ---- return codes ------------------------------------------------------ */
#define NRLTB_OK             0
#define NRLTB_E_ARG         -1   /* bad argument (null pointer, size out of range)  */
#define NRLTB_E_CUDA        -2   /* a CUDA call failed; nrltb_last_error() has text */
#define NRLTB_E_NOMEM       -3   /* device or host allocation failed                */
#define NRLTB_E_CAPACITY    -4   /* caller-sized output too small (count returned)  */
#define NRLTB_E_PARSE       -5   /* input file format error                         */
#define NRLTB_E_IO          -6   /* input file missing / unreadable                 */
#define NRLTB_E_UNSUPPORTED -7   /* option outside the implemented scope            */
#define NRLTB_E_EOF         -8   /* no more structures in the SKIN file             */
#define NRLTB_E_NODEVICE    -9   /* no CUDA device / driver                          */
#define NRLTB_E_TIMEOUT    -10   /* a bounded device wait gave up (k_status has      */
                                 /* NRLTB_K_TIMEOUT at the k points it hit)         */

/* ---- per-k status (k_status[k]) ---------------------------------------- */
#define NRLTB_K_OK            0
#define NRLTB_K_S_NOT_PD      1  /* overlap not positive definite (diag.f:429-455)   */
#define NRLTB_K_DEGENERACY    2  /* reserved: degenerate group larger than handled   */
#define NRLTB_K_NOT_CONVERGED 3  /* mixed form: refinement did not reach tolerance   */
#define NRLTB_K_TIMEOUT       4  /* a bounded device wait gave up                    */

/* ---- precision forms ---------------------------------------------------- */
#define NRLTB_PREC_FP64   0      /* plain FP64 drop-in                              */
#define NRLTB_PREC_MIXED  1      /* FP32 eigensolve + FP64-accurate refinement      */

/* ---- option flags (nrltb_opts.flags) ------------------------------------ */
#define NRLTB_OPT_SPIN_DIRECTIONS 1  /* non-collinear runs: fill nrltb_result.spdir    */

/*
 * One periodic structure, after input1.f and the lattice-to-Cartesian conversion
 * of static.f:1088-1103 (the common blocks /codes/, /latt1/, /fazon/, /disply/).
 */
typedef struct {
    int natoms;
    const int *kkind;      /* [natoms] species 1..kinds                        */
    const double *posn;    /* [natoms][3] Cartesian positions, bohr            */
    const double *posq;    /* [natoms][3] Bloch phase offsets (/fazon/), or 0  */
    double plv[3][3];      /* plv[i][c]: Cartesian component c of vector i     */
    int nd[3];             /* search box half-widths nd1..nd3 (input1.f:488)   */
    double volume;         /* cell volume, bohr^3 (setlat.f:997-1000)          */
    double zcharge;        /* electrons above the nominal valence (static.f)   */
    const int *flip;       /* optional [natoms], jspins = 2 only: nonzero if the */
                           /* atom's spin is flipped (input1.f:778-787 magdir 2),*/
                           /* its density and on-site terms then take the other */
                           /* spin's parameters (setpar.f:500-536, 806-867)      */
    const double *spinat;  /* optional [natoms][3] unit spin direction per atom:  */
                           /* non-collinear spins (input1.f:754-771, flag N),    */
                           /* jspins = 2 sets, a 2N x 2N problem (per-k outputs  */
                           /* then have 2N columns, one block); flips ignored    */
} nrltb_structure;

/*
 * One NRL parameter set (input.f), spin-restricted.  Interaction types are numbered
 * as search2.f:138-144 does: like species t = kind, unlike (jk1<jk2)
 * t = kinds + (jk2-1)(jk2-2)/2 + jk1 (1-based), stored 0-based here.
 */
typedef struct {
    int kinds;
    int jsover;            /* 1 non-orthogonal (S computed), 0 orthogonal      */
    int nltype;            /* 0 old overlap, 1 realov, 2/3 Harrison, 90000 H   */
    const int *kbas;       /* [kinds] orbitals per species: 1, 4 or 9           */
    const double *valence; /* [kinds] formal valence (s+p+d occupancy)          */
    const double *dnn;     /* [kinds(kinds+1)/2] cutoff radius per type, bohr   */
    const double *screenl; /* [kinds(kinds+1)/2] screening length per type      */
    const double *param;   /* [jspins][kinds(29+68 kinds)] parameters, file order*/
    int jspins;            /* 1 (or 0) spin-restricted; 2 collinear spin-      */
                           /* polarized ("M" files, input.f:157-229): one set  */
                           /* per spin, one electron per band                 */
} nrltb_params;

/* Explicit k list in reciprocal-lattice coordinates (kptin.f -1313 path). */
typedef struct {
    int nk;
    const double *k;       /* [nk][3]                                           */
    const double *w;       /* [nk] weights, normalized to sum 1 (kptin.f:350)   */
} nrltb_kmesh;

typedef struct {
    int mode;              /* static.f modes: 3 E(T); 4 E(T), P(T); 1 and 2 the  */
                           /* same plus Gillan's T -> 0 extrapolation; 5, 6, 10 */
                           /* E(T) plus orbital charges (orbocc); 8, 9 E(T) for */
                           /* eigenvalue files (7 is not a mode of the reference)*/
    int precision;         /* NRLTB_PREC_FP64 or NRLTB_PREC_MIXED               */
    double tkb;            /* Fermi broadening kT, Ry                           */
    double eigcut;         /* eigenvalue cutoff for the pressure sums, Ry       */
    double fermi_tol;      /* |N - zfill| and bracket tolerance; 0 -> 1e-8      */
    int kneigh_in;         /* search2's carried /relat/ kneigh flag (0 at start)*/
    int flags;             /* NRLTB_OPT_* bits, 0 for none                      */
} nrltb_opts;

/* Pair list of search2.f (common /pairs/ and /neigh/), caller-allocated. */
typedef struct {
    int capacity;          /* in: length of every array below, in pairs         */
    int npairs;            /* out                                               */
    double *tt;            /* [cap][3] direction cosines                        */
    int *dlv;              /* [cap][3] lattice translation of atom 2            */
    double *dist;          /* [cap]                                             */
    double *screen;        /* [cap]                                             */
    double *dscrn;         /* [cap] d(screen)/dR / screen                       */
    int *jkind;            /* [cap][2] species of atom 1, atom 2                */
    int *jatm;             /* [cap][2] atom numbers, 1-based, jatm1 <= jatm2     */
} nrltb_pairs;

typedef struct {
    double efermi;         /* Fermi level, Ry                                   */
    double e_total;        /* E(T) band energy per cell, Ry                     */
    double pressure;       /* P(T) = -dE/dV, Ry/bohr^3 (modes 2 and 4)          */
    double fermi_shift;    /* dE_F/dV term (bande.f:1440)                       */
    double dismin;         /* shortest pair distance (search2.f:226)            */
    int npairs, nv, nk;
    int kneigh_out;        /* search2's flag after this structure               */
    int nonphysical_k;     /* count of (spin, k) with a non-PD overlap          */
    /* per-k outputs hold jspins blocks of nk rows, spin 1 first               */
    double *eig;           /* optional out [jspins][nk][nv] ascending eigenvalues*/
    double *deig;          /* optional out [jspins][nk][nv] dE_i/dV (modes 2, 4) */
    int *ncut;             /* optional out [jspins][nk] states <= eigcut         */
    int *k_status;         /* optional out [jspins][nk] NRLTB_K_*                */
    /* Gillan's free-energy extrapolation (bande.f:1409-1470), modes 1 and 2;
     * 0 in modes 3 and 4 */
    double entropy;        /* S(T), window states only (bande.f:1234)           */
    double free_energy;    /* A(T) = E(T) - kT S(T)                             */
    double entropy_shift;  /* -T dS/dV term (bande.f:1457), mode 2              */
    /* bande's two outputs, as SKENG prints them (bande.f:96-123):
     *   mode 1: E(0) = (E+A)/2, E(T)     mode 2: E(0), P(0) = P - shift/2
     *   mode 3: E(T), 0                  mode 4: E(T), P(T)                  */
    double earg1, earg2;
    double smag;           /* jspins = 2: spin-up minus spin-down electrons per */
                           /* cell (bande.f:1336-1395), SKENG's last column; 0  */
    double *spdir;         /* optional out [natoms][3], non-collinear runs with  */
                           /* NRLTB_OPT_SPIN_DIRECTIONS: each atom's spin vector */
                           /* summed over occupied states (diag.f:458-524,      */
                           /* bande.f:1480-1537), SPNDIR's columns              */
    double *orbocc;        /* optional out [jspins][nk][nv][nv], modes 5, 6, 10: */
                           /* [row][state n][orbital i] = |(S^1/2 z_n)_i|^2, the */
                           /* Lowdin charges of diag.f:526-700; -1 at a k whose  */
                           /* overlap is not positive definite                  */
} nrltb_result;

typedef struct nrltb_ctx nrltb_ctx;

/* ---- library and context ------------------------------------------------ */
int nrltb_abi_version(void);
const char *nrltb_last_error(void);
/* Create a context on one CUDA device: its stream, library-owned device
 * buffers, and four internal streams onto which the mixed form forks
 * independent work (the refinement's digits and the dH, dS Bloch sums during
 * the tridiagonalisation; the back-transform's WY factors during the
 * tridiagonal solve) and which it joins back with events, so that every call's
 * work stays ordered on the context's stream. */
int nrltb_ctx_create(nrltb_ctx **out, int device);
int nrltb_ctx_destroy(nrltb_ctx *ctx);
/* Run the context's work on a caller stream (cudaStream_t passed as void*), or
 * NULL for the context's own stream; the internal streams fork from and join
 * back to it. */
int nrltb_ctx_set_stream(nrltb_ctx *ctx, void *stream);
/* Number of kernels this library has launched through ctx (for accounting). */
long long nrltb_ctx_launch_count(const nrltb_ctx *ctx);

/* ---- per-structure drop-in (replaces bande, bande.f:1-4, and the search2 call
 *      before it, static.f:1114,1218) ------------------------------------- */
int nrltb_bande(nrltb_ctx *ctx, const nrltb_structure *st, const nrltb_params *par,
                const nrltb_kmesh *km, const nrltb_opts *opt, nrltb_result *res);

/* Many structures of uneven size in one call (the MPI k split becomes a batch).
 * Structures are processed concurrently by up to 8 host worker threads, each
 * with its own context and stream created on first use (kept until the
 * context is destroyed), largest structures first; each result equals what
 * nrltb_bande returns for that structure alone.  On error the first failing
 * structure's message is kept. */
int nrltb_bande_batch(nrltb_ctx *ctx, int nstruct, const nrltb_structure *st,
                      const nrltb_params *par, const nrltb_kmesh *km,
                      const nrltb_opts *opt, nrltb_result *res);

/* Split form of nrltb_bande for device-resident timing: upload the inputs,
 * run the path on the device with no host copies, download the results. */
int nrltb_stage(nrltb_ctx *ctx, const nrltb_structure *st, const nrltb_params *par,
                const nrltb_kmesh *km, const nrltb_opts *opt);
int nrltb_run(nrltb_ctx *ctx);
int nrltb_fetch(nrltb_ctx *ctx, nrltb_result *res);

/* ---- stage entry points (one per reference routine) -------------------- */
/* With jspins = 2 these compute spin channel 1 (jspin = 1 of setpar.f: the
 * first parameter set, the second for flipped atoms' densities and on-site
 * terms). */
/* search2.f:1-240 */
int nrltb_search2(nrltb_ctx *ctx, const nrltb_structure *st, const nrltb_params *par,
                  int kneigh_in, nrltb_pairs *out, int *kneigh_out, double *dismin);
/* setpar.f:1-891 and, if dhop != NULL, setparv.f:1-888 (for the given pair list) */
int nrltb_setpar(nrltb_ctx *ctx, const nrltb_structure *st, const nrltb_params *par,
                 const nrltb_pairs *pairs, double *hop, double *over, double *paros,
                 double *den, double *dhop, double *dover, double *dparos);
/* setham.f + rotate.f (which=0: H, S) or sethamv.f (which=1: dH/dV, dS/dV) for each
 * k of km; writes full Hermitian column-major complex matrices [nk][nv][nv] as
 * interleaved (re, im) doubles. */
int nrltb_setham(nrltb_ctx *ctx, const nrltb_structure *st, const nrltb_params *par,
                 const nrltb_kmesh *km, int which, double *hmat, double *smat);
/* diag.f:385-455 (zhpgv 'V','U'): nk generalized problems H z = e S z of order nv,
 * full column-major complex input; eigenvalues ascending into eig[nk][nv]; if z is
 * not NULL, S-orthonormal eigenvectors into z[nk][nv][nv]. */
int nrltb_diag(nrltb_ctx *ctx, int nv, int nk, const double *hmat, const double *smat,
               int precision, double *eig, double *z, int *k_status);
/* fermi.f:1-434, non-spin (el = 2): Fermi level of eig[nk][nv] with weights w. */
int nrltb_fermi(nrltb_ctx *ctx, int nv, int nk, const double *eig, const double *w,
                double tkb, double zfill, double tol, double *efermi);
/* fermi.f:1-434 and the sums of bande.f:1162-1330 on caller eigenvalues
 * eig[nk][nv] (ascending per row), weights w[nk], and in modes 2 and 4 the
 * eigenvalue derivatives deig[nk][nv] (all states below eigcut); el electrons
 * per band (2 spin-restricted, 1 one spin channel).  out = {E_F, E(T), P(T),
 * Fermi-level shift, S(T) (modes 1, 2), the two entropy-derivative sums
 * (mode 2), Newton iterations}.  Every sum is compensated. */
int nrltb_sums(nrltb_ctx *ctx, int nv, int nk, const double *eig, const double *deig, const double *w,
               int mode, double el, double tkb, double zfill, double tol, double out[8]);

/* ---- neighbour list without allocation ----------------------------------
 * No counterpart in the reference.  nrltb_search2 above sizes its buffers with
 * cudaMalloc; this variant is for callers that cannot allocate device memory
 * at call time -- codes whose own allocator already owns the GPU (a framework's
 * caching pool, an arena reserved at start-up), or whose pipeline must not be
 * stalled by the device-wide synchronisation a cudaMalloc/cudaFree can cause.
 * It performs no allocation: positions, kinds and the pair arrays are the
 * caller's device buffers (pair arrays of `capacity` entries, laid out as in
 * nrltb_pairs; every atom kind must lie in 1..kinds, others are refused with
 * NRLTB_E_ARG before the search reads them), and its scratch is a fixed device array of
 * NRLTB_NOALLOC_SCRATCH_BYTES that every GPU which loads the library keeps
 * until the process exits.  Search boxes with more than
 * NRLTB_NOALLOC_MAX_CANDIDATES candidate images (natoms^2 (2nd1+1)(2nd2+1)
 * (2nd3+1)) are rejected with NRLTB_E_CAPACITY.  The first call on a device
 * looks the scratch array up on that device; make that first call before any
 * stream capture.  All calls share the one array, so calls that overlap on the
 * GPU (different streams or host threads) race; serialise them.  The call runs
 * on `stream` (NULL = legacy default stream) and returns when the results are
 * written; *npairs gets the full pair count even when it exceeds capacity
 * (then NRLTB_E_CAPACITY is returned and only the first `capacity` pairs
 * are written). */
#define NRLTB_NOALLOC_MAX_CANDIDATES 16777216L
#define NRLTB_NOALLOC_SCRATCH_BYTES 16844288UL
int nrltb_search2_noalloc(int device, void *stream, int natoms, const int *d_kkind, const double *d_posn,
                          const double plv[3][3], const int nd[3], int kinds, const double *dnn,
                          const double *screenl, int kneigh_in, int capacity, double *d_tt, int *d_dlv,
                          double *d_dist, double *d_screen, double *d_dscrn, int *d_jkind, int *d_jatm,
                          int *npairs, int *kneigh_out, double *dismin);

#ifdef __cplusplus
}
#endif
#endif /* NRLTB_H */
