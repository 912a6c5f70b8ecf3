/*
 * nrltb_qlmt.c -- the eigenvalue files of the reference's modes 6, 8, 9 and 10:
 * QLMT (LAPW-like: k points, eigenvalues below eigcut and per-atom s, p, d or
 * per-orbital Lowdin charges) and QAPW (eigenvalues per k point).  Records
 * and edit descriptors follow static.f:1132-1145 (the per-structure header)
 * and bande.f:1642-1697 (the k records written from diag.f's data,
 * diag.f:526-758).
 *
 * Fortran's F, E and D editing is reproduced here: F prints asterisks when the
 * value does not fit its field, E and D print a 0.ddd mantissa.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "nrltb.h"
#include "nrltb_input.h"

/* Fw.d */
static void put_f(FILE *f, double v, int w, int d)
{
    char b[64];
    int n = snprintf(b, sizeof b, "%*.*f", w, d, v);
    if (n > w) {
        for (int i = 0; i < w; ++i) fputc('*', f);
        return;
    }
    fputs(b, f);
}

/* Ew.d / Dw.d with a two-digit exponent: [-]0.ddd...E+xx, right-justified */
static void put_e(FILE *f, double v, int w, int d, char letter)
{
    char mant[64], out[80];
    int ex = 0;
    if (v == 0.0) {
        memset(mant, '0', (size_t)d);
        mant[d] = 0;
    } else {
        char t[64];
        snprintf(t, sizeof t, "%.*e", d - 1, fabs(v));   /* d significant digits: D.DDDe+XX */
        int j = 0;
        for (const char *p = t; *p && *p != 'e'; ++p)
            if (*p != '.') mant[j++] = *p;
        mant[j] = 0;
        ex = atoi(strchr(t, 'e') + 1) + 1;               /* 0.DDDD times 10^ex */
    }
    snprintf(out, sizeof out, "%s0.%s%c%c%02d", v < 0 ? "-" : "", mant, letter, ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
    fprintf(f, "%*s", w, out);
}

/* (3f10.6,2X,f10.5,i10,d20.10,' K'): k point, weight, number of states, weight */
static void put_krec(FILE *f, const double *k, double w, int ntot)
{
    for (int c = 0; c < 3; ++c) put_f(f, k[c], 10, 6);
    fputs("  ", f);
    put_f(f, w, 10, 5);
    fprintf(f, "%10d", ntot);
    put_e(f, w, 20, 10, 'D');
    fputs(" K\n", f);
}

int nrltb_qlmt_write(const char *path, int append, int mode, const nrltb_structure *st, const nrltb_params *par,
                     const nrltb_kmesh *km, double eigcut, const nrltb_result *res)
{
    if (!path || !st || !par || !km || !res || !res->eig || !st->kkind || !par->kbas) return NRLTB_E_ARG;
    if (!(mode == 6 || mode == 8 || mode == 9 || mode == 10)) return NRLTB_E_UNSUPPORTED;
    if ((mode == 6 || mode == 10) && !res->orbocc) return NRLTB_E_ARG;
    FILE *f = fopen(path, append ? "a" : "w");
    if (!f) return NRLTB_E_IO;
    /* a non-collinear run is one 2N x 2N problem per k, its charges on 2 natoms
     * pseudo-atoms: every atom's spin-up orbitals, then the spin-down copies
     * (diag.f:670-693) */
    const int noncol = st->spinat != NULL;
    const int nv = res->nv, nk = km->nk, nsp = (par->jspins == 2 && !noncol) ? 2 : 1;
    const int natx = noncol ? 2 * st->natoms : st->natoms;
    /* static.f:1138-1144: one header line per structure (spins written as 1) */
    if (mode == 6 || mode == 10) fprintf(f, "%5d%5d%5d%5d     SPINS, WIND., SC. WIND.\n", 1, 1, 0, st->natoms);
    else if (mode == 9) fprintf(f, "%5d%5d%5d%5d     SPINS, WIND., SC. WIND.\n", 1, 1, 0, 0);
    for (int js = 0; js < nsp; ++js)
        for (int k = 0; k < nk; ++k) {
            const int row = js * nk + k;
            const double *en = res->eig + (size_t)row * nv;
            const double *kq = km->k + 3 * (size_t)k;
            if (mode == 8) {   /* (1x,3f9.6,10x,4f9.5/(38x,4f9.5)) */
                fputc(' ', f);
                for (int c = 0; c < 3; ++c) put_f(f, kq[c], 9, 6);
                fputs("          ", f);
                for (int i = 0; i < nv; ++i) {
                    if (i > 0 && i % 4 == 0) fprintf(f, "\n%38s", "");
                    put_f(f, en[i], 9, 5);
                }
                fputc('\n', f);
                /* exactly four values: the slash after them still ends a record */
                if (nv == 4) fputc('\n', f);
                continue;
            }
            if (mode == 9) {   /* the k record, then (f12.7,e15.6) per state */
                put_krec(f, kq, km->w[k], nv);
                for (int i = 0; i < nv; ++i) {
                    put_f(f, en[i], 12, 7);
                    put_e(f, 0.0, 15, 6, 'E');
                    fputc('\n', f);
                }
                continue;
            }
            /* modes 6, 10: states up to the first above eigcut (diag.f:635-641);
             * a 1x1 problem always writes its one state (diag.f:354-357) */
            int ntot = nv;
            for (int i = 0; i < nv; ++i)
                if (en[i] > eigcut) { ntot = i; break; }
            if (nv == 1) ntot = 1;
            put_krec(f, kq, km->w[k], ntot);
            const double *orb = res->orbocc + (size_t)row * nv * nv;
            for (int n = 0; n < ntot; ++n) {
                const double e = en[n];
                if (mode == 6 && (e <= -10.0 || e >= 100.0)) put_f(f, e, 10, 6);
                else put_f(f, e, 10, 7);
                put_e(f, 0.0, 15, 6, 'E');
                fputc('\n', f);
                const double *oc = orb + (size_t)n * nv;
                int i0 = 0;
                for (int a = 0; a < natx; ++a) {
                    const int nbas = par->kbas[st->kkind[a % st->natoms] - 1];
                    if (mode == 6) {   /* s, p, d sums (diag.f:705-721), then 0 */
                        double s = oc[i0], p = 0.0, d = 0.0;
                        for (int q = 1; q < (nbas < 4 ? nbas : 4); ++q) p = p + oc[i0 + q];
                        for (int q = 4; q < nbas; ++q) d = d + oc[i0 + q];
                        put_f(f, s, 15, 9);
                        put_f(f, p, 15, 9);
                        put_f(f, d, 15, 9);
                        put_f(f, 0.0, 15, 9);
                    } else {           /* every orbital (diag.f:727-731) */
                        for (int q = 0; q < nbas; ++q) put_f(f, oc[i0 + q], 15, 9);
                    }
                    fputc('\n', f);
                    i0 += nbas;
                }
            }
        }
    int rc = ferror(f) ? NRLTB_E_IO : NRLTB_OK;
    if (fclose(f)) rc = NRLTB_E_IO;
    return rc;
}
