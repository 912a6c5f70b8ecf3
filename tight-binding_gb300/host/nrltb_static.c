/*
 * nrltb_static.c -- the C host driver: the structure loop of the reference's
 * "static" program (static.f:919-1259) on top of the GPU k-point path.
 *
 *   nrltb_static [--precision fp64|mixed] [--device N] [--fermi-tol T] [SKIN]
 *
 * Reads the SKIN file (default ./SKIN) and the parameter and k-point files it
 * names with the C readers (nrltb_input.h), then for every structure calls
 * nrltb_bande -- the drop-in for search2 + bande (static.f:1114, 1218) -- and
 * appends one line to SKENG in the reference's format (static.f:1238-1254) and
 * a summary block to SKOUT (bande.f:1405-1476 wording); in modes 6, 8, 9, 10
 * the QLMT / QAPW records (bande.f:1568-1700), for spin flag S the SPNDIR lines
 * (bande.f:1545-1560), for flag D an SKDERIV file, which the reference opens
 * and never writes.  Output files go to the current directory, as in the
 * reference.  search2's carried kneigh flag passes from one structure to the
 * next as the reference's common block does.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "nrltb.h"
#include "nrltb_input.h"

static void usage(void)
{
    fprintf(stderr, "usage: nrltb_static [--precision fp64|mixed] [--device N] [--fermi-tol T] [SKIN]\n");
}

int main(int argc, char **argv)
{
    const char *skin_path = "SKIN";
    int precision = NRLTB_PREC_FP64, device = 0;
    double fermi_tol = 0.0;
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "--precision") && i + 1 < argc) {
            ++i;
            if (!strcmp(argv[i], "fp64")) precision = NRLTB_PREC_FP64;
            else if (!strcmp(argv[i], "mixed")) precision = NRLTB_PREC_MIXED;
            else { usage(); return 2; }
        } else if (!strcmp(argv[i], "--device") && i + 1 < argc) {
            device = atoi(argv[++i]);
        } else if (!strcmp(argv[i], "--fermi-tol") && i + 1 < argc) {
            fermi_tol = atof(argv[++i]);
        } else if (argv[i][0] == '-') {
            usage();
            return 2;
        } else {
            skin_path = argv[i];
        }
    }
    nrltb_skin *skin = NULL;
    int rc = nrltb_skin_open(skin_path, &skin);
    if (rc != NRLTB_OK) {
        fprintf(stderr, "nrltb_static: cannot read %s (error %d)\n", skin_path, rc);
        return 1;
    }
    int mode;
    double tkb, eigcut;
    nrltb_params par;
    nrltb_skin_info(skin, &mode, &tkb, &eigcut, &par);
    /* mode 7 stops the reference (static.f:732-743); its mode 5 writes formatted
     * records into an unformatted QLMT and stops there (bande.f:1631-1640) */
    if (mode < 1 || mode > 10 || mode == 5 || mode == 7) {
        fprintf(stderr, "nrltb_static: Mode=%d is not built (modes 1-4, 6 and 8-10 are)\n", mode);
        nrltb_skin_close(skin);
        return 1;
    }
    nrltb_ctx *ctx = NULL;
    rc = nrltb_ctx_create(&ctx, device);
    if (rc != NRLTB_OK) {
        fprintf(stderr, "nrltb_static: no GPU context: %s\n", nrltb_last_error());
        nrltb_skin_close(skin);
        return 1;
    }
    FILE *skout = fopen("SKOUT", "w"), *skeng = fopen("SKENG", "w");
    if (!skout || !skeng) {
        fprintf(stderr, "nrltb_static: cannot write SKOUT/SKENG\n");
        return 1;
    }
    fprintf(skout, " mode=%12d\n", mode);
    fprintf(skout, "  temp. broad. (ryd): %.17G  eigenvalue cutoff = %.17G\n", tkb, eigcut);
    fprintf(skout, " precision form: %s\n", precision == NRLTB_PREC_FP64 ? "FP64" : "mixed (FP32 + FP64 refinement)");
    /* static.f:759-781: QLMT for modes 6, 9, 10, QAPW for mode 8, one file for
     * every structure */
    const char *qfile = (mode == 8) ? "QAPW" : (mode == 6 || mode == 9 || mode == 10) ? "QLMT" : NULL;
    FILE *spndir = NULL;   /* static.f:1012-1017: SPNDIR for flag S, SKDERIV for flag D */
    int kneigh = 0, jstruc = 0, status = 0;
    for (;;) {
        nrltb_structure st;
        nrltb_kmesh km;
        char title[72], label[24];
        rc = nrltb_skin_next(skin, &st, &km, title, label);
        if (rc == NRLTB_E_EOF) break;
        if (rc != NRLTB_OK) {
            fprintf(stderr, "nrltb_static: SKIN error %d near line %d\n", rc, nrltb_skin_error_line(skin));
            status = 1;
            break;
        }
        ++jstruc;
        nrltb_opts opt;
        memset(&opt, 0, sizeof opt);
        opt.mode = mode;
        opt.precision = precision;
        opt.tkb = tkb;
        opt.eigcut = eigcut;
        opt.fermi_tol = fermi_tol;
        opt.kneigh_in = kneigh;
        const int spinopt = nrltb_skin_spin_options(skin);
        if (spinopt & NRLTB_SKIN_SPIN_DIRECTIONS) opt.flags |= NRLTB_OPT_SPIN_DIRECTIONS;
        if (spinopt & NRLTB_SKIN_TORQUES) {   /* opened, never written, as in the reference */
            FILE *fd = fopen("SKDERIV", "a");
            if (fd) fclose(fd);
        }
        nrltb_result res;
        memset(&res, 0, sizeof res);
        double *spdir = (spinopt & NRLTB_SKIN_SPIN_DIRECTIONS) ? malloc(sizeof(double) * 3 * (size_t)st.natoms) : NULL;
        if ((spinopt & NRLTB_SKIN_SPIN_DIRECTIONS) && !spdir) {
            fprintf(stderr, "nrltb_static: structure %d: out of host memory\n", jstruc);
            status = 1;
            break;
        }
        res.spdir = spdir;
        const int nsp = (par.jspins == 2) ? 2 : 1;
        size_t nv = 0;
        for (int i = 0; i < st.natoms; ++i) nv += (size_t)par.kbas[st.kkind[i] - 1];
        double *eigbuf = NULL, *orbbuf = NULL;
        if (qfile) {
            eigbuf = malloc(sizeof(double) * nv * (size_t)km.nk * nsp);
            if (mode == 6 || mode == 10) orbbuf = malloc(sizeof(double) * nv * nv * (size_t)km.nk * nsp);
            if (!eigbuf || ((mode == 6 || mode == 10) && !orbbuf)) {
                fprintf(stderr, "nrltb_static: structure %d: out of host memory\n", jstruc);
                free(eigbuf); free(orbbuf); free(spdir);
                status = 1;
                break;
            }
            res.eig = eigbuf;
            res.orbocc = orbbuf;
        }
        rc = nrltb_bande(ctx, &st, &par, &km, &opt, &res);
        if (rc == NRLTB_OK && qfile) {
            rc = nrltb_qlmt_write(qfile, jstruc > 1, mode, &st, &par, &km, eigcut, &res);
            if (rc != NRLTB_OK) fprintf(stderr, "nrltb_static: cannot write %s (error %d)\n", qfile, rc);
        }
        free(eigbuf);
        free(orbbuf);
        if (rc != NRLTB_OK) {
            free(spdir);
            if (rc != NRLTB_E_IO) fprintf(stderr, "nrltb_static: structure %d: %s\n", jstruc, nrltb_last_error());
            status = 1;
            break;
        }
        kneigh = res.kneigh_out;
        fprintf(skout, "-------------------------------\n\nstructure %5d\n\n%s\n\n", jstruc, title);
        fprintf(skout, " Minimum distance this configuration = %.17G\n", res.dismin);
        fprintf(skout, "Number of pairs = %6d\n", res.npairs);
        fprintf(skout, " Secular equation size = %12d\n", res.nv);
        fprintf(skout, " Volume= %.17G\n", st.volume);
        if (res.nonphysical_k)
            fprintf(skout, " Found non-physical overlap at %d k-points\n", res.nonphysical_k);
        fprintf(skout, " Temperature = %.17G\n", tkb);
        fprintf(skout, " EFermi = %.17G\n", res.efermi);
        fprintf(skout, " E(T) = %.17G\n", res.e_total);
        if (mode < 3) {   /* bande.f:1409-1420 */
            fprintf(skout, " S(T) = %.17G\n", res.entropy);
            fprintf(skout, " A(T) = %.17G\n", res.free_energy);
            fprintf(skout, " E(0) = %.17G + O[T**4]\n", res.earg1);
        }
        if (mode == 2 || mode == 4) {   /* bande.f:1430-1476 */
            fprintf(skout, " Fermi level shift: %.17G\n", res.fermi_shift);
            fprintf(skout, " P(T) = %.17G\n", res.pressure);
            if (mode == 2) {
                fprintf(skout, " Entropy shift = %.17G\n", res.entropy_shift);
                fprintf(skout, " P_A(T) = %.17G\n", res.pressure - res.entropy_shift);
                fprintf(skout, " P(0) = %.17G + O[T**4]\n", res.earg2);
            }
        }
        if (res.spdir && st.spinat) {   /* bande.f:1545-1560, (a20,i5,4f10.6,2f12.6) */
            if (!spndir) spndir = fopen("SPNDIR", "w");
            for (int i = 0; spndir && i < st.natoms; ++i) {
                const double *v = spdir + 3 * i;
                const double sm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                const double rad2deg = 180.0 / 3.14159265358979323846;
                fprintf(spndir, "%-20.20s%5d%10.6f%10.6f%10.6f%10.6f%12.6f%12.6f\n", label, i + 1, v[0], v[1], v[2], sm,
                        rad2deg * acos(v[2] / sm), rad2deg * atan2(v[1], v[0]));
            }
            if (spndir) fflush(spndir);
        }
        free(spdir);
        if (par.jspins == 2 && !st.spinat)   /* bande.f:1390-1394; none for a non-collinear run */
            fprintf(skout, "for a total magnetization of %10.5f electrons per unit cell.\n", res.smag);
        /* static.f:1238-1254: E_F and bande's two outputs (mode 3 has one), then
         * the moment for a collinear spin-polarized set */
        char tail[32] = "";
        if (par.jspins == 2 && !st.spinat) snprintf(tail, sizeof tail, "%10.6f", res.smag);   /* static.f:1238 */
        if (mode == 3 || mode > 4)
            fprintf(skeng, "%-20.20s%12.6f%15.9f%15.9f%s\n", label, st.volume, res.efermi, res.earg1, tail);
        else
            fprintf(skeng, "%-20.20s%12.6f%15.9f%15.9f%15.9f%s\n", label, st.volume, res.efermi, res.earg1,
                    res.earg2, tail);
        fflush(skeng);
        fflush(skout);
    }
    fclose(skout);
    fclose(skeng);
    if (spndir) fclose(spndir);
    nrltb_ctx_destroy(ctx);
    nrltb_skin_close(skin);
    return status;
}
