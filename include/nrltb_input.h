/*
 * nrltb_input.h -- C restatement of the reference's input API: the SKIN file
 * (static.f:697-1030), the NRL parameter file (input.f:137-359), the structure
 * block (input1.f:466-862), lattice construction (setlat.f:147-1024) and the
 * k-point list (kptin.f:66-366, explicit-list paths).  Host-only, no device.
 *
 * A SKIN handle owns every array that the returned structs point into; the
 * arrays of a structure stay valid until the next nrltb_skin_next call.
 */
#ifndef NRLTB_INPUT_H
#define NRLTB_INPUT_H
#include "nrltb.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct nrltb_skin nrltb_skin;

/* Open a SKIN file, read Mode= (static.f:706-708, modeparse.f), tkb and eigcut
 * (static.f:818) and the parameter file it names (input.f), resolved relative
 * to the SKIN file's directory. */
int nrltb_skin_open(const char *path, nrltb_skin **out);
/* Global settings of an open SKIN file.  par's arrays are owned by the handle. */
int nrltb_skin_info(const nrltb_skin *s, int *mode, double *tkb, double *eigcut,
                    nrltb_params *par);
/* Read the next structure: title, label, zcharge (static.f:938-950), input1.f,
 * setlat.f, the lattice-to-Cartesian step (static.f:1088-1103) and kptin.f.
 * With the spin-flip flag T on the (2a1) line each atom line carries magdir
 * and st->flip marks the atoms with magdir 2 (NULL when none is flipped); with
 * the non-collinear flags N, D, S it carries theta, phi and st->spinat holds
 * the unit directions.  Returns NRLTB_E_EOF
 * after the last structure.  title must hold 71 chars and label 21 (NUL
 * included). */
int nrltb_skin_next(nrltb_skin *s, nrltb_structure *st, nrltb_kmesh *km,
                    char *title, char *label);
/* The spin options of the structure nrltb_skin_next last read: flag S asks for
 * output spin directions (SPNDIR), flag D for torques (SKDERIV, which the
 * reference opens but never writes); both make the run non-collinear. */
#define NRLTB_SKIN_SPIN_DIRECTIONS 1
#define NRLTB_SKIN_TORQUES         2
int nrltb_skin_spin_options(const nrltb_skin *s);
/* Line number (1-based) of the SKIN file where the last error happened. */
int nrltb_skin_error_line(const nrltb_skin *s);
void nrltb_skin_close(nrltb_skin *s);

/* Parameter file alone (input.f:137-359).  A magnetic file ("M" as the header's
 * second letter) holds one parameter set per spin: par->jspins = 2 and
 * par->param has 2 nrltb_nparams(kinds) values. */
typedef struct nrltb_parfile nrltb_parfile;
int nrltb_parfile_read(const char *path, nrltb_parfile **out, nrltb_params *par);
void nrltb_parfile_close(nrltb_parfile *p);

/* Number of parameters for `kinds` species: kinds(29 + 68 kinds) (input.f:275). */
int nrltb_nparams(int kinds);

/* Eigenvalue files (static.f:759-781, 1132-1145; bande.f:1568-1700): append one
 * structure's records (append != 0) or start the file, for mode 6 or 10 (QLMT
 * with per-atom s, p, d or per-orbital Lowdin charges of the states below
 * eigcut; res->orbocc required), 9 (QLMT with every eigenvalue, no atoms) or 8
 * (QAPW, eigenvalues per k point).  res holds nrltb_bande's per-k arrays for
 * par->jspins spin blocks (one block of 2N columns for non-collinear spins,
 * whose charges go to 2 natoms pseudo-atoms, spin-down copies second); km is
 * the k list the structure was run on.  Mode 5
 * is not written: the reference mixes formatted records into its unformatted
 * QLMT and stops there. */
int nrltb_qlmt_write(const char *path, int append, int mode, const nrltb_structure *st,
                     const nrltb_params *par, const nrltb_kmesh *km, double eigcut,
                     const nrltb_result *res);

#ifdef __cplusplus
}
#endif
#endif
