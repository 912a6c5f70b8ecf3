/*
 * nrltb_input.c -- readers for the reference's SKIN, parameter and k-point files.
 *
 * Restates the Fortran reads of static.f:697-1030, input.f:137-359,
 * input1.f:466-862, setlat.f:147-1024 and kptin.f:66-366, including their
 * formatted-field rules: the SKIN file is opened with blank='zero'
 * (static.f:682), so blanks inside I/F fields read from it count as zeros,
 * while the k-point and parameter files use the default (blanks ignored).
 * List-directed reads start on a new line, may continue onto following lines,
 * and drop the rest of the last line once their list is satisfied.
 */
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "nrltb.h"
#include "nrltb_input.h"

#define LINE_MAX_LEN 1024

typedef struct {
    FILE *f;
    int line;
    char buf[LINE_MAX_LEN];
} lreader;

static int lr_open(lreader *r, const char *path)
{
    r->f = fopen(path, "r");
    r->line = 0;
    return r->f ? 0 : -1;
}
static void lr_close(lreader *r) { if (r->f) fclose(r->f); r->f = NULL; }

/* next record, newline stripped; 0 ok, -1 EOF */
static int lr_next(lreader *r)
{
    if (!r->f || !fgets(r->buf, sizeof r->buf, r->f)) return -1;
    r->line++;
    size_t n = strlen(r->buf);
    if (n == sizeof(r->buf) - 1 && r->buf[n - 1] != '\n') {
        int c; /* drop the tail of an over-long record */
        while ((c = fgetc(r->f)) != EOF && c != '\n') {}
    }
    while (n && (r->buf[n - 1] == '\n' || r->buf[n - 1] == '\r')) r->buf[--n] = 0;
    return 0;
}

/* column slice [c0, c0+w) of the current record, blank padded */
static void field(const char *rec, int c0, int w, char *out)
{
    int n = (int)strlen(rec);
    for (int i = 0; i < w; ++i) out[i] = (c0 + i < n) ? rec[c0 + i] : ' ';
    out[w] = 0;
}

/* Fortran I edit descriptor; bz: blanks are zeros */
static int fmt_int(const char *fld, int bz, long *v)
{
    char t[64];
    int n = 0, any = 0;
    for (const char *p = fld; *p && n < 62; ++p) {
        if (*p == ' ') { if (bz && any) t[n++] = '0'; continue; }
        if (!(isdigit((unsigned char)*p) || *p == '-' || *p == '+')) return -1;
        t[n++] = *p; any = 1;
    }
    t[n] = 0;
    if (!any) { *v = 0; return 0; }
    char *e;
    *v = strtol(t, &e, 10);
    return *e ? -1 : 0;
}

/* Fortran Fw.d edit descriptor */
static int fmt_real(const char *fld, int d, int bz, double *v)
{
    char t[96];
    int n = 0, any = 0, dot = 0, exp = 0;
    for (const char *p = fld; *p && n < 94; ++p) {
        char c = *p;
        if (c == ' ') { if (bz && any && !exp) t[n++] = '0'; continue; }
        if (c == 'd' || c == 'D' || c == 'e' || c == 'E') { c = 'e'; exp = 1; }
        if (c == '.') dot = 1;
        t[n++] = c; any = 1;
    }
    t[n] = 0;
    if (!any) { *v = 0; return 0; }
    char *e;
    double x = strtod(t, &e);
    if (*e) return -1;
    if (!dot && !exp) x = x / pow(10.0, d);
    *v = x;
    return 0;
}

/* ---- list-directed reads ------------------------------------------------ */
typedef struct { lreader *r; char *p; int started; } ldctx;

static int ld_token(ldctx *c, char *tok, int maxlen)
{
    for (;;) {
        if (!c->started) {
            if (lr_next(c->r)) return -1;
            c->p = c->r->buf;
            c->started = 1;
        }
        while (*c->p && (isspace((unsigned char)*c->p) || *c->p == ',')) c->p++;
        if (*c->p == '/') return -2; /* slash ends the read, remaining items unchanged */
        if (!*c->p) { c->started = 0; continue; }
        int n = 0;
        while (*c->p && !isspace((unsigned char)*c->p) && *c->p != ',' && *c->p != '/' && n < maxlen - 1)
            tok[n++] = *c->p++;
        tok[n] = 0;
        return 0;
    }
}

static int tok_real(const char *tok, double *v)
{
    char t[96];
    int n = 0;
    for (const char *p = tok; *p && n < 94; ++p) t[n++] = (*p == 'd' || *p == 'D') ? 'e' : *p;
    t[n] = 0;
    char *e;
    *v = strtod(t, &e);
    return (*e || e == t) ? -1 : 0;
}

static int tok_int(const char *tok, long *v)
{
    char *e;
    *v = strtol(tok, &e, 10);
    return (*e || e == tok) ? -1 : 0;
}

static int tok_logical(const char *tok, int *v)
{
    const char *p = tok;
    if (*p == '.') ++p;
    if (*p == 'T' || *p == 't') { *v = 1; return 0; }
    if (*p == 'F' || *p == 'f') { *v = 0; return 0; }
    return -1;
}

/* read n reals with one list-directed READ */
static int ld_reals(lreader *r, int n, double *out)
{
    ldctx c = {r, NULL, 0};
    char tok[128];
    for (int i = 0; i < n; ++i) {
        int rc = ld_token(&c, tok, sizeof tok);
        if (rc == -2) return 0;
        if (rc) return -1;
        if (tok_real(tok, &out[i])) return -2;
    }
    return 0;
}
static int ld_ints(lreader *r, int n, long *out)
{
    ldctx c = {r, NULL, 0};
    char tok[128];
    for (int i = 0; i < n; ++i) {
        int rc = ld_token(&c, tok, sizeof tok);
        if (rc == -2) return 0;
        if (rc) return -1;
        if (tok_int(tok, &out[i])) return -2;
    }
    return 0;
}

/* ---- parameter file (input.f:137-359) ---------------------------------- */
struct nrltb_parfile {
    int kinds, jsover, nltype, jspins;
    int kbas[16];
    double valence[16], dnn[136], screenl[136];
    double *param;
    int nparam;
    char title[80];
};

int nrltb_nparams(int kinds) { return kinds * (29 + 68 * kinds); }

int nrltb_parfile_read(const char *path, nrltb_parfile **out, nrltb_params *par)
{
    lreader r;
    if (lr_open(&r, path)) return NRLTB_E_IO;
    nrltb_parfile *p = (nrltb_parfile *)calloc(1, sizeof *p);
    int rc = NRLTB_E_PARSE;
    char fld[16];
    long iv;
    if (lr_next(&r)) goto fail;
    /* '(2a1,i5)': basis type, magnetic type, nltype (input.f:181) */
    char ov = r.buf[0] ? r.buf[0] : ' ', mag = (r.buf[0] && r.buf[1]) ? r.buf[1] : ' ';
    field(r.buf, 2, 5, fld);
    if (fmt_int(fld, 0, &iv)) goto fail;
    p->nltype = (int)iv;
    p->jsover = !(ov == 'O' || ov == 'o');
    p->jspins = (mag == 'M' || mag == 'm') ? 2 : 1;   /* input.f:213-229 */
    if (p->nltype != 90000 && (p->nltype > 3 || p->nltype < 0)) p->nltype = 0; /* input.f:239-242 */
    if (lr_next(&r)) goto fail;
    field(r.buf, 0, 79, p->title);
    if (ld_ints(&r, 1, &iv)) goto fail;
    p->kinds = (int)iv;
    if (p->kinds < 1 || p->kinds > 16) goto fail;
    int nint = p->kinds * (p->kinds + 1) / 2;
    for (int i = 0; i < nint; ++i) {
        double v[2];
        if (ld_reals(&r, 2, v)) goto fail;
        p->dnn[i] = v[0];
        p->screenl[i] = v[1];
    }
    for (int i = 0; i < p->kinds; ++i) {
        double occ[3], wt;
        if (ld_ints(&r, 1, &iv)) goto fail;
        p->kbas[i] = (int)iv;
        if (ld_reals(&r, 1, &wt)) goto fail;
        if (ld_reals(&r, 3, occ)) goto fail;
        p->valence[i] = occ[0] + occ[1] + occ[2];
    }
    /* one set per spin, read in sequence (input.f:327-358) */
    int npards = nrltb_nparams(p->kinds) * p->jspins;
    p->param = (double *)calloc((size_t)npards, sizeof(double));
    if (!p->param) { rc = NRLTB_E_NOMEM; goto fail; }
    p->nparam = npards;
    for (int i = 0; i < npards; ++i) {
        /* a short file leaves the remaining parameters zero (input.f:330-351) */
        if (ld_reals(&r, 1, &p->param[i])) { p->nparam = i; break; }
    }
    lr_close(&r);
    par->kinds = p->kinds;
    par->jsover = p->jsover;
    par->nltype = p->nltype;
    par->kbas = p->kbas;
    par->valence = p->valence;
    par->dnn = p->dnn;
    par->screenl = p->screenl;
    par->param = p->param;
    par->jspins = p->jspins;
    *out = p;
    return NRLTB_OK;
fail:
    lr_close(&r);
    free(p->param);
    free(p);
    return rc;
}

void nrltb_parfile_close(nrltb_parfile *p)
{
    if (!p) return;
    free(p->param);
    free(p);
}

/* ---- SKIN handle -------------------------------------------------------- */
struct nrltb_skin {
    lreader r;
    char dir[1024];
    int mode;
    double tkb, eigcut;
    nrltb_parfile *pf;
    nrltb_params par;
    /* current structure */
    int natoms;
    int *kkind, *flip;
    double *posn, *posq, *spinat;
    int spinopt;   /* NRLTB_SKIN_* of the current structure */
    /* k list, kept across structures (kptin.f `save nk`) */
    int nk;
    double *kq, *kw;
    int errline;
};

static void join_path(const char *dir, const char *name, char *out, size_t n)
{
    if (name[0] == '/' || !dir[0]) snprintf(out, n, "%s", name);
    else snprintf(out, n, "%s/%s", dir, name);
}

static void rtrim(char *s)
{
    size_t n = strlen(s);
    while (n && isspace((unsigned char)s[n - 1])) s[--n] = 0;
}

int nrltb_skin_open(const char *path, nrltb_skin **out)
{
    nrltb_skin *s = (nrltb_skin *)calloc(1, sizeof *s);
    if (!s) return NRLTB_E_NOMEM;
    snprintf(s->dir, sizeof s->dir, "%s", path);
    char *slash = strrchr(s->dir, '/');
    if (slash) *slash = 0; else s->dir[0] = 0;
    if (lr_open(&s->r, path)) { free(s); return NRLTB_E_IO; }
    int rc = NRLTB_E_PARSE;
    char fld[8];
    /* '(5x,a2)' Mode=NN, modeparse.f */
    if (lr_next(&s->r)) goto fail;
    field(s->r.buf, 5, 2, fld);
    {
        int d[2];
        for (int j = 0; j < 2; ++j) d[j] = isdigit((unsigned char)fld[j]) ? fld[j] - '0' : -1;
        if (d[0] < 0) d[0] = 0;
        s->mode = d[1] < 0 ? d[0] : 10 * d[0] + d[1];
    }
    double v[2];
    if (ld_reals(&s->r, 2, v)) goto fail;
    s->tkb = v[0];
    s->eigcut = v[1];
    /* '(a79)' parameter file name (input.f:137) */
    if (lr_next(&s->r)) goto fail;
    char name[96], full[1200];
    field(s->r.buf, 0, 79, name);
    rtrim(name);
    join_path(s->dir, name, full, sizeof full);
    rc = nrltb_parfile_read(full, &s->pf, &s->par);
    if (rc) goto fail;
    *out = s;
    return NRLTB_OK;
fail:
    s->errline = s->r.line;
    lr_close(&s->r);
    free(s);
    return rc;
}

int nrltb_skin_info(const nrltb_skin *s, int *mode, double *tkb, double *eigcut, nrltb_params *par)
{
    if (!s) return NRLTB_E_ARG;
    if (mode) *mode = s->mode;
    if (tkb) *tkb = s->tkb;
    if (eigcut) *eigcut = s->eigcut;
    if (par) *par = s->par;
    return NRLTB_OK;
}

int nrltb_skin_spin_options(const nrltb_skin *s) { return s ? s->spinopt : 0; }

int nrltb_skin_error_line(const nrltb_skin *s) { return s ? s->errline : 0; }

/* setlat.f:147-1000: lattice types 0-16 (and their volume forms, latnum < 0)
 * and the elastic strain options 0, 1, +-2, +-21, +-3, 4, 5, 6.  alat[i][j]
 * is the jth Cartesian component of the ith primitive vector (setlat.f's
 * alat(i,j)). */
static int read_setlat(lreader *r, double alat[3][3], double *vol)
{
    long latnum = 0;
    double a, b, c, v[9], theta, cellv;
    double scale[3] = {1, 1, 1};
    memset(alat, 0, sizeof(double) * 9);
    if (ld_ints(r, 1, &latnum)) return NRLTB_E_PARSE;
    const double half = 0.5, third = 1.0 / 3.0;
    const double fac1 = 0.866025403784438647, fac2 = 1.0 / fac1;
    switch (labs(latnum)) {
    case 0:
        if (ld_reals(r, 9, v)) return NRLTB_E_PARSE;
        for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) alat[i][j] = v[3 * i + j];
        if (ld_reals(r, 3, scale)) return NRLTB_E_PARSE;
        for (int i = 0; i < 3; ++i) if (scale[i] == 0.0) scale[i] = 1.0;
        break;
    case 1:
        if (ld_reals(r, 1, &a)) return NRLTB_E_PARSE;
        if (latnum < 0) a = pow(4.0 * fabs(a), third);
        for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) if (i != j) alat[j][i] = half * a;
        break;
    case 2:
        if (ld_reals(r, 1, &a)) return NRLTB_E_PARSE;
        if (latnum < 0) a = pow(2.0 * fabs(a), third);
        for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) alat[j][i] = (i == j) ? -half * a : half * a;
        break;
    case 3:
        if (ld_reals(r, 2, v)) return NRLTB_E_PARSE;
        if (latnum > 0) { a = v[0]; c = v[1]; }
        else { a = pow(fac2 * fabs(v[0]) / fabs(v[1]), third); c = fabs(v[1]) * a; }
        alat[0][0] = half * a; alat[1][0] = alat[0][0];
        alat[0][1] = -fac1 * a; alat[1][1] = -alat[0][1];
        alat[2][2] = c;
        break;
    case 4:
        if (ld_reals(r, 1, &a)) return NRLTB_E_PARSE;
        if (latnum < 0) a = pow(fabs(a), third);
        for (int i = 0; i < 3; ++i) alat[i][i] = a;
        break;
    case 5:
        if (ld_reals(r, 2, v)) return NRLTB_E_PARSE;
        if (latnum > 0) { a = v[0]; c = v[1]; }
        else { a = pow(fabs(v[0]) / fabs(v[1]), third); c = v[1] * a; }
        alat[0][0] = a; alat[1][1] = a; alat[2][2] = c;
        break;
    case 6:   /* body-centered tetragonal (setlat.f:347-371) */
        if (ld_reals(r, 2, v)) return NRLTB_E_PARSE;
        if (latnum > 0) { a = v[0]; c = v[1]; }
        else { a = pow(2.0 * fabs(v[0]) / fabs(v[1]), third); c = v[1] * a; }
        alat[0][0] = a; alat[1][1] = a;
        alat[2][0] = half * a; alat[2][1] = half * a; alat[2][2] = half * c;
        break;
    case 7:
        if (ld_reals(r, 3, v)) return NRLTB_E_PARSE;
        if (latnum > 0) { a = v[0]; b = v[1]; c = v[2]; }
        else { a = pow(fabs(v[0]) / fabs(v[1] * v[2]), third); b = v[1] * a; c = v[2] * a; }
        alat[0][0] = a; alat[1][1] = b; alat[2][2] = c;
        break;
    case 8:   /* base-centered orthorhombic: (a/2, -b/2, 0), (a/2, b/2, 0), (0, 0, c) */
        if (ld_reals(r, 3, v)) return NRLTB_E_PARSE;
        if (latnum > 0) { a = v[0]; b = v[1]; c = v[2]; }
        else { a = pow(fabs(2.0 * v[0]) / fabs(v[1] * v[2]), third); b = v[1] * a; c = v[2] * a; }
        alat[0][0] = half * a; alat[1][0] = half * a;
        alat[1][1] = half * b; alat[0][1] = -half * b;
        alat[2][2] = c;
        break;
    case 9:   /* simple tetragonal with in-plane vectors along (110), (1-10) */
    case 10:  /* face-centered tetragonal, the same in-plane vectors */
        if (ld_reals(r, 2, v)) return NRLTB_E_PARSE;
        if (latnum > 0) { a = v[0]; c = v[1]; }
        else { a = pow(fabs((labs(latnum) == 9 ? 2.0 : 4.0) * v[0] / v[1]), third); c = v[1] * a; }
        alat[0][0] = half * a; alat[0][1] = -half * a;
        alat[1][0] = half * a; alat[1][1] = half * a;
        if (labs(latnum) == 9) alat[2][2] = c;
        else { alat[2][0] = half * a; alat[2][2] = half * c; }
        break;
    case 11:  /* fcc-like face-centered tetragonal */
        if (ld_reals(r, 2, v)) return NRLTB_E_PARSE;
        if (latnum > 0) { a = v[0]; c = v[1]; }
        else { a = pow(4.0 * fabs(v[0]) / fabs(v[1]), third); c = v[1] * a; }
        alat[1][0] = half * a; alat[2][0] = half * a;
        alat[0][1] = half * a; alat[2][1] = half * a;
        alat[0][2] = half * c; alat[1][2] = half * c;
        break;
    case 12:  /* rhombohedral (a, b, b), (b, a, b), (b, b, a); or V and the angle */
        if (ld_reals(r, 2, v)) return NRLTB_E_PARSE;
        if (latnum > 0) { a = v[0]; b = v[1]; }
        else {
            const double ct = cos(v[1]);   /* cosine of the angle between the vectors */
            if (ct < -half) return NRLTB_E_PARSE;   /* setlat.f stops: angle too large */
            const double bo = third * (sqrt((1.0 + 2.0 * ct) / (1.0 - ct)) - 1.0);
            c = pow(fabs(v[0]) / (1.0 + 3.0 * bo), third);
            a = c * (1.0 + bo);
            b = c * bo;
        }
        for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) alat[j][i] = (i == j) ? a : b;
        break;
    case 13:  /* bcc-like body-centered tetragonal */
        if (ld_reals(r, 2, v)) return NRLTB_E_PARSE;
        if (latnum > 0) { a = v[0]; c = v[1]; }
        else { a = pow(2.0 * fabs(v[0]) / fabs(v[1]), third); c = v[1] * a; }
        alat[0][0] = -half * a; alat[0][1] = half * a; alat[0][2] = half * c;
        alat[1][0] = half * a; alat[1][1] = -half * a; alat[1][2] = half * c;
        alat[2][0] = half * a; alat[2][1] = half * a; alat[2][2] = -half * c;
        break;
    case 14:  /* base-centered orthorhombic from a, c and the in-plane angle */
        if (ld_reals(r, 3, v)) return NRLTB_E_PARSE;
        theta = v[2];
        if (latnum > 0) { a = v[0]; c = v[1]; }
        else { a = pow(v[0] / (v[1] * sin(theta)), third); c = a * v[1]; }
        theta = half * theta;
        alat[0][0] = a * cos(theta); alat[0][1] = -a * sin(theta);
        alat[1][0] = alat[0][0]; alat[1][1] = -alat[0][1];
        alat[2][2] = c;
        break;
    case 15:  /* "magic strain" lattices around fcc: w (0, y, z), (x, 0, z), (x, y, 0) */
    case 16:  /* ... around bcc: w (-x, y, z), (x, -y, z), (x, y, -z) */
    {
        if (ld_reals(r, 3, v)) return NRLTB_E_PARSE;
        const int fcc_based = labs(latnum) == 15;
        const double rm = v[1], tpi3 = 2.0 * 3.14159265358979323846 / 3.0;
        theta = v[2];
        if (latnum > 0) cellv = (fcc_based ? half : 0.25) * v[0] * v[0] * v[0];   /* from a_bcc or a_fcc */
        else cellv = v[0];
        const double w = pow((fcc_based ? half : 0.25) * cellv, third), sg = fcc_based ? -1.0 : 1.0;
        const double x = w * exp(sg * rm * cos(theta + tpi3)), y = w * exp(sg * rm * cos(theta - tpi3));
        const double z = w * exp(sg * rm * cos(theta));
        if (fcc_based) {
            alat[0][1] = y; alat[0][2] = z;
            alat[1][0] = x; alat[1][2] = z;
            alat[2][0] = x; alat[2][1] = y;
        } else {
            alat[0][0] = -x; alat[0][1] = y; alat[0][2] = z;
            alat[1][0] = x; alat[1][1] = -y; alat[1][2] = z;
            alat[2][0] = x; alat[2][1] = y; alat[2][2] = -z;
        }
        break;
    }
    default:
        return NRLTB_E_UNSUPPORTED;
    }
    /* elastic strains (setlat.f:862-978): the explicit e_i or one of the
     * one-parameter menus */
    long strain = 0;
    if (ld_ints(r, 1, &strain)) return NRLTB_E_PARSE;
    if (strain != 0) {
        double e[6] = {0, 0, 0, 0, 0, 0}, x, x2;
        switch (strain) {
        case 1:
            if (ld_reals(r, 6, e)) return NRLTB_E_PARSE;
            break;
        case 2: case -2: case 21: case -21:
            /* volume-conserving e1 = sqrt((1+x)/(1-x)) - 1, e2 = sqrt((1-x)/(1+x)) - 1, or
             * e1 = x, e2 = -x, e3 = x^2/(1-x^2); +-2 read x^2, +-21 read x */
            if (ld_reals(r, 1, &x)) return NRLTB_E_PARSE;
            if (labs(strain) == 2) { x2 = x; x = sqrt(x2); } else x2 = x * x;
            if (strain > 0) { e[0] = sqrt((1.0 + x) / (1.0 - x)) - 1.0; e[1] = sqrt((1.0 - x) / (1.0 + x)) - 1.0; }
            else { e[0] = x; e[1] = -x; e[2] = x2 / (1.0 - x2); }
            break;
        case 3: case -3:   /* read x^2 = e6^2 */
            if (ld_reals(r, 1, &x2)) return NRLTB_E_PARSE;
            e[5] = sqrt(x2);
            if (strain > 0) { e[0] = sqrt(1.0 + 0.25 * x2) - 1.0; e[1] = e[0]; }
            else e[2] = x2 / (4.0 - x2);
            break;
        case 4:   /* c/a changed by 1 + x at constant volume */
            if (ld_reals(r, 1, &x)) return NRLTB_E_PARSE;
            e[0] = pow(1.0 + x, -third) - 1.0;
            e[1] = e[0];
            e[2] = pow(1.0 + x, 2.0 / 3.0) - 1.0;
            break;
        case 5:   /* [111] strain of the Cartesian unit vectors */
            if (ld_reals(r, 1, &x)) return NRLTB_E_PARSE;
            e[0] = (1.0 + x) * pow(1.0 + 3.0 * x, -third) - 1.0;
            e[1] = e[0];
            e[2] = e[0];
            e[3] = 2.0 * x * pow(1.0 + 3.0 * x, -third);
            e[4] = e[3];
            e[5] = e[4];
            break;
        case 6:   /* hexagonal C44 strain: e4 = x, e3 = x^2/4 (x < 0 when x^2 is entered negative) */
            if (ld_reals(r, 1, &x2)) return NRLTB_E_PARSE;
            x = x2 < 0 ? -sqrt(fabs(x2)) : sqrt(x2);
            e[3] = x;
            e[2] = 0.25 * x * x;
            break;
        default:
            return NRLTB_E_PARSE;   /* setlat.f: unknown strain type */
        }
        double est[3][3] = {{1 + e[0], half * e[5], half * e[4]},
                            {half * e[5], 1 + e[1], half * e[3]},
                            {half * e[4], half * e[3], 1 + e[2]}};
        double as[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double sum = 0;
                for (int k = 0; k < 3; ++k) sum = sum + alat[j][k] * est[k][i];
                as[j][i] = sum;
            }
        memcpy(alat, as, sizeof as);
    }
    if (latnum == 0)
        for (int j = 0; j < 3; ++j) for (int i = 0; i < 3; ++i) alat[i][j] = alat[i][j] * scale[j];
    *vol = fabs(alat[0][0] * (alat[1][1] * alat[2][2] - alat[2][1] * alat[1][2]) +
                alat[1][0] * (alat[2][1] * alat[0][2] - alat[0][1] * alat[2][2]) +
                alat[2][0] * (alat[0][1] * alat[1][2] - alat[1][1] * alat[0][2]));
    if (*vol == 0.0) return NRLTB_E_PARSE;
    return NRLTB_OK;
}

/* ---- k-point mesh generator (kptin.f:90-150, rdspgp.f, kptgen.f, mapk.f,
 * gdot.f, hsort.f, matmlt.f).  Matrices are kept with the Fortran indices:
 * m[i][j] is M(i+1, j+1); sums run in the Fortran routines' order. */
static const double KG_TPI = 2.0 * 3.14159265358979323846;

/* C = A B in matmlt.f's order: c(i,k) = a(i,j) b(j,k) + c(i,k), j ascending */
static void kg_matmlt(const double a[3][3], const double b[3][3], double c[3][3])
{
    for (int i = 0; i < 3; ++i) for (int k = 0; k < 3; ++k) c[i][k] = 0.0;
    for (int k = 0; k < 3; ++k)
        for (int j = 0; j < 3; ++j) {
            const double sv = b[j][k];
            for (int i = 0; i < 3; ++i) c[i][k] = a[i][j] * sv + c[i][k];
        }
}

/* gdot.f: a^T G b, inner sum over i first */
static double kg_gdot(const double a[3], const double b[3], const double g[3][3])
{
    double d = 0.0;
    for (int j = 0; j < 3; ++j) {
        double sum = 0.0;
        for (int i = 0; i < 3; ++i) sum = sum + a[i] * g[i][j];
        d = d + sum * b[j];
    }
    return d;
}

/* hsort.f: heap sort of a[0..n-1] into the index list ind (1-based values) */
static void kg_hsort(int n, const double *a, int *ind)
{
    for (int j = 1; j <= n; ++j) ind[j - 1] = j;
    if (n <= 1) return;
    int l = n / 2 + 1, ir = n, indxt;
    double q;
    for (;;) {
        if (l > 1) {
            l = l - 1;
            indxt = ind[l - 1];
            q = a[indxt - 1];
        } else {
            indxt = ind[ir - 1];
            q = a[indxt - 1];
            ind[ir - 1] = ind[0];
            ir = ir - 1;
            if (ir == 1) { ind[0] = indxt; return; }
        }
        int i = l, j = l + l;
        while (j <= ir) {
            if (j < ir && a[ind[j - 1] - 1] < a[ind[j] - 1]) j = j + 1;
            if (q < a[ind[j - 1] - 1]) {
                ind[i - 1] = ind[j - 1];
                i = j;
                j = j + j;
            } else {
                j = ir + 1;
            }
        }
        ind[i - 1] = indxt;
    }
}

/* kptin.f:94-136: AVEC(I,J) = PLV(J,I), the reciprocal vectors BVEC (column j
 * = b_j) and the metric BIJ; returns the cell volume |A . B| */
static double kg_recip(const double plv[3][3], double avec[3][3], double bvec[3][3], double bij[3][3])
{
    double A[9], B[9];
    int l = 0;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) { avec[i][j] = plv[j][i]; A[l++] = avec[i][j]; }
    B[0] = A[4] * A[8] - A[5] * A[7];
    B[1] = A[5] * A[6] - A[3] * A[8];
    B[2] = A[3] * A[7] - A[4] * A[6];
    B[3] = A[7] * A[2] - A[8] * A[1];
    B[4] = A[8] * A[0] - A[6] * A[2];
    B[5] = A[6] * A[1] - A[7] * A[0];
    B[6] = A[1] * A[5] - A[2] * A[4];
    B[7] = A[2] * A[3] - A[0] * A[5];
    B[8] = A[0] * A[4] - A[1] * A[3];
    double ws = A[0] * B[0] + A[1] * B[1] + A[2] * B[2];
    const double pre = KG_TPI / ws;
    l = 0;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) bvec[i][j] = pre * B[l++];
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) bij[j][i] = 0.0;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) bij[i][j] = bvec[k][i] * bvec[k][j] + bij[i][j];
    return fabs(ws);
}

/* rdspgp.f: the space group's rotations in reciprocal-lattice coordinates
 * (RSPCT), from a file giving them in direct-lattice (ilat) or Cartesian
 * coordinates; the non-primitive translations are not needed here */
static int kg_spacegroup(const char *path, int ilat, int lattic, const double avec[3][3], const double bvec[3][3],
                         int *nop, double (**rspct)[3][3])
{
    lreader g;
    if (lr_open(&g, path)) return NRLTB_E_IO;
    int rc = NRLTB_OK;
    char fld[64];
    double (*rc_t)[3][3] = NULL;
    if (lr_next(&g)) { rc = NRLTB_E_PARSE; goto out; }
    long n;
    field(g.buf, 10, 5, fld);                        /* (A10,I5,5X,3F10.5) */
    if (fmt_int(fld, 1, &n) || n <= 0) { rc = NRLTB_E_PARSE; goto out; }
    double (*rspc)[3][3] = malloc(sizeof(double) * 9 * n);
    rc_t = malloc(sizeof(double) * 9 * n);
    const double tpiinv = 1.0 / KG_TPI;
    double t[3][3], tinv[3][3], work[3][3];
    if (ilat) {
        /* (18F4.0): (((RSPDIR(I,J,K),J=1,3),I=1,3),K=1,NOP); RSPC = TINV RSPDIR T */
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) { t[i][j] = bvec[j][i] * tpiinv; tinv[i][j] = avec[i][j]; }
        long got = 0, tot = 9 * n;
        double *dir = malloc(sizeof(double) * tot);
        while (got < tot) {
            if (lr_next(&g)) { free(dir); free(rspc); rc = NRLTB_E_PARSE; goto out; }
            for (int f = 0; f < 18 && got < tot; ++f) {
                field(g.buf, 4 * f, 4, fld);
                if (fmt_real(fld, 0, 1, &dir[got])) { free(dir); free(rspc); rc = NRLTB_E_PARSE; goto out; }
                ++got;
            }
        }
        for (long k = 0; k < n; ++k) {
            double rd[3][3];
            for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) rd[i][j] = dir[9 * k + 3 * i + j];
            kg_matmlt(rd, t, work);
            kg_matmlt(tinv, work, rspc[k]);
        }
        free(dir);
    } else {
        /* (3D20.10) per row: ((RSPC(I,J,K),J=1,3),I=1,3) */
        for (long k = 0; k < n; ++k)
            for (int i = 0; i < 3; ++i) {
                if (lr_next(&g)) { free(rspc); rc = NRLTB_E_PARSE; goto out; }
                for (int j = 0; j < 3; ++j) {
                    field(g.buf, 20 * j, 20, fld);
                    if (fmt_real(fld, 10, 1, &rspc[k][i][j])) { free(rspc); rc = NRLTB_E_PARSE; goto out; }
                }
            }
        if (lattic == 4) {   /* hexagonal: snap +-sqrt(3)/2 */
            const double c32 = sqrt(3.0) / 2.0;
            for (long k = 0; k < n; ++k)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        if (fabs(rspc[k][i][j] - c32) < 0.001) rspc[k][i][j] = c32;
                        if (fabs(rspc[k][i][j] + c32) < 0.001) rspc[k][i][j] = -c32;
                    }
        }
    }
    /* RSPCT = T RSPC TINV with T(I,J) = AVEC(J,I)/2pi, TINV = BVEC */
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { t[i][j] = avec[j][i] / KG_TPI; tinv[i][j] = bvec[i][j]; }
    for (long k = 0; k < n; ++k) {
        kg_matmlt(rspc[k], tinv, work);
        kg_matmlt(t, work, rc_t[k]);
    }
    free(rspc);
    *nop = (int)n;
    *rspct = rc_t;
    rc_t = NULL;
out:
    free(rc_t);
    lr_close(&g);
    return rc;
}

/* kptgen.f: the mesh of kdiv divisions (special points when lspec) reduced to
 * the irreducible wedge: points shifted to the Wigner-Seitz cell, sorted by
 * |k| (hsort), grouped in shells of radius within 1e-4, each merged with an
 * earlier point of its shell that a rotation (plus a reciprocal lattice
 * vector, or the time reversal k -> -k) maps onto it.  Returns the
 * irreducible points (reciprocal-lattice coordinates) and weights. */
/* full-zone mesh points kg_generate accepts (about 161^3) */
#define KG_MAX_POINTS 4194304L

static int kg_generate(const double plv[3][3], int lattic, int nop, double (*rspct)[3][3], int lspec,
                       const long kpdiv[3], double **q_out, double **w_out, int *nk_out)
{
    double avec[3][3], bvec[3][3], bij[3][3];
    const double wsvol = kg_recip(plv, avec, bvec, bij);
    const int lbcc = lattic == 2, lhex = lattic == 4, ltet = lattic == 7 || lattic == 8 || lattic == 9;
    double alat = 0.0;
    if (lbcc) {   /* bcc: the mesh of the simple cubic cell */
        alat = pow(2.0 * wsvol, 0.33333333333333333);
        alat = 2.0 * KG_TPI / alat;
    }
    long kdiv1 = kpdiv[0], kdiv2 = kpdiv[1], kdiv3 = kpdiv[2], max1, max2, max3;
    if (kdiv1 <= 0 || kdiv2 <= 0 || kdiv3 <= 0) return NRLTB_E_PARSE;
    if (ltet) { kdiv1 = 2 * kdiv1; kdiv2 = 2 * kdiv2; }
    if (lspec) {
        if (lhex) {
            max1 = kdiv1 + kdiv1 % 2;
            max2 = max1;
            if (kdiv1 != kdiv2) return NRLTB_E_PARSE;   /* kptgen.f stops: KDIV error for hex */
        } else {
            max1 = kdiv1 + 1;
            max2 = kdiv2 + 1;
        }
        max3 = kdiv3 + 1;
    } else {
        max1 = kdiv1; max2 = kdiv2; max3 = kdiv3;
    }
    /* kptgen.f:141-145 stops when the full-zone mesh passes its array bound
     * (2 nkd points); the bound here is KG_MAX_POINTS, checked before any work */
    if (max1 >= KG_MAX_POINTS || max2 >= KG_MAX_POINTS || max3 >= KG_MAX_POINTS ||
        (max1 + 1) * (max2 + 1) > KG_MAX_POINTS || (max1 + 1) * (max2 + 1) * (max3 + 1) > KG_MAX_POINTS)
        return NRLTB_E_UNSUPPORTED;
    const long cnt = (max1 + 1) * (max2 + 1) * (max3 + 1);
    double *rk = malloc(sizeof(double) * 3 * cnt), *rad = malloc(sizeof(double) * cnt);
    char *lin = malloc(cnt);
    int *index = malloc(sizeof(int) * cnt), *ist = malloc(sizeof(int) * (cnt + 2));
    double *srk = malloc(sizeof(double) * 3 * cnt), *srad = malloc(sizeof(double) * cnt);
    double *q = malloc(sizeof(double) * 3 * cnt), *w = malloc(sizeof(double) * cnt);
    if (!rk || !rad || !lin || !index || !ist || !srk || !srad || !q || !w) {
        free(rk); free(rad); free(lin); free(index); free(ist); free(srk); free(srad); free(q); free(w);
        return NRLTB_E_NOMEM;
    }
    const double f1 = 0.5 / (double)kdiv1, f2 = 0.5 / (double)kdiv2, f3 = 0.5 / (double)kdiv3;
    const double tpiinv = 1.0 / KG_TPI;
    long nk = 0, kin = 0;
    for (long ii = -max1; ii <= max1; ii += 2)
        for (long jj = -max2; jj <= max2; jj += 2)
            for (long kk = -max3; kk <= max3; kk += 2) {
                double uk[3] = {f1 * (double)ii, f2 * (double)jj, f3 * (double)kk}, u[3];
                if (lattic == 7 || lattic == 8 || lattic == 9) {
                    uk[0] = (double)ii / (double)kdiv1;
                    uk[1] = (double)jj / (double)kdiv2;
                    if (lattic == 7) uk[2] = uk[2] + 0.5 * (uk[0] - uk[1]);
                    else if (lattic == 8) uk[2] = uk[2] + 0.5 * uk[0];
                    else uk[2] = uk[2] + 0.5 * (uk[0] + uk[1]);
                }
                u[0] = uk[0]; u[1] = uk[1]; u[2] = uk[2];
                lin[nk] = ii <= kdiv1 && ii > -kdiv1 && jj <= kdiv2 && jj > -kdiv2 && kk <= kdiv3 && kk > -kdiv3;
                if (lin[nk]) ++kin;
                if (lbcc) {   /* Cartesian point -> reciprocal-lattice coordinates (mapk.f, inv = 1) */
                    double uu[3];
                    for (int j = 0; j < 3; ++j) uu[j] = uk[j] * alat;
                    for (int j = 0; j < 3; ++j)
                        u[j] = (uu[0] * avec[0][j] + uu[1] * avec[1][j] + uu[2] * avec[2][j]) * tpiinv;
                }
                /* the shortest equivalent vector, among shifts by -3..3 reciprocal vectors */
                double r2 = 1e50, ut[3] = {0, 0, 0};
                for (int i1 = -3; i1 <= 3; ++i1)
                    for (int i2 = -3; i2 <= 3; ++i2)
                        for (int i3 = -3; i3 <= 3; ++i3) {
                            const double uu[3] = {u[0] + i1, u[1] + i2, u[2] + i3};
                            const double rr = kg_gdot(uu, uu, bij);
                            if (rr <= r2) { r2 = rr; ut[0] = uu[0]; ut[1] = uu[1]; ut[2] = uu[2]; }
                        }
                rk[3 * nk] = ut[0]; rk[3 * nk + 1] = ut[1]; rk[3 * nk + 2] = ut[2];
                rad[nk] = r2;
                ++nk;
            }
    kg_hsort((int)nk, rad, index);
    for (long j = 0; j < nk; ++j) {
        srad[j] = rad[index[j] - 1];
        for (int c = 0; c < 3; ++c) srk[3 * j + c] = rk[3 * (index[j] - 1) + c];
    }
    const double f = 1.0 / (double)kin, toler = 1e-4;
    double r2 = srad[0] + toler;
    int nst = 1;
    ist[0] = 1;
    for (long j = 2; j <= nk; ++j)
        if (srad[j - 1] > r2) { r2 = srad[j - 1] + toler; ist[nst++] = (int)j; }
    ist[nst] = (int)nk + 1;
    int novk = 0;
    for (int sh = 0; sh < nst; ++sh) {
        const int k1 = novk + 1;
        for (int j = ist[sh]; j <= ist[sh + 1] - 1; ++j) {
            int ieq = 0;
            const double xx = srk[3 * (j - 1)], yy = srk[3 * (j - 1) + 1], zz = srk[3 * (j - 1) + 2];
            for (int k = k1; k <= novk; ++k) {
                const double *u = q + 3 * (k - 1);
                for (int iox = 0; iox < nop; ++iox) {
                    const double (*r)[3] = rspct[iox];
                    for (int i1 = -1; i1 <= 1; ++i1) {
                        const double x = r[0][0] * u[0] + r[0][1] * u[1] + r[0][2] * u[2] + (double)i1;
                        for (int i2 = -1; i2 <= 1; ++i2) {
                            const double y = r[1][0] * u[0] + r[1][1] * u[1] + r[1][2] * u[2] + (double)i2;
                            for (int i3 = -1; i3 <= 1; ++i3) {
                                const double z = r[2][0] * u[0] + r[2][1] * u[1] + r[2][2] * u[2] + (double)i3;
                                if (fabs(x - xx) + fabs(y - yy) + fabs(z - zz) <= 1e-4) ieq = k;
                                if (ieq == 0 && fabs(x + xx) + fabs(y + yy) + fabs(z + zz) <= 1e-4) ieq = k;
                            }
                        }
                    }
                }
            }
            const int inmesh = lin[index[j - 1] - 1];
            if (ieq == 0) {
                ++novk;
                q[3 * (novk - 1)] = xx; q[3 * (novk - 1) + 1] = yy; q[3 * (novk - 1) + 2] = zz;
                w[novk - 1] = inmesh ? f : 0.0;
            } else if (inmesh) {
                w[ieq - 1] = w[ieq - 1] + f;
            }
        }
    }
    free(rk); free(rad); free(lin); free(index); free(ist); free(srk); free(srad);
    *q_out = q;
    *w_out = w;
    *nk_out = novk;
    return NRLTB_OK;
}

/* kptin.f:66-366: the explicit-list (-1313 file, inline list), path (999) and
 * generated-mesh (NKV <= 0, kptgen.f) forms */
static int read_kpoints(nrltb_skin *s, const double plv[3][3])
{
    lreader *r = &s->r;
    char fld[300];
    if (lr_next(r)) return NRLTB_E_PARSE;
    field(r->buf, 7, 1, fld);
    int newsym = (fld[0] == 'T' || fld[0] == 't');
    if (!newsym) return s->nk > 0 ? NRLTB_OK : NRLTB_E_PARSE;
    if (lr_next(r)) return NRLTB_E_PARSE;           /* (7x,I1) LATTIC */
    long lattic = 0;
    field(r->buf, 7, 1, fld);
    if (fmt_int(fld, 1, &lattic)) return NRLTB_E_PARSE;
    if (lr_next(r)) return NRLTB_E_PARSE;           /* (A) space group file */
    char sg[300], full[1400], sgpath[1400];
    field(r->buf, 0, 255, sg);
    rtrim(sg);
    join_path(s->dir, sg, sgpath, sizeof sgpath);
    {
        FILE *f = fopen(sgpath, "r");                /* OPEN(25,...,STATUS='OLD') */
        if (!f) return NRLTB_E_IO;
        fclose(f);
    }
    if (lr_next(r)) return NRLTB_E_PARSE;           /* (5x,L1) ILAT */
    field(r->buf, 5, 1, fld);
    const int ilat = (fld[0] == 'T' || fld[0] == 't');
    if (lr_next(r)) return NRLTB_E_PARSE;           /* (I5,2F10.6) NKV, SFK */
    long nkv;
    double sfk;
    field(r->buf, 0, 5, fld);
    if (fmt_int(fld, 1, &nkv)) return NRLTB_E_PARSE;
    field(r->buf, 5, 10, fld);
    if (fmt_real(fld, 6, 1, &sfk)) return NRLTB_E_PARSE;
    lreader kr, *kio = r;
    int own = 0;
    if (nkv == -1313) {
        if (lr_next(r)) return NRLTB_E_PARSE;
        char kf[300];
        field(r->buf, 0, 255, kf);
        rtrim(kf);
        join_path(s->dir, kf, full, sizeof full);
        if (lr_open(&kr, full)) return NRLTB_E_IO;
        kio = &kr;
        own = 1;
        if (lr_next(kio)) { lr_close(&kr); return NRLTB_E_PARSE; }
        field(kio->buf, 0, 5, fld);
        if (fmt_int(fld, 0, &nkv)) { lr_close(&kr); return NRLTB_E_PARSE; }
        field(kio->buf, 5, 10, fld);
        if (fmt_real(fld, 6, 0, &sfk)) { lr_close(&kr); return NRLTB_E_PARSE; }
    }
    if (sfk <= 1e-6) sfk = 1.0;
    int rc = NRLTB_OK;
    if (nkv <= 0) {
        /* generated mesh: (6X,L1,8X,L1) LSPEC, LINFOK; (5I5) KPDIV1-3, KPST, KPEND */
        if (lr_next(kio)) { rc = NRLTB_E_PARSE; goto done; }
        field(kio->buf, 6, 1, fld);
        const int lspec = (fld[0] == 'T' || fld[0] == 't');
        field(kio->buf, 15, 1, fld);
        const int linfok = (fld[0] == 'T' || fld[0] == 't');
        if (lr_next(kio)) { rc = NRLTB_E_PARSE; goto done; }
        long kp[5];
        for (int i = 0; i < 5; ++i) {
            field(kio->buf, 5 * i, 5, fld);
            if (fmt_int(fld, 1, &kp[i])) { rc = NRLTB_E_PARSE; goto done; }
        }
        double avec[3][3], bvec[3][3], bij[3][3];
        kg_recip(plv, avec, bvec, bij);
        int nop = 0;
        double (*rspct)[3][3] = NULL;
        if ((rc = kg_spacegroup(sgpath, ilat, (int)lattic, avec, bvec, &nop, &rspct))) goto done;
        double *q = NULL, *w = NULL;
        int nk = 0;
        rc = kg_generate(plv, (int)lattic, nop, rspct, lspec, kp, &q, &w, &nk);
        free(rspct);
        if (rc) goto done;
        if (linfok) {   /* information-only points: weight 0 */
            const long ninfo = -nkv;
            if (ninfo > KG_MAX_POINTS) { free(q); free(w); rc = NRLTB_E_UNSUPPORTED; goto done; }
            double *q2 = realloc(q, sizeof(double) * 3 * (nk + ninfo));
            if (q2) q = q2;
            double *w2 = q2 ? realloc(w, sizeof(double) * (nk + ninfo)) : NULL;
            if (w2) w = w2;
            if (!q2 || !w2) { free(q); free(w); rc = NRLTB_E_NOMEM; goto done; }
            for (long i = 0; i < ninfo; ++i) {
                double v[3];
                if (ld_reals(kio, 3, v)) { free(q); free(w); rc = NRLTB_E_PARSE; goto done; }
                for (int j = 0; j < 3; ++j) q[3 * nk + j] = v[j] / sfk;
                w[nk++] = 0.0;
            }
        }
        double wsum = 0.0;
        for (int i = 0; i < nk; ++i) wsum = wsum + w[i];
        if (fabs(wsum - 1.0) > 1e-6) {
            const double wi = 1.0 / wsum;
            for (int i = 0; i < nk; ++i) w[i] = w[i] * wi;
        }
        long kpst = kp[3] <= 0 ? 1 : kp[3], kpend = kp[4] == 0 ? nk : kp[4];
        if (kpst > 1 || kpend < nk) {   /* keep points KPST..KPEND, renormalised */
            if (kpend > nk || kpst > kpend) { free(q); free(w); rc = NRLTB_E_PARSE; goto done; }
            int m = 0;
            wsum = 0.0;
            for (long i = kpst; i <= kpend; ++i) {
                w[m] = w[i - 1];
                wsum = wsum + w[m];
                for (int j = 0; j < 3; ++j) q[3 * m + j] = q[3 * (i - 1) + j];
                ++m;
            }
            nk = m;
            wsum = 1.0 / wsum;
        }
        for (int i = 0; i < nk; ++i) w[i] = w[i] * wsum;   /* kptin.f's final WGHTK*WGHTS */
        free(s->kq); free(s->kw);
        s->kq = q; s->kw = w; s->nk = nk;
        goto done;
    }
    if (nkv == 999) {
        /* path mode: segments of KD equally spaced points, weight 1 each */
        long kpdir;
        if (lr_next(kio)) { rc = NRLTB_E_PARSE; goto done; }
        field(kio->buf, 0, 5, fld);
        if (fmt_int(fld, !own, &kpdir)) { rc = NRLTB_E_PARSE; goto done; }
        long cap = 1024, nk = 0;
        double *q = malloc(sizeof(double) * 3 * cap), *w = malloc(sizeof(double) * cap);
        if (!q || !w) { free(q); free(w); rc = NRLTB_E_NOMEM; goto done; }
        for (long d = 0; d < kpdir; ++d) {
            double v[7];
            if (ld_reals(kio, 7, v)) { free(q); free(w); rc = NRLTB_E_PARSE; goto done; }
            if (!(v[0] > -1e9 && v[0] <= (double)KG_MAX_POINTS) || nk + (long)v[0] > KG_MAX_POINTS) {
                free(q); free(w); rc = NRLTB_E_UNSUPPORTED; goto done;
            }
            int kd = (int)v[0];
            if (nk + kd + 1 > cap) {
                cap = 2 * (nk + kd + 1);
                double *q2 = realloc(q, sizeof(double) * 3 * cap);
                if (q2) q = q2;
                double *w2 = q2 ? realloc(w, sizeof(double) * cap) : NULL;
                if (w2) w = w2;
                if (!q2 || !w2) { free(q); free(w); rc = NRLTB_E_NOMEM; goto done; }
            }
            double el[3];
            for (int i = 0; i < 3; ++i) el[i] = (v[4 + i] - v[1 + i]) / (double)(kd - 1);
            for (int i = 0; i < 3; ++i) q[3 * nk + i] = v[1 + i];
            w[nk++] = 1.0;
            for (int kk = 2; kk <= kd; ++kk) {
                for (int i = 0; i < 3; ++i) q[3 * nk + i] = q[3 * (nk - 1) + i] + el[i];
                w[nk++] = 1.0;
            }
        }
        for (long i = 0; i < nk; ++i) w[i] = w[i] * (double)nk; /* WGHTS = NK here */
        free(s->kq); free(s->kw);
        s->kq = q; s->kw = w; s->nk = (int)nk;
    } else {
        if (nkv > KG_MAX_POINTS) { rc = NRLTB_E_UNSUPPORTED; goto done; }
        double *q = malloc(sizeof(double) * 3 * nkv), *w = malloc(sizeof(double) * nkv);
        if (!q || !w) { free(q); free(w); rc = NRLTB_E_NOMEM; goto done; }
        double wsum = 0;
        for (long i = 0; i < nkv; ++i) {
            double v[4];
            if (ld_reals(kio, 4, v)) { free(q); free(w); rc = NRLTB_E_PARSE; goto done; }
            for (int j = 0; j < 3; ++j) q[3 * i + j] = v[j] / sfk;
            w[i] = v[3];
            wsum = wsum + w[i];
        }
        wsum = 1.0 / wsum;
        for (long i = 0; i < nkv; ++i) w[i] = w[i] * wsum;
        free(s->kq); free(s->kw);
        s->kq = q; s->kw = w; s->nk = (int)nkv;
    }
done:
    if (own) lr_close(&kr);
    return rc;
}

int nrltb_skin_next(nrltb_skin *s, nrltb_structure *st, nrltb_kmesh *km, char *title, char *label)
{
    if (!s || !st || !km) return NRLTB_E_ARG;
    lreader *r = &s->r;
    int rc = NRLTB_E_PARSE;
    char fld[80];
    if (lr_next(r)) return NRLTB_E_EOF;
    field(r->buf, 0, 70, fld);
    if (title) { memcpy(title, fld, 71); }
    if (lr_next(r)) return NRLTB_E_EOF;
    field(r->buf, 0, 20, fld);
    if (label) { memcpy(label, fld, 21); }
    double zcharge;
    if (ld_reals(r, 1, &zcharge)) return NRLTB_E_EOF;
    double plv[3][3], vol;
    rc = read_setlat(r, plv, &vol);
    if (rc) goto fail;
    long iv[3] = {0, 0, 0};
    rc = NRLTB_E_PARSE;
    if (ld_ints(r, 1, iv)) goto fail;
    int natoms = (int)labs(iv[0]);
    if (natoms < 1) goto fail;
    if (ld_ints(r, 3, iv)) goto fail;
    int nd[3] = {(int)iv[0], (int)iv[1], (int)iv[2]};
    if (lr_next(r)) goto fail;                     /* '(2a1)' lphonon, spin flag */
    char c1 = r->buf[0] ? r->buf[0] : ' ', c2 = (r->buf[0] && r->buf[1]) ? r->buf[1] : ' ';
    int lphonon = (c1 == 'T' || c1 == 't');
    /* input1.f:535-546: T spin flips (a magdir per atom); N, D, S non-collinear
     * runs (not built); anything else plain */
    /* D (torques) and S (spin directions) imply N (input1.f:535-546) */
    int spinflip = (c2 == 'T' || c2 == 't');
    int noncol = (c2 == 'N' || c2 == 'n' || c2 == 'D' || c2 == 'd' || c2 == 'S' || c2 == 's');
    s->spinopt = (c2 == 'S' || c2 == 's') ? NRLTB_SKIN_SPIN_DIRECTIONS : (c2 == 'D' || c2 == 'd') ? NRLTB_SKIN_TORQUES : 0;
    /* reciprocal vectors without 2 pi (input1.f:612-624) */
    double bvec[3][3];
    for (int i = 0; i < 3; ++i) {
        int i1 = (i + 1) % 3, i2 = (i1 + 1) % 3;
        for (int j = 0; j < 3; ++j) {
            int j1 = (j + 1) % 3, j2 = (j1 + 1) % 3;
            bvec[i][j] = (plv[i1][j1] * plv[i2][j2] - plv[i1][j2] * plv[i2][j1]) / vol;
        }
    }
    int *shift = calloc((size_t)natoms, sizeof(int));
    double *epsl = calloc(3 * (size_t)natoms, sizeof(double));
    if (lphonon) {
        long nshift = 0;
        if (ld_ints(r, 1, &nshift) || nshift > natoms) { free(shift); free(epsl); goto fail; }
        for (long k = 0; k < nshift; ++k) {
            ldctx c = {r, NULL, 0};
            char tok[128];
            long ia;
            int lc;
            double e[3];
            if (ld_token(&c, tok, sizeof tok) || tok_int(tok, &ia) || ia < 1 || ia > natoms) { free(shift); free(epsl); goto fail; }
            if (ld_token(&c, tok, sizeof tok) || tok_logical(tok, &lc)) { free(shift); free(epsl); goto fail; }
            for (int i = 0; i < 3; ++i)
                if (ld_token(&c, tok, sizeof tok) || tok_real(tok, &e[i])) { free(shift); free(epsl); goto fail; }
            shift[ia - 1] = 1;
            if (lc) {
                for (int i = 0; i < 3; ++i) {
                    double sum = 0;
                    for (int j = 0; j < 3; ++j) sum = sum + e[j] * bvec[i][j];
                    epsl[3 * (ia - 1) + i] = sum;
                }
            } else {
                for (int i = 0; i < 3; ++i) epsl[3 * (ia - 1) + i] = e[i];
            }
        }
    }
    free(s->kkind); free(s->flip); free(s->spinat); free(s->posn); free(s->posq);
    s->natoms = natoms;
    s->kkind = malloc(sizeof(int) * natoms);
    s->flip = calloc((size_t)natoms, sizeof(int));
    s->spinat = calloc(3 * (size_t)natoms, sizeof(double));
    s->posn = malloc(sizeof(double) * 3 * natoms);
    s->posq = malloc(sizeof(double) * 3 * natoms);
    if (!s->kkind || !s->flip || !s->spinat || !s->posn || !s->posq) {
        free(shift); free(epsl); rc = NRLTB_E_NOMEM; goto fail;
    }
    int anyflip = 0;
    const double deg2rad = 3.14159265358979323846 / 180.0;
    for (int i = 0; i < natoms; ++i) {
        double v[9];
        if (ld_reals(r, noncol ? 9 : spinflip ? 8 : 7, v)) { free(shift); free(epsl); goto fail; }
        if (spinflip) {   /* input1.f:778-787: magdir 2 flips the atom */
            s->flip[i] = (v[7] == 2.0);
            anyflip |= s->flip[i];
        }
        if (noncol) {     /* unit vector from theta, phi in degrees (input1.f:760-762) */
            s->spinat[3 * i] = sin(deg2rad * v[7]) * cos(deg2rad * v[8]);
            s->spinat[3 * i + 1] = sin(deg2rad * v[7]) * sin(deg2rad * v[8]);
            s->spinat[3 * i + 2] = cos(deg2rad * v[7]);
        }
        int kind = (int)v[0];
        double p[3] = {v[1], v[2], v[3]};
        if (kind < 0) {
            kind = -kind;
            double vl[3];
            for (int a = 0; a < 3; ++a) {
                double sum = 0;
                for (int b = 0; b < 3; ++b) sum = sum + bvec[a][b] * p[b];
                vl[a] = sum;
            }
            for (int a = 0; a < 3; ++a) p[a] = vl[a];
        }
        if (kind < 1 || kind > s->par.kinds) { free(shift); free(epsl); goto fail; }
        if (lphonon && shift[i]) for (int j = 0; j < 3; ++j) p[j] = p[j] + epsl[3 * i + j];
        s->kkind[i] = kind;
        /* lattice to Cartesian, static.f:1088-1103 */
        for (int c = 0; c < 3; ++c) {
            double t = 0;
            for (int j = 0; j < 3; ++j) t = t + plv[j][c] * p[j];
            s->posn[3 * i + c] = t;
        }
        for (int c = 0; c < 3; ++c) s->posq[3 * i + c] = v[4 + c];
    }
    free(shift);
    free(epsl);
    rc = read_kpoints(s, plv);
    if (rc) goto fail;
    memset(st, 0, sizeof *st);
    st->natoms = natoms;
    st->kkind = s->kkind;
    st->posn = s->posn;
    st->posq = s->posq;
    st->flip = anyflip ? s->flip : NULL;
    st->spinat = noncol ? s->spinat : NULL;
    memcpy(st->plv, plv, sizeof plv);
    memcpy(st->nd, nd, sizeof nd);
    st->volume = vol;
    st->zcharge = zcharge;
    km->nk = s->nk;
    km->k = s->kq;
    km->w = s->kw;
    return NRLTB_OK;
fail:
    s->errline = r->line;
    return rc;
}

void nrltb_skin_close(nrltb_skin *s)
{
    if (!s) return;
    lr_close(&s->r);
    nrltb_parfile_close(s->pf);
    free(s->kkind); free(s->flip); free(s->spinat); free(s->posn); free(s->posq); free(s->kq); free(s->kw);
    free(s);
}
