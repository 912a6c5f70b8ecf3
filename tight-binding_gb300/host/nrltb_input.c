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
    p->jspins = (mag == 'M' || mag == 'm') ? 2 : 1;
    if (p->jspins != 1) { rc = NRLTB_E_UNSUPPORTED; goto fail; }
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
    int npards = nrltb_nparams(p->kinds);
    p->param = (double *)calloc((size_t)npards, sizeof(double));
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
    int *kkind;
    double *posn, *posq;
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

/* kptin.f:66-366 for the explicit-list (-1313 file, inline list) and path
 * (999) forms.  The mesh generator path (kptgen.f) is not restated. */
static int read_kpoints(nrltb_skin *s)
{
    lreader *r = &s->r;
    char fld[300];
    if (lr_next(r)) return NRLTB_E_PARSE;
    field(r->buf, 7, 1, fld);
    int newsym = (fld[0] == 'T' || fld[0] == 't');
    if (!newsym) return s->nk > 0 ? NRLTB_OK : NRLTB_E_PARSE;
    if (lr_next(r)) return NRLTB_E_PARSE;           /* (7x,I1) LATTIC */
    if (lr_next(r)) return NRLTB_E_PARSE;           /* (A) space group file */
    char sg[300], full[1400];
    field(r->buf, 0, 255, sg);
    rtrim(sg);
    join_path(s->dir, sg, full, sizeof full);
    {
        FILE *f = fopen(full, "r");                  /* OPEN(25,...,STATUS='OLD') */
        if (!f) return NRLTB_E_IO;
        fclose(f);
    }
    if (lr_next(r)) return NRLTB_E_PARSE;           /* (5x,L1) ILAT */
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
    if (nkv <= 0) { rc = NRLTB_E_UNSUPPORTED; goto done; }
    if (nkv == 999) {
        /* path mode: segments of KD equally spaced points, weight 1 each */
        long kpdir;
        if (lr_next(kio)) { rc = NRLTB_E_PARSE; goto done; }
        field(kio->buf, 0, 5, fld);
        if (fmt_int(fld, !own, &kpdir)) { rc = NRLTB_E_PARSE; goto done; }
        int cap = 1024, nk = 0;
        double *q = malloc(sizeof(double) * 3 * cap), *w = malloc(sizeof(double) * cap);
        for (long d = 0; d < kpdir; ++d) {
            double v[7];
            if (ld_reals(kio, 7, v)) { free(q); free(w); rc = NRLTB_E_PARSE; goto done; }
            int kd = (int)v[0];
            if (nk + kd + 1 > cap) {
                cap = 2 * (nk + kd + 1);
                q = realloc(q, sizeof(double) * 3 * cap);
                w = realloc(w, sizeof(double) * cap);
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
        for (int i = 0; i < nk; ++i) w[i] = w[i] * (double)nk; /* WGHTS = NK here */
        free(s->kq); free(s->kw);
        s->kq = q; s->kw = w; s->nk = nk;
    } else {
        double *q = malloc(sizeof(double) * 3 * nkv), *w = malloc(sizeof(double) * nkv);
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
    if (!(c2 == ' ' || c2 == 'F' || c2 == 'f')) { rc = NRLTB_E_UNSUPPORTED; goto fail; }
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
        long nshift;
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
    free(s->kkind); free(s->posn); free(s->posq);
    s->natoms = natoms;
    s->kkind = malloc(sizeof(int) * natoms);
    s->posn = malloc(sizeof(double) * 3 * natoms);
    s->posq = malloc(sizeof(double) * 3 * natoms);
    for (int i = 0; i < natoms; ++i) {
        double v[7];
        if (ld_reals(r, 7, v)) { free(shift); free(epsl); goto fail; }
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
    rc = read_kpoints(s);
    if (rc) goto fail;
    memset(st, 0, sizeof *st);
    st->natoms = natoms;
    st->kkind = s->kkind;
    st->posn = s->posn;
    st->posq = s->posq;
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
    free(s->kkind); free(s->posn); free(s->posq); free(s->kq); free(s->kw);
    free(s);
}
