/* Test-oracle glue for the reference's data-store sources, compiled in place
 * into oracle/_ref/libmodalfiles.so (parameter.c, fixed_data.c, io.c,
 * arrays.c, basis_functions.c).  Nothing here is used by the library; the
 * tests and tests/golden/make_golden.py call the entry points at the end to
 * read what the reference's own initilise / set_terms_* / create_basis_late /
 * load_* / read_qtilde produce for a given INI file.
 *
 * Stand-ins for what the reference links against but the checkout lacks:
 *   - iniparser (parameter.c:6): a small INI reader following iniparser's
 *     published rules (';' or '#' comment lines, [section], key = value, keys
 *     "section:key" in lower case, quoted values, unquoted values cut at ';'
 *     or '#'; getint by strtol base 0, getdouble by atof);
 *   - GSL's gsl_interp_cspline: a natural cubic spline written here from its
 *     definition (zero second derivative at both ends);
 *   - MPI_Send / MPI_Recv (one rank; never called on these paths). */
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "global.h"
#include "iniparser/src/iniparser.h"
#include "mpi.h"

/* ------------------------------------------------------------ iniparser */

#define DICT_MAX 1024
struct refshim_dict {
    int n;
    char key[DICT_MAX][128];
    char val[DICT_MAX][512];
};

static char *strip(char *s)
{
    while (*s && isspace((unsigned char)*s)) s++;
    char *e = s + strlen(s);
    while (e > s && isspace((unsigned char)e[-1])) *--e = '\0';
    return s;
}

dictionary *iniparser_load(const char *path)
{
    FILE *f = fopen(path, "r");
    if (!f) return NULL;
    dictionary *d = calloc(1, sizeof(dictionary));
    char line[1024], section[128] = "";
    while (fgets(line, sizeof line, f)) {
        char *s = strip(line);
        if (!*s || *s == ';' || *s == '#') continue;
        if (*s == '[') {
            char *e = strchr(s, ']');
            if (!e) continue;
            *e = '\0';
            snprintf(section, sizeof section, "%s", strip(s + 1));
            for (char *c = section; *c; c++) *c = (char)tolower((unsigned char)*c);
            continue;
        }
        char *eq = strchr(s, '=');
        if (!eq || d->n >= DICT_MAX) continue;
        *eq = '\0';
        char *k = strip(s), *v = strip(eq + 1);
        if (*v == '"' || *v == '\'') {
            char q = *v++;
            char *e = strchr(v, q);
            if (e) *e = '\0';
        } else {
            v[strcspn(v, ";#")] = '\0';
            v = strip(v);
        }
        snprintf(d->key[d->n], sizeof d->key[0], "%s:%s", section, k);
        for (char *c = d->key[d->n]; *c; c++) *c = (char)tolower((unsigned char)*c);
        snprintf(d->val[d->n], sizeof d->val[0], "%s", v);
        d->n++;
    }
    fclose(f);
    return d;
}

static const char *lookup(dictionary *d, const char *key)
{
    char k[128];
    snprintf(k, sizeof k, "%s", key);
    for (char *c = k; *c; c++) *c = (char)tolower((unsigned char)*c);
    for (int i = d->n - 1; i >= 0; i--)  /* a repeated key: the last one wins */
        if (strcmp(d->key[i], k) == 0) return d->val[i];
    return NULL;
}

int iniparser_getint(dictionary *d, const char *key, int notfound)
{
    const char *v = lookup(d, key);
    return v ? (int)strtol(v, NULL, 0) : notfound;
}

double iniparser_getdouble(dictionary *d, const char *key, double notfound)
{
    const char *v = lookup(d, key);
    return v ? atof(v) : notfound;
}

char *iniparser_getstring(dictionary *d, const char *key, char *def)
{
    const char *v = lookup(d, key);
    return v ? (char *)v : def;
}

void iniparser_freedict(dictionary *d) { free(d); }

/* ------------------------------------------------------ natural spline */

struct refshim_spline { size_t n; double *x, *y, *m; };
struct refshim_interp_accel { int unused; };
struct refshim_interp_type { int unused; };
static const struct refshim_interp_type cspline_type = {0};
const gsl_interp_type *gsl_interp_cspline = &cspline_type;

gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t n)
{
    (void)T;
    gsl_spline *s = calloc(1, sizeof *s);
    s->n = n;
    s->x = calloc(n, sizeof(double));
    s->y = calloc(n, sizeof(double));
    s->m = calloc(n, sizeof(double));
    return s;
}

/* second derivatives m: h[i-1] m[i-1] + 2 (h[i-1] + h[i]) m[i] + h[i] m[i+1]
 * = 6 ((y[i+1]-y[i])/h[i] - (y[i]-y[i-1])/h[i-1]), m[0] = m[n-1] = 0,
 * solved by forward elimination and back substitution. */
int gsl_spline_init(gsl_spline *s, const double xa[], const double ya[], size_t n)
{
    if (n != s->n || n < 3) { fprintf(stderr, "spline: %zu points\n", n); abort(); }
    memcpy(s->x, xa, n * sizeof(double));
    memcpy(s->y, ya, n * sizeof(double));
    size_t m = n - 2;
    double *c = calloc(m, sizeof(double)), *r = calloc(m, sizeof(double));
    for (size_t i = 0; i < m; i++) {
        double h0 = xa[i + 1] - xa[i], h1 = xa[i + 2] - xa[i + 1];
        double diag = 2.0 * (h0 + h1);
        double rhs = 6.0 * ((ya[i + 2] - ya[i + 1]) / h1 - (ya[i + 1] - ya[i]) / h0);
        double den = diag - (i ? h0 * c[i - 1] : 0.0);
        c[i] = (i + 1 < m) ? h1 / den : 0.0;
        r[i] = (rhs - (i ? h0 * r[i - 1] : 0.0)) / den;
    }
    s->m[0] = s->m[n - 1] = 0.0;
    for (size_t i = m; i-- > 0;) s->m[i + 1] = r[i] - ((i + 1 < m) ? c[i] * s->m[i + 2] : 0.0);
    free(c);
    free(r);
    return 0;
}

double gsl_spline_eval(const gsl_spline *s, double t, gsl_interp_accel *acc)
{
    (void)acc;
    size_t n = s->n;
    if (t < s->x[0] || t > s->x[n - 1]) { fprintf(stderr, "spline: %g outside the table\n", t); abort(); }
    size_t lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        size_t mid = (lo + hi) / 2;
        if (s->x[mid] <= t) lo = mid; else hi = mid;
    }
    double h = s->x[lo + 1] - s->x[lo], a = s->x[lo + 1] - t, b = t - s->x[lo];
    return (s->m[lo] * a * a * a + s->m[lo + 1] * b * b * b) / (6.0 * h) + (s->y[lo] / h - s->m[lo] * h / 6.0) * a +
           (s->y[lo + 1] / h - s->m[lo + 1] * h / 6.0) * b;
}

double gsl_spline_eval_integ(const gsl_spline *s, double a, double b, gsl_interp_accel *acc)
{
    (void)s; (void)a; (void)b; (void)acc;
    fprintf(stderr, "gsl_spline_eval_integ is not stood in\n");
    abort();
}

gsl_interp_accel *gsl_interp_accel_alloc(void) { return calloc(1, sizeof(gsl_interp_accel)); }
void gsl_interp_accel_free(gsl_interp_accel *a) { free(a); }
void gsl_spline_free(gsl_spline *s)
{
    if (!s) return;
    free(s->x); free(s->y); free(s->m); free(s);
}

/* ------------------------------------------------------------------ MPI */

int MPI_Send(const void *b, int n, MPI_Datatype t, int dest, int tag, MPI_Comm c)
{
    (void)b; (void)n; (void)t; (void)dest; (void)tag; (void)c;
    fprintf(stderr, "MPI_Send on one rank\n");
    abort();
}

int MPI_Recv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *st)
{
    (void)b; (void)n; (void)t; (void)src; (void)tag; (void)c; (void)st;
    fprintf(stderr, "MPI_Recv on one rank\n");
    abort();
}

/* ------------------------------------------------ entry points for tests */

extern int initilise(char *inifile);
extern int set_terms_prim(void);
extern int set_terms_late(void);
extern int get_terms_prim(void);
extern int get_terms_late(void);
extern int get_pmax_prim(void);
extern int get_pmax_late_T(void);
extern int get_pmax_late_E(void);
extern int create_basis_late(int Tsize, int Esize, double Tmin, double Tmax, double Emin, double Emax, double *Tvec,
                             double *Evec);
extern double get_basis_late_T(int i, int j);
extern double get_basis_late_E(int i, int j);
extern int load_cl(void);
extern int load_BN(void);
extern int load_lens(void);
extern int load_TL(int l_size, int *l_values);
extern double get_cl_TT(int i), get_cl_TE(int i), get_cl_EE(int i), get_cl_TP(int i);
extern double get_beam_TT(int i), get_beam_TE(int i), get_beam_EE(int i);
extern double get_noise_TT(int i), get_noise_TE(int i), get_noise_EE(int i), get_t_wgt(int i);
extern int read_qtilde(void);
extern int get_qtilde_T_lsize(void), get_qtilde_E_lsize(void), get_qtilde_xsize(void);
extern int get_qtilde_T_lvec(int *vec), get_qtilde_E_lvec(int *vec), get_qtilde_xvec(double *vec);
extern double get_qtilde_T(int i, int j, int k), get_qtilde_E(int i, int j, int k);
extern void find_perm_prim(int r, int *p1, int *p2, int *p3);
extern void find_perm_late_TTT(int r, int *p1, int *p2, int *p3);
extern void find_perm_late_TTE(int r, int *p1, int *p2, int *p3);
extern void find_perm_late_TEE(int r, int *p1, int *p2, int *p3);
extern void find_perm_late_EEE(int r, int *p1, int *p2, int *p3);
extern int eflag_T_lmax, eflag_E_lmax, eflag_T_lmin, eflag_E_lmin, do_polarisation;

/* initilise(ini) as in a fresh process: parameter.c builds the absolute-path
 * proj size names with strcat onto zero-initialised globals (parameter.c:731-734),
 * so those start empty here for every INI file loaded. */
int files_init(const char *ini)
{
    char path[MAXLEN];
    snprintf(path, sizeof path, "%s", ini);
    proj_T_size_file[0] = proj_E_size_file[0] = '\0';
    return initilise(path);
}

/* The file-name globals of parameter.c as "name=value" lines. */
int files_names(char *buf, int len)
{
    struct { const char *name; const char *v; } t[] = {
        {"orthol_TTT", orthol_TTT_data_file}, {"orthol_TTE", orthol_TTE_data_file},
        {"orthol_TEE", orthol_TEE_data_file}, {"orthol_EEE", orthol_EEE_data_file},
        {"lambdal_TTT", lambdal_TTT_data_file}, {"lambdal_TTE", lambdal_TTE_data_file},
        {"lambdal_TEE", lambdal_TEE_data_file}, {"lambdal_EEE", lambdal_EEE_data_file},
        {"modes_TTT", modes_TTT_data_file}, {"modes_TTE", modes_TTE_data_file},
        {"modes_TEE", modes_TEE_data_file}, {"modes_EEE", modes_EEE_data_file},
        {"gamma_TTT", gamma_TTT_data_file}, {"gamma_TTE", gamma_TTE_data_file},
        {"gamma_TEE", gamma_TEE_data_file}, {"gamma_EEE", gamma_EEE_data_file},
        {"proj_T_data", proj_T_data_file}, {"proj_E_data", proj_E_data_file},
        {"proj_T_size", proj_T_size_file}, {"proj_E_size", proj_E_size_file},
        {"pixw", pixw_file}, {"BN_TT", BN_TT_file}, {"BN_EE", BN_EE_file}, {"transfer_wgt", transfer_wgt_file},
    };
    int off = 0;
    for (size_t i = 0; i < sizeof t / sizeof t[0]; i++) {
        int w = snprintf(buf + off, (size_t)(len - off), "%s=%s\n", t[i].name, t[i].v);
        if (w < 0 || off + w >= len) return 1;
        off += w;
    }
    return 0;
}

/* set_terms_prim + set_terms_late; orders as [N][3]; pm = pmax_prim, pmax_T, pmax_E.
 * tte/tee/eee are filled only with do_polarisation. */
int files_terms(int *prim, int *ttt, int *tte, int *tee, int *eee, int *pm)
{
    set_terms_prim();
    set_terms_late();
    int Np = get_terms_prim(), N = get_terms_late();
    for (int n = 0; n < Np; n++) find_perm_prim(n, prim + 3 * n, prim + 3 * n + 1, prim + 3 * n + 2);
    for (int n = 0; n < N; n++) {
        find_perm_late_TTT(n, ttt + 3 * n, ttt + 3 * n + 1, ttt + 3 * n + 2);
        if (do_polarisation == 1) {
            find_perm_late_TTE(n, tte + 3 * n, tte + 3 * n + 1, tte + 3 * n + 2);
            find_perm_late_TEE(n, tee + 3 * n, tee + 3 * n + 1, tee + 3 * n + 2);
            find_perm_late_EEE(n, eee + 3 * n, eee + 3 * n + 1, eee + 3 * n + 2);
        }
    }
    pm[0] = get_pmax_prim();
    pm[1] = get_pmax_late_T();
    pm[2] = do_polarisation == 1 ? get_pmax_late_E() : 0;
    return 0;
}

/* load_cl, load_BN, load_lens (lens != 0), load_TL (tl != 0); out [11][T_lmax+1]:
 * cl TT, TE, EE, beam TT, TE, EE, noise TT, TE, EE (E rows up to E_lmax, zero
 * beyond), cl TP, t_wgt. */
int files_spectra(int lens, int tl, double *out)
{
    const int lT = eflag_T_lmax, lE = eflag_E_lmax, n = lT + 1;
    if (load_cl() != 0 || load_BN() != 0) return 1;
    if (lens && load_lens() != 0) return 1;
    if (tl) {
        int *lv = malloc(sizeof(int) * (size_t)n);
        for (int i = 0; i < n; i++) lv[i] = i;
        int r = load_TL(n, lv);
        free(lv);
        if (r != 0) return 1;
    }
    memset(out, 0, sizeof(double) * 11 * (size_t)n);
    for (int l = 0; l < n; l++) {
        out[0 * n + l] = get_cl_TT(l);
        out[3 * n + l] = get_beam_TT(l);
        out[6 * n + l] = get_noise_TT(l);
        if (lens) out[9 * n + l] = get_cl_TP(l);
        if (tl) out[10 * n + l] = get_t_wgt(l);
    }
    if (do_polarisation == 1)
        for (int l = 0; l <= lE && l < n; l++) {
            out[1 * n + l] = get_cl_TE(l);
            out[2 * n + l] = get_cl_EE(l);
            out[4 * n + l] = get_beam_TE(l);
            out[5 * n + l] = get_beam_EE(l);
            out[7 * n + l] = get_noise_TE(l);
            out[8 * n + l] = get_noise_EE(l);
        }
    return 0;
}

/* create_basis_late on T_lmin..T_lmax (E_lmin..E_lmax); bt [Tsize][pmax_T+1],
 * be [Esize][pmax_E+1] with do_polarisation. */
int files_basis(double *bt, double *be)
{
    const int Tsize = eflag_T_lmax - eflag_T_lmin + 1, Esize = eflag_E_lmax - eflag_E_lmin + 1;
    double *Tv = malloc(sizeof(double) * (size_t)Tsize), *Ev = malloc(sizeof(double) * (size_t)Esize);
    for (int i = 0; i < Tsize; i++) Tv[i] = (double)i + eflag_T_lmin;
    for (int i = 0; i < Esize; i++) Ev[i] = (double)i + eflag_E_lmin;
    create_basis_late(Tsize, Esize, eflag_T_lmin, eflag_T_lmax, eflag_E_lmin, eflag_E_lmax, Tv, Ev);
    const int PT = get_pmax_late_T() + 1;
    for (int l = 0; l < Tsize; l++)
        for (int p = 0; p < PT; p++) bt[(size_t)l * PT + p] = get_basis_late_T(l, p);
    if (do_polarisation == 1) {
        const int PE = get_pmax_late_E() + 1;
        for (int l = 0; l < Esize; l++)
            for (int p = 0; p < PE; p++) be[(size_t)l * PE + p] = get_basis_late_E(l, p);
    }
    free(Tv);
    free(Ev);
    return 0;
}

/* read_qtilde; sizes = lsize_T, lsize_E, xsize (call with qt == NULL first). */
int files_qtilde(int *sizes, double *x, int *lvec_t, double *qt_t, int *lvec_e, double *qt_e)
{
    if (!qt_t) {
        read_qtilde();
        sizes[0] = get_qtilde_T_lsize();
        sizes[1] = do_polarisation == 1 ? get_qtilde_E_lsize() : 0;
        sizes[2] = get_qtilde_xsize();
        return 0;
    }
    const int LT = sizes[0], LE = sizes[1], X = sizes[2], P = get_pmax_prim() + 1;
    get_qtilde_xvec(x);
    get_qtilde_T_lvec(lvec_t);
    for (int n = 0; n < P; n++)
        for (int l = 0; l < LT; l++)
            for (int i = 0; i < X; i++) qt_t[((size_t)n * LT + l) * X + i] = get_qtilde_T(n, l, i);
    if (do_polarisation == 1) {
        get_qtilde_E_lvec(lvec_e);
        for (int n = 0; n < P; n++)
            for (int l = 0; l < LE; l++)
                for (int i = 0; i < X; i++) qt_e[((size_t)n * LE + l) * X + i] = get_qtilde_E(n, l, i);
    }
    return 0;
}
