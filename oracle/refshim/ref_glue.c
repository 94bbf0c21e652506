/* Glue for compiling the Modal-CMB reference's own hot-path sources in place
 * (orthogonalisation_late.c, gl_integration.c, basis_functions.c,
 * calculate_geometric.c, tetrapyd_tools.c, calculate_mode_3D.c,
 * calculate_modes.c, arrays.c) into oracle/_ref/libmodalref.so.
 *
 * TEST INFRASTRUCTURE ONLY.  This file supplies what those sources expect
 * from the rest of the reference (fixed_data.c accessors, parameter.c
 * globals, GSL/MPI entry points) and exports a few driver functions that
 * the tests call through ctypes to produce reference outputs.  Nothing in
 * the product links or loads it.
 *
 * Stand-ins, each restating the behaviour the reference relies on:
 *  - gsl_sf_legendre_Pl: GSL's upward three-term recurrence (GSL uses it for
 *    l < 100000; P_2 in closed form).
 *  - gsl_sf_bessel_J0/J1/Jn: the C library's j0/j1/jn.
 *  - MPI: one rank; reductions copy.
 *  - accessors get_basis_late_T / find_perm_late_TTT / get_cl_TT ... read the
 *    tables passed to ref_setup (layouts of fixed_data.c:1764 basis_late_T
 *    [Tsize][pmax+1] and order_late_TTT[n][3]).
 *  - calculate_xint_TTT returns the synthetic shape for term 0 and 0 for the
 *    rest, and get_eigen returns 1 for term 0, so calculate_3D_bispectrum
 *    (calculate_mode_3D.c:266-281) evaluates exactly that shape.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>
#include "mpi.h"
#include "../shapes.h"

/* ---- globals the reference declares extern (global.h:161-174) ---- */
int eflag_T_lmax, eflag_T_lmin, eflag_E_lmax, eflag_E_lmin;
int do_polarisation = 0;
int model = 0;
int l1, l2, l3, l4;
int offload_target = 0;

/* ---- reference functions compiled from the in-place sources ---- */
extern int asy(double *nodes, double *weights, unsigned long n);
extern double init_orthol_glint(void);
extern void calculate_orthoMij_T(int i, int j);
extern void calculate_orthoMij_E(int i, int j);
extern void sync_orthoMij(void);
extern int calculate_orthol(int m, int n, double *result);
extern double plijk_TTT(int r, int i, int j, int k);
extern double calculate_geometric(int i, int j, int k);
extern int basis_functions_legendre(double **array, int size, int pmax, double min, double max, double *values);
extern double **create_array(int dim_x, int dim_y);
extern int get_ijk_next_XXX(int lmax, int *i, int *j, int *k);
extern void check_ijk_min_XXX(int lmin, int *i, int *j, int *k);

typedef struct { int i_bgn, j_bgn, k_bgn, loops; } ref_tetrapyd_limits; /* tetrapyd_tools.h:333-339 */
extern void decompose_tetrapyd_XXX(ref_tetrapyd_limits *block, int rank, int nranks, int nthreads, int lmin, int lmax);
extern void init_3D(int mode);
extern void calculate_mode_3D(int min, int max, ref_tetrapyd_limits *block, double *alpha);

/* ---- state behind the accessors ---- */
static int g_P, g_N, g_L;
static double *g_basis;   /* [L][P] */
static int *g_triples;    /* [N][3] */
/* polarisation (ref_setup_pol): E basis [L_E][P_E], TTE/TEE/EEE triples in
 * the find_perm_late_XXX conventions (T,T,E), (T,E,E), (E,E,E) */
static int g_PE;
static double *g_basisE;
static int *g_tte, *g_tee, *g_eee;
static double *g_cl;      /* [lmax+1], C_l + N_l/b_l^2 */
static orc_shape g_shape;

/* ---- Intel aligned allocation used by calculate_gamma.c ---- */
void *_mm_malloc(size_t size, size_t align)
{
    void *p = NULL;
    if (align < sizeof(void *)) align = sizeof(void *);
    return posix_memalign(&p, align, size) == 0 ? p : NULL;
}
void _mm_free(void *p) { free(p); }

/* ---- MPI, one rank ---- */
int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(MPI_Comm c, int *rank) { (void)c; *rank = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int *size) { (void)c; *size = 1; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static size_t mpi_bytes(MPI_Datatype t) { return t == MPI_INT ? sizeof(int) : (t == MPI_LONG ? sizeof(long) : sizeof(double)); }
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{ (void)op; (void)c; memmove(r, s, (size_t)n * mpi_bytes(t)); return 0; }
int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c)
{ (void)op; (void)root; (void)c; memmove(r, s, (size_t)n * mpi_bytes(t)); return 0; }

/* ---- GSL stand-ins ---- */
double gsl_sf_bessel_J0(double x) { return j0(x); }
double gsl_sf_bessel_J1(double x) { return j1(x); }
double gsl_sf_bessel_Jn(int n, double x) { return jn(n, x); }
struct refshim_glfixed { int unused; };
struct refshim_glfixed *gsl_integration_glfixed_table_alloc(size_t n) { (void)n; return NULL; }
void gsl_integration_glfixed_table_free(struct refshim_glfixed *t) { (void)t; }
double gsl_sf_legendre_Pl(int l, double x)
{
    if (l == 0) return 1.0;
    if (l == 1) return x;
    if (l == 2) return 0.5 * (3.0 * x * x - 1.0);
    if (x == 1.0) return 1.0;
    if (x == -1.0) return (l & 1) ? -1.0 : 1.0;
    double pm2 = 1.0, pm1 = x, p = x;
    for (int ell = 2; ell <= l; ell++) {
        p = (x * (2 * ell - 1) * pm1 - (ell - 1) * pm2) / ell;
        pm2 = pm1;
        pm1 = p;
    }
    return p;
}

/* ---- fixed_data.c accessors ---- */
int get_pmax_late_T(void) { return g_P - 1; }
int get_pmax_late_E(void) { return do_polarisation ? g_PE - 1 : g_P - 1; }
double get_basis_late_T(int i, int j) { return g_basis[(long)i * g_P + j]; }
double get_basis_late_E(int i, int j) { return do_polarisation ? g_basisE[(long)i * g_PE + j] : g_basis[(long)i * g_P + j]; }
static void perm_of(int r, int *p1, int *p2, int *p3) { *p1 = g_triples[3 * r]; *p2 = g_triples[3 * r + 1]; *p3 = g_triples[3 * r + 2]; }
void find_perm_late_TTT(int r, int *p1, int *p2, int *p3) { perm_of(r, p1, p2, p3); }
static void perm_in(const int *t, int r, int *p1, int *p2, int *p3) { *p1 = t[3 * r]; *p2 = t[3 * r + 1]; *p3 = t[3 * r + 2]; }
void find_perm_late_TTE(int r, int *p1, int *p2, int *p3) { if (do_polarisation) perm_in(g_tte, r, p1, p2, p3); else perm_of(r, p1, p2, p3); }
void find_perm_late_TEE(int r, int *p1, int *p2, int *p3) { if (do_polarisation) perm_in(g_tee, r, p1, p2, p3); else perm_of(r, p1, p2, p3); }
void find_perm_late_EEE(int r, int *p1, int *p2, int *p3) { if (do_polarisation) perm_in(g_eee, r, p1, p2, p3); else perm_of(r, p1, p2, p3); }
int get_terms_late(void) { return g_N; }
int get_terms_prim(void) { return g_N; }
int get_lmax(void) { return eflag_T_lmax; }
double get_tau0(void) { return 0.0; }
/* radial grid and transfer functions q~_p(l, x) (qtilde, fixed_data.c:2045-2495);
 * one dummy point unless ref_setup_transfer installed some */
static int g_xsize = 1, g_Pp = 1, g_Nprim = 0;
static double g_x0 = 0.0, *g_xvec = &g_x0, *g_qt;  /* g_qt[x][p][l], l = 0..lmax */
static int *g_prim;                                 /* [Nprim][3] */
double deltaphi = 1.0;
double fskyT = 1.0, fskyE = 1.0;
int get_qtilde_xsize(void) { return g_xsize; }
int get_qtilde_xvec(double *v) { for (int i = 0; i < g_xsize; i++) v[i] = g_xvec[i]; return 0; }
double get_qtilde_T(int p, int l, int x) { return g_qt[((long)x * g_Pp + p) * (eflag_T_lmax + 1) + l]; }
static double *g_qtE;                               /* polarised runs: g_qtE[x][p][l] */
double get_qtilde_E(int p, int l, int x)
{ return g_qtE ? g_qtE[((long)x * g_Pp + p) * (eflag_T_lmax + 1) + l] : get_qtilde_T(p, l, x); }
/* polarised spectra (ref_setup_pol_spectra): TT, TE, EE signal, beams, noise */
static double *g_spec;  /* [9][lmax+1]: cl_tt, cl_te, cl_ee, b_tt, b_te, b_ee, n_tt, n_te, n_ee */
static int g_spec_n;
#define SPEC(i, l) g_spec[(long)(i) * g_spec_n + (l)]
int destroy_qtilde(void) { return 0; }
int get_pmax_prim(void) { return g_Pp - 1; }
void find_perm_prim(int r, int *p1, int *p2, int *p3) { *p1 = g_prim[3 * r]; *p2 = g_prim[3 * r + 1]; *p3 = g_prim[3 * r + 2]; }
double get_beam_EE(int l) { return g_spec ? SPEC(5, l) : 1.0; }
double get_beam_TE(int l) { return g_spec ? SPEC(4, l) : 1.0; }
double get_cl_TE(int l) { return g_spec ? SPEC(1, l) : 0.0; }
double get_cl_EE(int l) { return g_spec ? SPEC(2, l) : 1.0; }
double get_cl_TP(int l) { (void)l; return 0.0; }
double get_noise_TE(int l) { return g_spec ? SPEC(7, l) : 0.0; }
double get_noise_EE(int l) { return g_spec ? SPEC(8, l) : 0.0; }
/* GSL cubic-spline link stubs (calculate_gamma() is not exercised) */
#include <stdio.h>
#include "gsl/gsl_spline.h"
const gsl_interp_type *gsl_interp_cspline = NULL;
gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t n) { (void)T; (void)n; fprintf(stderr, "gsl_spline stub called\n"); abort(); }
int gsl_spline_init(gsl_spline *s, const double xa[], const double ya[], size_t n) { (void)s; (void)xa; (void)ya; (void)n; abort(); }
double gsl_spline_eval_integ(const gsl_spline *s, double a, double b, gsl_interp_accel *acc) { (void)s; (void)a; (void)b; (void)acc; abort(); }
double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *acc) { (void)s; (void)x; (void)acc; abort(); }
gsl_interp_accel *gsl_interp_accel_alloc(void) { abort(); }
void gsl_interp_accel_free(gsl_interp_accel *a) { (void)a; }
void gsl_spline_free(gsl_spline *s) { (void)s; }
int read_eigen(int a, int b, int c) { (void)a; (void)b; (void)c; return 0; }
double get_eigen(int i) { return i == 0 ? 1.0 : 0.0; }
double get_cl_TT(int l) { return g_spec ? SPEC(0, l) : g_cl[l]; }
double get_noise_TT(int l) { return g_spec ? SPEC(6, l) : 0.0; }
double get_beam_TT(int l) { return g_spec ? SPEC(3, l) : 1.0; }
double calculate_ISW_bispectrum(int i, int j, int k) { (void)i; (void)j; (void)k; return 0.0; }
double calculate_xint_TTT(int a, int b, int c, int n, int xsize, double *xvec)
{ (void)xsize; (void)xvec; return n == 0 ? orc_shape_eval(&g_shape, a, b, c) : 0.0; }
double permsix(int i, int j, int k)
{ if (i == j && j == k) return 1.0; if (i == j || j == k || i == k) return 3.0; return 6.0; }
int sync_tasks(int mode, int size) { (void)mode; (void)size; return 0; }
double get_orthol_TTT(int i, int j) { (void)i; (void)j; return 0.0; }
double get_lambdal_TTT(int i, int j) { (void)i; (void)j; return 0.0; }
double get_lambdal_TTE(int i, int j) { (void)i; (void)j; return 0.0; }
double get_lambdal_TEE(int i, int j) { (void)i; (void)j; return 0.0; }
double get_lambdal_EEE(int i, int j) { (void)i; (void)j; return 0.0; }
double get_modes_TTT(int i) { (void)i; return 0.0; }
double get_modes_TTE(int i) { (void)i; return 0.0; }
double get_modes_TEE(int i) { (void)i; return 0.0; }
double get_modes_EEE(int i) { (void)i; return 0.0; }
double get_modesR_TTT(int i) { (void)i; return 0.0; }

/* ===================== exported drivers (ctypes) ===================== */

/* Install the basis q[L][P] (basis_late_T layout), the mode triples [N][3]
 * (order_late_TTT layout) and the total spectrum cl[lmax+1]. */
int ref_setup(int lmin, int lmax, int P, const double *basis, int N, const int *triples, const double *cl)
{
    g_P = P; g_N = N; g_L = lmax - lmin + 1;
    do_polarisation = 0;
    free(g_spec); g_spec = NULL; fskyT = fskyE = 1.0;
    eflag_T_lmin = eflag_E_lmin = lmin;
    eflag_T_lmax = eflag_E_lmax = lmax;
    free(g_basis); free(g_triples); free(g_cl);
    g_basis = malloc(sizeof(double) * (size_t)g_L * P);
    g_triples = malloc(sizeof(int) * 3 * (size_t)N);
    g_cl = malloc(sizeof(double) * (size_t)(lmax + 1));
    memcpy(g_basis, basis, sizeof(double) * (size_t)g_L * P);
    memcpy(g_triples, triples, sizeof(int) * 3 * (size_t)N);
    memcpy(g_cl, cl, sizeof(double) * (size_t)(lmax + 1));
    return 0;
}

int ref_asy(int n, double *nodes, double *weights) { return asy(nodes, weights, (unsigned long)n); }

double ref_legendre_Pl(int l, double x) { return gsl_sf_legendre_Pl(l, x); }

int ref_basis_legendre(int size, int pmax, double min, double max, const double *values, double *out)
{
    double **a = create_array(size, pmax + 1);
    basis_functions_legendre(a, size, pmax, min, max, (double *)values);
    for (int i = 0; i < size; i++) memcpy(out + (long)i * (pmax + 1), a[i], sizeof(double) * (pmax + 1));
    free(a[0]); free(a);
    return 0;
}

extern int basis_functions_fourier(double **array, int size, int pmax, double min, double max, double *values);
extern int basis_functions_sinlog(double **array, int size, int pmax, double min, double max, double *values);
extern int basis_functions_bi(double **array, int size, int pmax, double min, double max, double *values);

/* One of the basis families of basis_functions.c: 0 legendre, 1 fourier,
 * 2 sinlog, 3 bi (pmax <= 30). */
int ref_basis_family(int kind, int size, int pmax, double min, double max, const double *values, double *out)
{
    if (kind < 0 || kind > 3 || (kind == 3 && pmax > 30)) return 1;
    double **a = create_array(size, pmax + 1);
    if (kind == 0) basis_functions_legendre(a, size, pmax, min, max, (double *)values);
    if (kind == 1) basis_functions_fourier(a, size, pmax, min, max, (double *)values);
    if (kind == 2) basis_functions_sinlog(a, size, pmax, min, max, (double *)values);
    if (kind == 3) basis_functions_bi(a, size, pmax, min, max, (double *)values);
    for (int i = 0; i < size; i++) memcpy(out + (long)i * (pmax + 1), a[i], sizeof(double) * (pmax + 1));
    free(a[0]); free(a);
    return 0;
}

/* init_orthol_glint + calculate_orthoMij_T over all P^2 (i,j) pairs + sync,
 * the sequence of ortho_late_mpi.c:170-229 on one rank. */
int ref_init_gamma(void)
{
    init_orthol_glint();
    for (int i = 0; i < g_P; i++)
        for (int j = 0; j < g_P; j++) calculate_orthoMij_T(i, j);
    if (do_polarisation)
        for (int i = 0; i < g_PE; i++)
            for (int j = 0; j < g_PE; j++) calculate_orthoMij_E(i, j);
    sync_orthoMij();
    return 0;
}

/* Switch on polarisation after ref_setup: the E basis [lmaxE-lminE+1][PE]
 * (basis_late_E layout) and the TTE/TEE/EEE mode triples [N][3] as
 * find_perm_late_XXX returns them. */
int ref_setup_pol(int lminE, int lmaxE, int PE, const double *basisE, const int *tte, const int *tee, const int *eee)
{
    const int LE = lmaxE - lminE + 1;
    eflag_E_lmin = lminE;
    eflag_E_lmax = lmaxE;
    g_PE = PE;
    free(g_basisE); free(g_tte); free(g_tee); free(g_eee);
    g_basisE = malloc(sizeof(double) * (size_t)LE * PE);
    g_tte = malloc(sizeof(int) * 3 * (size_t)g_N);
    g_tee = malloc(sizeof(int) * 3 * (size_t)g_N);
    g_eee = malloc(sizeof(int) * 3 * (size_t)g_N);
    memcpy(g_basisE, basisE, sizeof(double) * (size_t)LE * PE);
    memcpy(g_tte, tte, sizeof(int) * 3 * (size_t)g_N);
    memcpy(g_tee, tee, sizeof(int) * 3 * (size_t)g_N);
    memcpy(g_eee, eee, sizeof(int) * 3 * (size_t)g_N);
    do_polarisation = 1;
    return 0;
}

/* All four matrices of calculate_orthol (TTT, TTE, TEE, EEE) over every
 * pair, out[4][N][N] (ortho_late_mpi.c:261-287 fills ortho_XXX the same way). */
int ref_gamma_pol(double *out)
{
    const long N = g_N, NN = N * N;
    for (long i = 0; i < N; i++)
        for (long j = i; j < N; j++) {
            double r[4];
            calculate_orthol((int)i, (int)j, r);
            for (int c = 0; c < 4; c++) out[c * NN + i * N + j] = out[c * NN + j * N + i] = r[c];
        }
    return 0;
}

int ref_orthol_pair(int m, int n, double *result) { return calculate_orthol(m, n, result); }

/* Gamma over the upper triangle, pairs split over `nranks` single-threaded
 * workers exactly as ortho_late_mpi.c:242-266 splits them over MPI ranks
 * (the per-pair OpenMP region inside calculate_orthol runs one thread).
 * `npairs_limit` > 0 stops after that many pairs (bounded timing sample).
 * Writes the full symmetric matrix out[N][N] (ortho_late_mpi.c:344-363). */
long ref_gamma(int nranks, long npairs_limit, double *out)
{
    const int N = g_N;
    const long total = (long)N * (N + 1) / 2;
    const long todo = (npairs_limit > 0 && npairs_limit < total) ? npairs_limit : total;
    int *pi = malloc(sizeof(int) * (size_t)total), *pj = malloc(sizeof(int) * (size_t)total);
    long n = 0;
    for (int i = 0; i < N; i++)
        for (int j = i; j < N; j++) { pi[n] = i; pj[n] = j; n++; }
    omp_set_max_active_levels(1);
    #pragma omp parallel num_threads(nranks)
    {
        const int rank = omp_get_thread_num(), nproc = omp_get_num_threads();
        long loops = todo / nproc, aux = todo % nproc;
        long start = rank * loops, end = (rank + 1) * loops - 1;
        if (aux) {
            if (rank < aux) { start += rank; end += rank + 1; }
            else { start += aux; end += aux; }
        }
        double r[4];
        for (long p = start; p <= end; p++) {
            calculate_orthol(pi[p], pj[p], r);
            out[(long)pi[p] * N + pj[p]] = r[0];
            out[(long)pj[p] * N + pi[p]] = r[0];
        }
    }
    free(pi); free(pj);
    return todo;
}

double ref_geometric(int i, int j, int k) { return calculate_geometric(i, j, k); }
double ref_plijk(int r, int i, int j, int k) { return plijk_TTT(r, i, j, k); }

/* Walk the tetrapyd with get_ijk_next_XXX from the start given by
 * check_ijk_min_XXX; writes up to `cap` points (i,j,k) and returns the count
 * decompose_tetrapyd_XXX would assign in total. */
long ref_tetrapyd_walk(int lmin, int lmax, long cap, int *pts)
{
    int i = lmin, j = lmin, k = lmin;
    check_ijk_min_XXX(lmin, &i, &j, &k);
    long count = 0;
    for (;;) {
        if (count < cap) { pts[3 * count] = i; pts[3 * count + 1] = j; pts[3 * count + 2] = k; }
        count++;
        if (!get_ijk_next_XXX(lmax, &i, &j, &k)) break;
    }
    if (count < cap) { pts[3 * count] = i; pts[3 * count + 1] = j; pts[3 * count + 2] = k; }
    return count + 1;
}

int ref_decompose(int nthreads, int lmin, int lmax, int *out /*[nthreads][4]*/)
{
    ref_tetrapyd_limits *b = malloc(sizeof(*b) * (size_t)nthreads);
    decompose_tetrapyd_XXX(b, 0, 1, nthreads, lmin, lmax);
    for (int t = 0; t < nthreads; t++) { out[4 * t] = b[t].i_bgn; out[4 * t + 1] = b[t].j_bgn; out[4 * t + 2] = b[t].k_bgn; out[4 * t + 3] = b[t].loops; }
    free(b);
    return 0;
}

/* calculate_mode_3D (calculate_mode_3D.c:217-264) for one shape with the
 * eigenmodetoday_mpi.c:235-261 set-up (init_3D, decompose_tetrapyd_XXX over
 * `nthreads` OpenMP threads).  shape: kind/nterms/tab/c/sigma as in shapes.h.
 * `max_points` > 0 limits every thread's block to its first points
 * (bounded timing sample).  beta[N] out. */
int ref_project(int nthreads, int kind, int nterms, const double *tab, double c1, double c2, double c3,
                double sigma, long max_points, double *beta)
{
    g_shape.kind = kind; g_shape.nterms = nterms; g_shape.lmax = eflag_T_lmax; g_shape.tab = tab;
    g_shape.c1 = c1; g_shape.c2 = c2; g_shape.c3 = c3; g_shape.sigma = sigma;
    omp_set_num_threads(nthreads);
    omp_set_max_active_levels(1);
    ref_tetrapyd_limits *b = malloc(sizeof(*b) * (size_t)nthreads);
    decompose_tetrapyd_XXX(b, 0, 1, nthreads, eflag_T_lmin, eflag_T_lmax);
    if (max_points > 0)
        for (int t = 0; t < nthreads; t++) if (b[t].loops > max_points) b[t].loops = (int)max_points;
    init_3D(1001);
    calculate_mode_3D(eflag_T_lmin, eflag_T_lmax, b, beta);
    free(b);
    return 0;
}

/* ---- serial dense form: modify_bispectrum + calculate_modes (calculate_modes.c:6-79) ---- */
extern void modify_bispectrum(int size, int *vec, double ***bispectrum);
extern double calculate_modes(int r, int size, double ***bispectrum);

static double ***view3(int size, double *flat)
{
    double ***b = malloc(sizeof(double **) * (size_t)size);
    double **rows = malloc(sizeof(double *) * (size_t)size * size);
    for (int i = 0; i < size; i++) {
        b[i] = rows + (size_t)i * size;
        for (int j = 0; j < size; j++) b[i][j] = flat + ((size_t)i * size + j) * size;
    }
    return b;
}

static void free_view3(double ***b) { free(b[0]); free(b); }

/* In place on flat[size^3]; the spectrum installed by ref_setup is indexed by i. */
int ref_modify_bispectrum(int size, const int *vec, double *flat)
{
    double ***b = view3(size, flat);
    modify_bispectrum(size, (int *)vec, b);
    free_view3(b);
    return 0;
}

int ref_calculate_modes(int size, double *flat, double *beta)
{
    double ***b = view3(size, flat);
    for (int r = 0; r < g_N; r++) beta[r] = calculate_modes(r, size, b);
    free_view3(b);
    return 0;
}

/* ---- late x primordial transfer Gamma (calculate_gamma.c, default 2D path) ---- */
extern void init_gamma_glint(void);
extern void precompute_gammaMij_T(void);
extern void calculate_gamma_2d(int m, int n, double *result);

/* qt[x][p][l] raw q~_p(l, x) for l = 0..lmax; prim[Nprim][3]; out[N][Nprim]
 * = calculate_gamma_2d(m, n) (calculate_gamma.c:773-842) after
 * init_gamma_glint + precompute_gammaMij_T, the gamma_mpi.c default path. */
int ref_gamma_transfer(int xsize, const double *xvec, int Pp, const double *qt, int Nprim, const int *prim,
                       double dphi, double *out)
{
    g_xsize = xsize; g_Pp = Pp; g_Nprim = Nprim; deltaphi = dphi;
    g_xvec = malloc(sizeof(double) * (size_t)xsize);
    memcpy(g_xvec, xvec, sizeof(double) * (size_t)xsize);
    size_t nq = (size_t)xsize * Pp * (eflag_T_lmax + 1);
    g_qt = malloc(sizeof(double) * nq);
    memcpy(g_qt, qt, sizeof(double) * nq);
    g_prim = malloc(sizeof(int) * 3 * (size_t)Nprim);
    memcpy(g_prim, prim, sizeof(int) * 3 * (size_t)Nprim);
    init_gamma_glint();
    precompute_gammaMij_T();
    double r[4];
    for (int m = 0; m < g_N; m++)
        for (int n = 0; n < Nprim; n++) {
            calculate_gamma_2d(m, n, r);
            out[(long)m * Nprim + n] = r[0];
        }
    free(g_xvec); g_xvec = &g_x0; g_xsize = 1; g_Pp = 1;
    free(g_qt); g_qt = NULL; free(g_prim); g_prim = NULL;
    return 0;
}

/* Polarised spectra for calculate_gamma's E weights (calculate_gamma.c:76-88,
 * 142-183): nine arrays over l = 0..n-1 in the order cl_tt, cl_te, cl_ee,
 * b_tt, b_te, b_ee, n_tt, n_te, n_ee. */
int ref_setup_pol_spectra(int n, const double *spec9, double fsky_t, double fsky_e)
{
    free(g_spec);
    g_spec = malloc(sizeof(double) * 9 * (size_t)n);
    memcpy(g_spec, spec9, sizeof(double) * 9 * (size_t)n);
    g_spec_n = n;
    fskyT = fsky_t;
    fskyE = fsky_e;
    return 0;
}

extern void precompute_gammaMij_E(void);

/* calculate_gamma_2d for every (late m, primordial n) with do_polarisation:
 * out[4][N][Nprim] = TTT, TTE, TEE, EEE.  qtT, qtE: [xsize][Pp][lmax_T+1]. */
int ref_gamma_transfer_pol(int xsize, const double *xvec, int Pp, const double *qtT, const double *qtE, int Nprim,
                           const int *prim, double dphi, double *out)
{
    g_xsize = xsize; g_Pp = Pp; g_Nprim = Nprim; deltaphi = dphi;
    g_xvec = malloc(sizeof(double) * (size_t)xsize);
    memcpy(g_xvec, xvec, sizeof(double) * (size_t)xsize);
    size_t nq = (size_t)xsize * Pp * (eflag_T_lmax + 1);
    g_qt = malloc(sizeof(double) * nq);
    g_qtE = malloc(sizeof(double) * nq);
    memcpy(g_qt, qtT, sizeof(double) * nq);
    memcpy(g_qtE, qtE, sizeof(double) * nq);
    g_prim = malloc(sizeof(int) * 3 * (size_t)Nprim);
    memcpy(g_prim, prim, sizeof(int) * 3 * (size_t)Nprim);
    init_gamma_glint();
    precompute_gammaMij_T();
    precompute_gammaMij_E();
    const long NP = (long)g_N * Nprim;
    double r[4];
    for (int m = 0; m < g_N; m++)
        for (int n = 0; n < Nprim; n++) {
            calculate_gamma_2d(m, n, r);
            for (int c = 0; c < 4; c++) out[c * NP + (long)m * Nprim + n] = r[c];
        }
    free(g_xvec); g_xvec = &g_x0; g_xsize = 1; g_Pp = 1;
    free(g_qt); g_qt = NULL; free(g_qtE); g_qtE = NULL; free(g_prim); g_prim = NULL;
    return 0;
}

/* ===================== primordial k-space side ===================== */
/* orthogonalisation.c (calculate_ortho), calculate_volume.c (calculate_weight),
 * calculate_eigen.c (calculate_eigen, integrate_template2) on the k-grid
 * tetrapyd: basis_prim[max+1][P] values on grid index i (get_basis_prim),
 * kmax (get_kmax), the primordial triples (find_perm_prim, g_prim). */
int alpha_points = 0;
static double *g_bprim;
static int g_Pprim, g_kgrid_max;
static double g_kmax = 1.0;
double get_basis_prim(int i, int j) { return g_bprim[(long)i * g_Pprim + j]; }
double get_kmax(void) { return g_kmax; }
double get_lambda(int i, int j) { (void)i; (void)j; return 0.0; }
int quad(int i, int j, int k, int l) { (void)i; (void)j; (void)k; (void)l; abort(); }
/* primordial template stand-in: the synthetic shape of ref_prim_eigen on the
 * grid index k/dk (separable tables are tabulated on grid indices; the bump
 * uses k/(k1+k2+k3), which the grid spacing cancels) */
typedef struct { double a1, a2, a3; } ref_shape_params; /* global.h:32-36 */
double shape3(double k1, double k2, double k3, ref_shape_params params)
{
    (void)params;
    const double dk = g_kmax / g_kgrid_max;
    return orc_shape_eval(&g_shape, (int)lround(k1 / dk), (int)lround(k2 / dk), (int)lround(k3 / dk));
}
/* Monte Carlo integration link stubs (calculate_ortho_mc is not exercised) */
struct refshim_rng_type;
struct refshim_rng;
struct refshim_monte_plain;
const struct refshim_rng_type *gsl_rng_default = NULL;
const struct refshim_rng_type *gsl_rng_env_setup(void) { abort(); }
struct refshim_rng *gsl_rng_alloc(const struct refshim_rng_type *T) { (void)T; abort(); }
void gsl_rng_free(struct refshim_rng *r) { (void)r; }
struct refshim_monte_plain *gsl_monte_plain_alloc(size_t dim) { (void)dim; abort(); }
int gsl_monte_plain_integrate(const void *f, const double xl[], const double xu[], size_t dim, size_t calls,
                              struct refshim_rng *r, struct refshim_monte_plain *st, double *res, double *err)
{ (void)f; (void)xl; (void)xu; (void)dim; (void)calls; (void)r; (void)st; (void)res; (void)err; abort(); }
void gsl_monte_plain_free(struct refshim_monte_plain *s) { (void)s; }

extern void calculate_ortho(int min, int max, ref_tetrapyd_limits *block, double *ortho);
extern void calculate_eigen(int min, int max, ref_shape_params params, ref_tetrapyd_limits *block, double *alpha);
extern void integrate_template2(int min, int max, ref_shape_params params, ref_tetrapyd_limits *block, double *res);
extern void decompose_tetrapyd_prim(ref_tetrapyd_limits *block, int rank, int nranks, int nthreads, int min, int max);

static void prim_install(int max, double kmax, int P, const double *basis, int N, const int *prim)
{
    g_kgrid_max = max;
    g_kmax = kmax;
    g_Pprim = P;
    free(g_bprim);
    g_bprim = malloc(sizeof(double) * (size_t)(max + 1) * P);
    memcpy(g_bprim, basis, sizeof(double) * (size_t)(max + 1) * P);
    g_Nprim = N;
    g_N = N;
    free(g_prim);
    g_prim = malloc(sizeof(int) * 3 * (size_t)N);
    memcpy(g_prim, prim, sizeof(int) * 3 * (size_t)N);
}

/* calculate_ortho over the whole k-grid tetrapyd on one rank and one thread:
 * out[N(N+1)/2], the packed upper triangle r <= s. */
int ref_prim_ortho(int min, int max, double kmax, int P, const double *basis, int N, const int *prim, double *out)
{
    prim_install(max, kmax, P, basis, N, prim);
    ref_tetrapyd_limits block[1];
    decompose_tetrapyd_prim(block, 0, 1, 1, min, max);
    for (long i = 0; i < (long)N * (N + 1) / 2; i++) out[i] = 0.0;
    calculate_ortho(min, max, block, out);
    return 0;
}

/* calculate_eigen and integrate_template2 for one synthetic shape (same
 * kinds as ref_project): alpha[N] and <S,S>. */
int ref_prim_eigen(int min, int max, double kmax, int P, const double *basis, int N, const int *prim, int kind,
                   int nterms, const double *tab, double c1, double c2, double c3, double sigma, double *alpha,
                   double *norm2)
{
    prim_install(max, kmax, P, basis, N, prim);
    g_shape.kind = kind;
    g_shape.nterms = nterms;
    g_shape.tab = tab;
    g_shape.lmax = max;
    g_shape.c1 = c1; g_shape.c2 = c2; g_shape.c3 = c3;
    g_shape.sigma = sigma;
    ref_tetrapyd_limits block[1];
    decompose_tetrapyd_prim(block, 0, 1, 1, min, max);
    ref_shape_params params = {0.0, 0.0, 0.0};
    for (int r = 0; r < N; r++) alpha[r] = 0.0;
    const int nt = omp_get_max_threads();
    omp_set_num_threads(1);  /* the block decomposition above is for one thread */
    calculate_eigen(min, max, params, block, alpha);
    *norm2 = 0.0;
    integrate_template2(min, max, params, block, norm2);
    omp_set_num_threads(nt);
    return 0;
}

/* ---- the 3D transfer Gamma (calculate_gamma_3d.c) ---------------------- */
#include "mkl.h"
#include "calculate_gamma_3d.h"

/* the qtilde l grid is l = 0..lmax (dense) */
int get_qtilde_T_lsize(void) { return eflag_T_lmax + 1; }
int get_qtilde_E_lsize(void) { return eflag_T_lmax + 1; }
int get_qtilde_T_lvec(int *v) { for (int l = 0; l <= eflag_T_lmax; l++) v[l] = l; return 0; }
int get_qtilde_E_lvec(int *v) { for (int l = 0; l <= eflag_T_lmax; l++) v[l] = l; return 0; }
double *get_basis_late_T_flat(void) { return g_basis; }

/* CBLAS dgemm semantics (row major), plain loops: C = alpha op(A) op(B) + beta C */
void cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int M, int N, int K, double alpha,
                 const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc)
{
    if (layout != CblasRowMajor) abort();
    for (int m = 0; m < M; m++)
        for (int n = 0; n < N; n++) {
            double s = 0.0;
            for (int k = 0; k < K; k++) {
                const double a = ta == CblasNoTrans ? A[(long)m * lda + k] : A[(long)k * lda + m];
                const double b = tb == CblasNoTrans ? B[(long)k * ldb + n] : B[(long)n * ldb + k];
                s += a * b;
            }
            C[(long)m * ldc + n] = alpha * s + beta * C[(long)m * ldc + n];
        }
}

extern void init_gamma_3Dint(void);

/* The reference's per-core barrier (local_barrier.c) synchronises the hardware
 * threads of one core; the glue runs one thread per core, for which the barrier
 * only flips its sense. */
void userCoreBarrier(barrier_t *bar) { bar->usersense = 1 - bar->usersense; }

/* gamma_3d_host (gamma_mpi.c:30-152) on one thread: init_gamma_3Dint, the
 * domain decomposition for one rank, calculate_gamma_TTT_3D_nested, and the
 * result [N][N] (the reference sizes it by the primordial term count, which
 * this glue ties to the late one: Nprim must equal N). */
int ref_gamma_3d(int xsize, const double *xvec, int Pp, const double *qt, int Nprim, const int *prim, double dphi,
                 double *out)
{
    if (Nprim != g_N) return -1;
    g_xsize = xsize; g_Pp = Pp; g_Nprim = Nprim; deltaphi = dphi;
    g_xvec = malloc(sizeof(double) * (size_t)xsize);
    memcpy(g_xvec, xvec, sizeof(double) * (size_t)xsize);
    size_t nq = (size_t)xsize * Pp * (eflag_T_lmax + 1);
    g_qt = malloc(sizeof(double) * nq);
    memcpy(g_qt, qt, sizeof(double) * nq);
    g_prim = malloc(sizeof(int) * 3 * (size_t)Nprim);
    memcpy(g_prim, prim, sizeof(int) * 3 * (size_t)Nprim);
    init_gamma_3Dint();
    const int N = g_N, Npad = (N + 7) & ~7, xpad = (xsize + 7) & ~7;
    double *xdiff = calloc((size_t)xsize, sizeof(double)), *ixdiff = calloc((size_t)xsize, sizeof(double));
    for (int i = 0; i < xsize - 1; i++) { xdiff[i] = g_xvec[i + 1] - g_xvec[i]; ixdiff[i] = 1.0 / xdiff[i]; }
    corebarrier_t cb = {0};
    barrier_t bar = {1, 0, 1, &cb};
    thread_g3d_data_t td;
    memset(&td, 0, sizeof td);
    td.mvec = calloc((size_t)Npad * Npad, sizeof(double));
    td.intgrlvec = calloc((size_t)MAXBLOCKSIZE * Npad, sizeof(double));
    td.plijkz = calloc((size_t)MAXBLOCKSIZE * Npad, sizeof(double));
    td.yvec = calloc((size_t)xpad, sizeof(double));
    td.xsize = xsize;
    td.xvec = g_xvec;
    td.xdiff = xdiff;
    td.ixdiff = ixdiff;
    td.bar = &bar;
    omp_set_num_threads(1);
    #pragma omp parallel num_threads(1)
    {
        decompose_gamma_TTT_3D_mpi(&td, 0, 1, 0.0);
        calculate_gamma_TTT_3D_nested(&td, MAXBLOCKSIZE);
    }
    for (int m = 0; m < N; m++)
        for (int n = 0; n < N; n++) out[(long)m * N + n] = td.mvec[(long)m * Npad + n];
    free(td.mvec); free(td.intgrlvec); free(td.plijkz); free(td.yvec); free(xdiff); free(ixdiff);
    free(g_xvec); g_xvec = &g_x0; g_xsize = 1; g_Pp = 1;
    free(g_qt); g_qt = NULL; free(g_prim); g_prim = NULL;
    return 0;
}
