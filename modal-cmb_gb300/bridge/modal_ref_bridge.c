/* modal_ref_bridge.c -- the Gamma entry points of orthogonalisation_late.c
 * (init_orthol_glint :23-97, calculate_orthoMij_T/E :99-157, sync_orthoMij
 * :159-237, calculate_orthol :239-336) over libmodal_gb300.
 *
 * Link it into a Modal-CMB driver (ortho_late_mpi.c, modes_from_file_mpi.c)
 * in place of those five functions; the driver, fixed_data.c and the file
 * formats stay as they are.  The rest of orthogonalisation_late.c (plijk_*,
 * rlijk_*, bijk_*, calculate_orthol_3D) is still needed: compile it with the
 * five names moved out of the way, e.g.
 *   cc -c orthogonalisation_late.c -Dinit_orthol_glint=cpu_init_orthol_glint \
 *      -Dcalculate_orthoMij_T=cpu_calculate_orthoMij_T -Dcalculate_orthoMij_E=cpu_calculate_orthoMij_E \
 *      -Dsync_orthoMij=cpu_sync_orthoMij -Dcalculate_orthol=cpu_calculate_orthol
 *   cc -c modal_ref_bridge.c -I<repo>/include
 *   cc ... -L<repo>/modal-cmb_gb300 -lmodal_gb300 -Wl,-rpath,<repo>/modal-cmb_gb300
 *
 * The quadrature is the reference's own asy() (gl_integration.c:46), passed to
 * the library, so Gamma matches the CPU code to rounding; define
 * MODAL_BRIDGE_GPU_NODES to use the library's GPU nodes instead.  On the first
 * calculate_orthol the whole N x N Gamma (and, with do_polarisation, the TTE,
 * TEE and EEE matrices) is computed on the GPU; every call then reads it.
 * Failures print the library's message and exit(1), as the reference does on
 * I/O errors.
 */
#include <stdio.h>
#include <stdlib.h>
#include "modal_gb300.h"

/* from the reference: parameter.c globals and fixed_data.c accessors (global.h) */
extern int eflag_T_lmin, eflag_T_lmax, eflag_E_lmin, eflag_E_lmax, do_polarisation;
extern int get_pmax_late_T(void), get_pmax_late_E(void), get_terms_late(void);
extern double get_basis_late_T(int i, int j), get_basis_late_E(int i, int j);
extern void find_perm_late_TTT(int r, int *p1, int *p2, int *p3);
extern void find_perm_late_TTE(int r, int *p1, int *p2, int *p3);
extern void find_perm_late_TEE(int r, int *p1, int *p2, int *p3);
extern void find_perm_late_EEE(int r, int *p1, int *p2, int *p3);
extern int asy(double *nodes, double *weights, unsigned long n);

static modal_ctx *g_ctx;
static double *g_gamma;     /* [N][N] */
static double *g_pol[3];    /* TTE, TEE, EEE [N][N] */
static int g_N;

static void check(modal_status s, const char *what)
{
    if (s != MODAL_OK) {
        fprintf(stderr, "modal %s: %s\n", what, modal_last_error());
        exit(1);
    }
}

static double *basis_table(int lsize, int P, double (*get)(int, int))
{
    double *q = malloc(sizeof(double) * (size_t)lsize * P);
    for (int l = 0; l < lsize; l++)
        for (int p = 0; p < P; p++) q[(size_t)l * P + p] = get(l, p);
    return q;
}

static int *mode_table(int N, void (*perm)(int, int *, int *, int *))
{
    int *t = malloc(sizeof(int) * 3 * (size_t)N);
    for (int n = 0; n < N; n++) perm(n, &t[3 * n], &t[3 * n + 1], &t[3 * n + 2]);
    return t;
}

double init_orthol_glint(void)
{
    const int lminT = eflag_T_lmin, lmaxT = eflag_T_lmax, PT = get_pmax_late_T() + 1;
    g_N = get_terms_late();
    if (!g_ctx) check(modal_ctx_create(0, &g_ctx), "ctx_create");
    double *qT = basis_table(lmaxT - lminT + 1, PT, get_basis_late_T);
    int *ttt = mode_table(g_N, find_perm_late_TTT);
    check(modal_set_basis(g_ctx, lminT, lmaxT, PT, qT), "set_basis");
    check(modal_set_modes(g_ctx, g_N, ttt), "set_modes");
    int lmax = lmaxT;
    if (do_polarisation == 1) {
        const int lminE = eflag_E_lmin, lmaxE = eflag_E_lmax, PE = get_pmax_late_E() + 1;
        double *qE = basis_table(lmaxE - lminE + 1, PE, get_basis_late_E);
        int *tte = mode_table(g_N, find_perm_late_TTE), *tee = mode_table(g_N, find_perm_late_TEE);
        int *eee = mode_table(g_N, find_perm_late_EEE);
        check(modal_set_basis_e(g_ctx, lminE, lmaxE, PE, qE), "set_basis_e");
        check(modal_set_modes_pol(g_ctx, tte, tee, eee), "set_modes_pol");
        if (lmaxE > lmax) lmax = lmaxE;
        free(qE); free(tte); free(tee); free(eee);
    }
#ifndef MODAL_BRIDGE_GPU_NODES
    const int npt = 3 * lmax / 2 + 1;  /* orthogonalisation_late.c:37 */
    double *x = malloc(sizeof(double) * npt), *w = malloc(sizeof(double) * npt);
    asy(x, w, (unsigned long)npt);
    check(modal_set_gl(g_ctx, npt, x, w), "set_gl");
    free(x); free(w);
#endif
    check(modal_init_glint(g_ctx), "init_glint");
    free(qT); free(ttt);
    free(g_gamma); g_gamma = NULL;
    for (int f = 0; f < 3; f++) { free(g_pol[f]); g_pol[f] = NULL; }
    return 0;
}

/* the M tables are built for all (i,j) by init_orthol_glint; one GPU needs no reduction */
void calculate_orthoMij_T(int i, int j) { (void)i; (void)j; }
void calculate_orthoMij_E(int i, int j) { (void)i; (void)j; }
void sync_orthoMij(void) {}

int calculate_orthol(int m, int n, double *result)
{
    const size_t N = (size_t)g_N;
    if (!g_gamma) {
        g_gamma = malloc(sizeof(double) * N * N);
        check(modal_gamma(g_ctx, MODAL_PREC_FP64, g_gamma), "gamma");
        if (do_polarisation == 1) {
            for (int f = 0; f < 3; f++) g_pol[f] = malloc(sizeof(double) * N * N);
            check(modal_gamma_pol(g_ctx, g_pol[0], g_pol[1], g_pol[2]), "gamma_pol");
        }
    }
    result[0] = g_gamma[(size_t)m * N + n];
    if (do_polarisation == 1)
        for (int f = 0; f < 3; f++) result[1 + f] = g_pol[f][(size_t)m * N + n];
    return 0;
}
