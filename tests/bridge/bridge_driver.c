/* Test driver for modal_ref_bridge.c: plays the part of ortho_late_mpi.c's
 * Gamma loop (init_orthol_glint, calculate_orthoMij_T over all pairs,
 * sync_orthoMij, calculate_orthol over the upper triangle; ortho_late_mpi.c:
 * 170-287) against accessors that serve tables read from a binary input file,
 * as fixed_data.c serves the basis and mode lists.  Test infrastructure.
 *
 * Input (native doubles/ints): lmin lmax P N pol [lminE lmaxE PE], basis
 * [L][P], triples [N][3], [E basis [LE][PE], tte, tee, eee [N][3] each];
 * nodes are produced by the asy() stand-in below from a nodes file.
 * Output: npol x N x N doubles of calculate_orthol's results. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

double init_orthol_glint(void);
void calculate_orthoMij_T(int i, int j);
void sync_orthoMij(void);
int calculate_orthol(int m, int n, double *result);

int eflag_T_lmin, eflag_T_lmax, eflag_E_lmin, eflag_E_lmax, do_polarisation;
static int P, PE, N;
static double *basis, *basisE, *nodes, *weights;
static int *tri[4], nnodes;

int get_pmax_late_T(void) { return P - 1; }
int get_pmax_late_E(void) { return PE - 1; }
int get_terms_late(void) { return N; }
double get_basis_late_T(int i, int j) { return basis[(size_t)i * P + j]; }
double get_basis_late_E(int i, int j) { return basisE[(size_t)i * PE + j]; }
static void perm(int t, int r, int *a, int *b, int *c) { *a = tri[t][3 * r]; *b = tri[t][3 * r + 1]; *c = tri[t][3 * r + 2]; }
void find_perm_late_TTT(int r, int *a, int *b, int *c) { perm(0, r, a, b, c); }
void find_perm_late_TTE(int r, int *a, int *b, int *c) { perm(1, r, a, b, c); }
void find_perm_late_TEE(int r, int *a, int *b, int *c) { perm(2, r, a, b, c); }
void find_perm_late_EEE(int r, int *a, int *b, int *c) { perm(3, r, a, b, c); }
/* asy() stand-in: returns the nodes and weights given to the driver */
int asy(double *x, double *w, unsigned long n)
{
    if ((int)n != nnodes) { fprintf(stderr, "asy: asked for %lu nodes, have %d\n", n, nnodes); exit(2); }
    memcpy(x, nodes, sizeof(double) * n);
    memcpy(w, weights, sizeof(double) * n);
    return 0;
}

static void rd(FILE *f, void *p, size_t sz, size_t n)
{
    if (fread(p, sz, n, f) != n) { fprintf(stderr, "short input\n"); exit(2); }
}

int main(int argc, char **argv)
{
    if (argc != 3) { fprintf(stderr, "usage: %s input output\n", argv[0]); return 2; }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[5];
    rd(f, hdr, sizeof(int), 5);
    eflag_T_lmin = hdr[0]; eflag_T_lmax = hdr[1]; P = hdr[2]; N = hdr[3]; do_polarisation = hdr[4];
    const int L = eflag_T_lmax - eflag_T_lmin + 1;
    basis = malloc(sizeof(double) * (size_t)L * P);
    rd(f, basis, sizeof(double), (size_t)L * P);
    tri[0] = malloc(sizeof(int) * 3 * (size_t)N);
    rd(f, tri[0], sizeof(int), 3 * (size_t)N);
    if (do_polarisation) {
        int e[3];
        rd(f, e, sizeof(int), 3);
        eflag_E_lmin = e[0]; eflag_E_lmax = e[1]; PE = e[2];
        const int LE = eflag_E_lmax - eflag_E_lmin + 1;
        basisE = malloc(sizeof(double) * (size_t)LE * PE);
        rd(f, basisE, sizeof(double), (size_t)LE * PE);
        for (int t = 1; t < 4; t++) {
            tri[t] = malloc(sizeof(int) * 3 * (size_t)N);
            rd(f, tri[t], sizeof(int), 3 * (size_t)N);
        }
    }
    rd(f, &nnodes, sizeof(int), 1);
    nodes = malloc(sizeof(double) * nnodes);
    weights = malloc(sizeof(double) * nnodes);
    rd(f, nodes, sizeof(double), nnodes);
    rd(f, weights, sizeof(double), nnodes);
    fclose(f);

    /* ortho_late_mpi.c:170-287 on one rank */
    init_orthol_glint();
    for (int i = 0; i < P; i++)
        for (int j = 0; j < P; j++) calculate_orthoMij_T(i, j);
    sync_orthoMij();
    const int npol = do_polarisation ? 4 : 1;
    double *out = calloc((size_t)npol * N * N, sizeof(double));
    double r[4];
    for (int i = 0; i < N; i++)
        for (int j = i; j < N; j++) {
            calculate_orthol(i, j, r);
            for (int c = 0; c < npol; c++)
                out[(size_t)c * N * N + (size_t)i * N + j] = out[(size_t)c * N * N + (size_t)j * N + i] = r[c];
        }
    FILE *o = fopen(argv[2], "wb");
    if (!o || fwrite(out, sizeof(double), (size_t)npol * N * N, o) != (size_t)npol * N * N) return 3;
    fclose(o);
    return 0;
}
