/* Driver glue for the reference's basis_optimisation_mpi.c main(), compiled in
 * place as a test oracle (oracle/_ref/basis_prune_ref).  Test infrastructure.
 *
 * The reference reads its inputs from fixed paths through array_read and
 * load_txt_int; here those read the files named by the environment:
 *   MODAL_PRUNE_N      number of modes N
 *   MODAL_PRUNE_GAMMA  raw FP64 N x N Gamma (the "master_orthol" file)
 *   MODAL_PRUNE_FAIL   text file of failed mode indices, or unset for none
 * MKL's LAPACKE_dsyevr (absent) is replaced by a cyclic Jacobi iteration on the
 * upper triangle, returning the il..iu smallest eigenvalues. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "mkl_lapacke.h"

int eflag_order_late = 0;
int eflag_T_lmax = 0;
int eflag_E_lmax = 0;

static int env_n(void)
{
    const char *s = getenv("MODAL_PRUNE_N");
    return s ? atoi(s) : 0;
}

int initilise(char *inifile)
{
    (void)inifile;
    return 0;
}
int set_terms_late(void) { return 0; }
int get_terms_late(void) { return env_n(); }

void find_perm_late_TTT(int r, int *p1, int *p2, int *p3)
{
    *p1 = r;
    *p2 = 0;
    *p3 = 0;
}

double csecond(void) { return (double)clock() / CLOCKS_PER_SEC; }

double **create_array(int dim_x, int dim_y)
{
    double **rows = malloc(sizeof(double *) * (size_t)dim_x);
    double *data = calloc((size_t)dim_x * dim_y, sizeof(double));
    for (int i = 0; i < dim_x; i++) rows[i] = data + (size_t)i * dim_y;
    return rows;
}

void array_read(int *n, char *filename, double *grid)
{
    (void)filename;
    const char *path = getenv("MODAL_PRUNE_GAMMA");
    FILE *f = path ? fopen(path, "rb") : NULL;
    if (!f || fread(grid, sizeof(double), (size_t)*n, f) != (size_t)*n) {
        fprintf(stderr, "prune_glue: cannot read %d doubles from MODAL_PRUNE_GAMMA\n", *n);
        exit(1);
    }
    fclose(f);
}

int load_txt_int(char *filename, int columns, int *values, int *size)
{
    (void)filename;
    (void)columns;
    *size = 0;
    const char *path = getenv("MODAL_PRUNE_FAIL");
    FILE *f = path ? fopen(path, "r") : NULL;
    if (!f) return 0;
    int v;
    while (fscanf(f, "%d", &v) == 1) values[(*size)++] = v;
    fclose(f);
    return 0;
}

int MPI_Init(int *argc, char ***argv)
{
    (void)argc;
    (void)argv;
    return 0;
}
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(int c, int *rank)
{
    (void)c;
    *rank = 0;
    return 0;
}
int MPI_Comm_size(int c, int *size)
{
    (void)c;
    *size = 1;
    return 0;
}
int MPI_Barrier(int c)
{
    (void)c;
    return 0;
}
int MPI_Allreduce(const void *s, void *r, int n, int t, int op, int c)
{
    (void)op;
    (void)c;
    memcpy(r, s, (size_t)n * (t == 2 ? sizeof(int) : sizeof(double)));
    return 0;
}

static int cmp_double(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

/* Eigenvalues il..iu (1-based, ascending) of the symmetric matrix whose upper
 * triangle is given (row-major: a[i*lda + j], j >= i), by cyclic Jacobi
 * rotations until the off-diagonal mass is below 1e-30 of the total. */
MKL_INT LAPACKE_dsyevr(int layout, char jobz, char range, char uplo, MKL_INT n, double *a, MKL_INT lda, double vl,
                       double vu, MKL_INT il, MKL_INT iu, double abstol, MKL_INT *m, double *w, double *z, MKL_INT ldz,
                       MKL_INT *isuppz)
{
    (void)layout; (void)jobz; (void)range; (void)uplo; (void)vl; (void)vu; (void)abstol; (void)z; (void)ldz;
    (void)isuppz;
    double *s = malloc(sizeof(double) * (size_t)n * n);
    for (int i = 0; i < n; i++)
        for (int j = i; j < n; j++) s[(size_t)i * n + j] = s[(size_t)j * n + i] = a[(size_t)i * lda + j];
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                double v = s[(size_t)i * n + j] * s[(size_t)i * n + j];
                tot += v;
                if (i != j) off += v;
            }
        if (off <= 1e-30 * tot) break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                double apq = s[(size_t)p * n + q];
                if (apq == 0.0) continue;
                double app = s[(size_t)p * n + p], aqq = s[(size_t)q * n + q];
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < n; k++) {
                    double akp = s[(size_t)k * n + p], akq = s[(size_t)k * n + q];
                    s[(size_t)k * n + p] = c * akp - sn * akq;
                    s[(size_t)k * n + q] = sn * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = s[(size_t)p * n + k], aqk = s[(size_t)q * n + k];
                    s[(size_t)p * n + k] = c * apk - sn * aqk;
                    s[(size_t)q * n + k] = sn * apk + c * aqk;
                }
            }
    }
    double *e = malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; i++) e[i] = s[(size_t)i * n + i];
    qsort(e, (size_t)n, sizeof(double), cmp_double);
    *m = iu - il + 1;
    for (int i = 0; i < *m; i++) w[i] = e[il - 1 + i];
    free(e);
    free(s);
    return 0;
}
