/* Stand-in for <mkl_lapacke.h> (MKL is absent): declares the one LAPACKE call
 * basis_optimisation_mpi.c makes.  prune_glue.c implements it with a cyclic
 * Jacobi eigenvalue iteration (test oracle only). */
#ifndef REFSHIM_MKL_LAPACKE_H
#define REFSHIM_MKL_LAPACKE_H
typedef int MKL_INT;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
MKL_INT LAPACKE_dsyevr(int layout, char jobz, char range, char uplo, MKL_INT n, double *a, MKL_INT lda, double vl,
                       double vu, MKL_INT il, MKL_INT iu, double abstol, MKL_INT *m, double *w, double *z, MKL_INT ldz,
                       MKL_INT *isuppz);
#endif
