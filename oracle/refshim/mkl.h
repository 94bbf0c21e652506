/* Stand-in for <mkl.h>: tetrapyd_tools.c includes it without calling into it;
 * calculate_gamma_3d.c calls cblas_dgemm, implemented in ref_glue.c. */
#ifndef REFSHIM_MKL_H
#define REFSHIM_MKL_H
typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
void cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int M, int N, int K, double alpha,
                 const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc);
#endif
