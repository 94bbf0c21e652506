// eig.cu -- PCA branch of the orthogonalisation (ortho_late_mpi.c:775-805),
// taken when pca_flag == 0 or the normalised Gamma is not positive definite.
//
// The symmetric eigen-decomposition of the normalised Gamma (the reference's
// gsl_eigen_symmv + gsl_eigen_symmv_sort descending, :775-776) is the
// library's own FP64 eigensolver (syev.cu): every eigenvalue, and the
// eigenvectors of the kept ones only.  The outputs follow the reference
// exactly, with eigenvalues e_i in descending order and r = the number of
// leading positive eigenvalues (or of those above floor * e_max):
//   lambda[i][j]    = V[j][i] / (norm_j sqrt(e_i))   for i < r, else 0
//   lambdainv[i][j] = norm_i V[i][j] sqrt(e_j)        for j < r, else 0
// stored as lambdal and orthol.  Eigenvector signs are those of the solver.
#include "common.cuh"

namespace modal {

// V_rm: row-major buffer whose row a < meig holds the eigenvector of W[a]
// (W: the meig kept eigenvalues, ascending).
// lambdainv: the lower triangle of orthol (zero above the diagonal), the matrix
// eigenmodetoday_mpi.c:148-160 builds from the orthol file for modesR.
__global__ void k_pca_outputs(int N, int meig, const double *__restrict__ V_rm, const double *__restrict__ W,
                              const double *__restrict__ norm, double *__restrict__ orthol,
                              double *__restrict__ lambdal, double *__restrict__ lambdainv)
{
    size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)N * N) return;
    const int r = meig;
    int i = (int)(e / N), j = (int)(e % N);
    // lambda[i][j] = V[j][desc i] / (norm_j sqrt(e_desc i))
    double lam = 0.0;
    if (i < r) {
        int a = meig - 1 - i;
        lam = V_rm[(size_t)a * N + j] / (norm[j] * sqrt(W[a]));
    }
    double inv = 0.0;
    if (j < r) {
        int a = meig - 1 - j;
        inv = norm[i] * V_rm[(size_t)a * N + i] * sqrt(W[a]);
    }
    lambdal[e] = lam;
    orthol[e] = inv;
    lambdainv[e] = (i >= j) ? inv : 0.0;
}

namespace {
// Leading eigenvalues (descending) above floor * e_max; floor 0: the leading
// positive ones, the reference's rule (ortho_late_mpi.c:786-789).
struct PcaCut { double floor; };
int pca_select(const double *w, int n, void *arg, int *first)
{
    const double floor = static_cast<PcaCut *>(arg)->floor;
    const double cut = (floor > 0.0 && n > 0) ? floor * w[n - 1] : 0.0;
    int r = 0;
    for (int i = 0; i < n && w[n - 1 - i] > cut; i++) r = i + 1;
    *first = n - r;
    return r;
}
}  // namespace

modal_status eig_pca_dev(modal_ctx *ctx)
{
    const int N = ctx->N;
    const size_t NN = (size_t)N * N;
    double *A = ctx->chol.as<double>();
    MODAL_TRY(ensure(ctx->scratch, sizeof(double) * (NN + (size_t)N)));
    double *V = ctx->scratch.as<double>(), *W = V + NN;
    PcaCut cut{ctx->pca_floor};
    int r = 0, first = 0;
    MODAL_TRY(syev_dev(ctx, N, A, W, V, pca_select, &cut, &r, &first));
    MODAL_TRY(ensure(ctx->linv, sizeof(double) * NN));
    k_pca_outputs<<<ceil_div((long)NN, 256), 256, 0, ctx->stream>>>(N, r, V, W + first, ctx->norm.as<double>(),
                                                                       ctx->orthol.as<double>(), ctx->lambdal.as<double>(),
                                                                       ctx->linv.as<double>());
    MODAL_TRY(launched(ctx, "pca_outputs"));
    ctx->ortho_rank = r;
    return MODAL_OK;
}

}  // namespace modal
