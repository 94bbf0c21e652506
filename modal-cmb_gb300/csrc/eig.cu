// eig.cu -- PCA branch of the orthogonalisation (ortho_late_mpi.c:775-805),
// taken when pca_flag == 0 or the normalised Gamma is not positive definite.
//
// The symmetric eigen-decomposition of the normalised Gamma (the reference's
// gsl_eigen_symmv + gsl_eigen_symmv_sort descending, :775-776) is the
// cuSOLVER library routine cusolverDnDsyevdx in FP64 on the GPU, asked only for
// the eigenpairs the outputs use (eigenvalues above the cut).  The outputs
// follow the reference exactly, with eigenvalues e_i in descending order and
// r = the number of leading positive eigenvalues:
//   lambda[i][j]    = V[j][i] / (norm_j sqrt(e_i))   for i < r, else 0
//   lambdainv[i][j] = norm_i V[i][j] sqrt(e_j)        for j < r, else 0
// stored as lambdal and orthol.  Eigenvector signs are those of the solver.
#include <cusolverDn.h>
#include "common.cuh"

namespace modal {

// Count leading eigenvalues above floor * e_max in descending order (W holds the
// meig returned eigenvalues ascending); floor = 0 is the reference's rule
// (leading positive ones).
__global__ void k_pca_rank(int meig, const double *__restrict__ W, double floor, int *rank)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double cut = (floor > 0.0 && meig > 0) ? floor * W[meig - 1] : 0.0;
    int r = 0;
    for (int i = 0; i < meig && W[meig - 1 - i] > cut; i++) r = i + 1;
    *rank = r;
}

// V_rm: row-major buffer whose row a < meig holds the eigenvector of ascending index a.
// lambdainv: the lower triangle of orthol (zero above the diagonal), the matrix
// eigenmodetoday_mpi.c:148-160 builds from the orthol file for modesR.
__global__ void k_pca_outputs(int N, int meig, const double *__restrict__ V_rm, const double *__restrict__ W,
                              const double *__restrict__ norm, const int *__restrict__ rank,
                              double *__restrict__ orthol, double *__restrict__ lambdal, double *__restrict__ lambdainv)
{
    size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)N * N) return;
    const int r = *rank;
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

// One cuSOLVER handle per context, bound to the context's stream.  Creating a
// handle sets up the library's state on the device; keeping it saves that cost
// on every orthogonalisation and pruning call.
modal_status solver_handle(modal_ctx *ctx, void **out)
{
    if (!ctx->solver) {
        cusolverDnHandle_t h = nullptr;
        if (cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS) { set_error("cusolverDnCreate failed"); return MODAL_ERR_CUDA; }
        if (cusolverDnSetStream(h, ctx->stream) != CUSOLVER_STATUS_SUCCESS) {
            cusolverDnDestroy(h);
            set_error("cusolverDnSetStream failed");
            return MODAL_ERR_CUDA;
        }
        ctx->solver = h;
    }
    *out = ctx->solver;
    return MODAL_OK;
}

void solver_release(modal_ctx *ctx)
{
    if (ctx->solver) cusolverDnDestroy(static_cast<cusolverDnHandle_t>(ctx->solver));
    ctx->solver = nullptr;
}

modal_status eig_pca_dev(modal_ctx *ctx)
{
    const int N = ctx->N;
    void *hv = nullptr;
    MODAL_TRY(solver_handle(ctx, &hv));
    cusolverDnHandle_t h = static_cast<cusolverDnHandle_t>(hv);
    modal_status st = MODAL_OK;
    int lwork = 0;
    double *A = ctx->chol.as<double>();  // symmetric: row-major == column-major
    if (ensure(ctx->scratch2, sizeof(double) * (size_t)N) != MODAL_OK) return MODAL_ERR_NOMEM;
    double *W = ctx->scratch2.as<double>();
    // Only eigenpairs above the cut are used, so the subset solver computes those
    // alone: eigenvalues in (vl, inf).  The normalised Gamma has a unit diagonal,
    // so e_max >= 1 and vl = floor (just below) never exceeds floor * e_max; the
    // exact cut is applied to the returned eigenvalues.  vl = 0 gives every
    // positive eigenvalue, the reference's rule.
    const double vl = ctx->pca_floor > 0.0 ? ctx->pca_floor * (1.0 - 1e-12) : 0.0, vu = 1e300;
    int meig = 0;
    if (cusolverDnDsyevdx_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUSOLVER_EIG_RANGE_V, CUBLAS_FILL_MODE_LOWER, N, A, N,
                                     vl, vu, 0, 0, &meig, W, &lwork) != CUSOLVER_STATUS_SUCCESS) {
        set_error("syevdx_bufferSize failed");
        return MODAL_ERR_CUDA;
    }
    st = ensure(ctx->scratch, sizeof(double) * (size_t)lwork + 64);
    if (st != MODAL_OK) return st;
    int *devinfo = ctx->info.as<int>() + 1;
    int *rank = ctx->info.as<int>() + 2;
    cusolverStatus_t cs = cusolverDnDsyevdx(h, CUSOLVER_EIG_MODE_VECTOR, CUSOLVER_EIG_RANGE_V, CUBLAS_FILL_MODE_LOWER, N,
                                            A, N, vl, vu, 0, 0, &meig, W, ctx->scratch.as<double>(), lwork, devinfo);
    if (cs != CUSOLVER_STATUS_SUCCESS) { set_error("cusolverDnDsyevdx failed (%d)", (int)cs); return MODAL_ERR_CUDA; }
    int hinfo = 0;
    MODAL_CUDA(cudaMemcpyAsync(&hinfo, devinfo, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MODAL_CUDA(cudaStreamSynchronize(ctx->stream));
    if (hinfo != 0) { set_error("syevdx info=%d", hinfo); return MODAL_ERR_NOCONV; }
    if (meig < 0 || meig > N) { set_error("syevdx returned %d eigenpairs for N=%d", meig, N); return MODAL_ERR_CUDA; }
    k_pca_rank<<<1, 1, 0, ctx->stream>>>(meig, W, ctx->pca_floor, rank);
    MODAL_TRY(launched(ctx, "pca_rank"));
    size_t NN = (size_t)N * N;
    MODAL_TRY(ensure(ctx->linv, sizeof(double) * NN));
    k_pca_outputs<<<ceil_div((long)NN, 256), 256, 0, ctx->stream>>>(N, meig, A, W, ctx->norm.as<double>(), rank,
                                                                       ctx->orthol.as<double>(), ctx->lambdal.as<double>(),
                                                                       ctx->linv.as<double>());
    MODAL_TRY(launched(ctx, "pca_outputs"));
    int hr = 0;
    MODAL_CUDA(cudaMemcpyAsync(&hr, rank, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MODAL_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->ortho_rank = hr;
    return MODAL_OK;
}

}  // namespace modal
