// prune.cu -- greedy basis pruning (basis_optimisation_mpi.c:184-337) and the
// smallest-eigenvalue objective of the normalised Gamma with its gradient.
//
// The reference normalises Gamma to unit diagonal over the active modes
// (array = ortho / (norm_i norm_j), :184-190), then repeatedly removes the mode
// whose removal leaves the largest smallest eigenvalue: for each candidate m it
// copies the leave-one-out minor and calls LAPACKE_dsyevr for its smallest
// eigenvalue (:256-281), takes the first maximum (:287-297) and deletes that
// row and column (:301-312) -- n eigenproblems of size n-1 per step.
//
// Here one eigendecomposition per step serves every candidate.  With
// A = V diag(lambda) V^T, the eigenvalues mu of the principal minor without row
// and column m are the roots of the secular function
//   g_m(mu) = sum_i V[m][i]^2 / (lambda_i - mu),
// because det(mu I - A_{-m}) / det(mu I - A) = [(mu I - A)^{-1}]_{mm}.  The
// smallest root lies in (lambda_1, lambda_2) (interlacing), where g_m increases
// from -inf to +inf, so bisection on delta = mu - lambda_1 in (0, lambda_2 -
// lambda_1) finds it to the last bit; with V[m][1] = 0 or lambda_1 = lambda_2 it
// is lambda_1 itself.  Per step: one eigen-decomposition of size n (the
// library's own FP64 eigensolver, syev.cu) and one warp per candidate for the
// root, O(n^3) instead of the reference's O(n^4).
// The argmax and the list update run on the host, exactly as the reference's.
#include <vector>
#include "common.cuh"

namespace modal {

namespace {

// Ahat[i][j] = gamma[i][j] / (norm_i norm_j), norm_i = sqrt(gamma_ii)
// (the reference's expression and evaluation order, :184-190).
__global__ void k_prune_normalise(int N, const double *__restrict__ gamma, double *__restrict__ Ahat)
{
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)N * N) return;
    const int i = (int)(e / N), j = (int)(e - (long)i * N);
    const double ni = sqrt(gamma[(size_t)i * N + i]), nj = sqrt(gamma[(size_t)j * N + j]);
    Ahat[e] = gamma[e] / (ni * nj);
}

// A[i][j] = Ahat[list[i]][list[j]] for the n active modes.
__global__ void k_prune_gather(int n, int N, const double *__restrict__ Ahat, const int *__restrict__ list,
                               double *__restrict__ A)
{
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)n * n) return;
    const int i = (int)(e / n), j = (int)(e - (long)i * n);
    A[e] = Ahat[(size_t)list[i] * N + list[j]];
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One warp per candidate m: smallest eigenvalue of the minor without m.
// V: eigenvectors as rows [n][n] (V[m + i*n] = component m of eigenvector i),
// W: eigenvalues ascending.  n == 2: the 1x1 minor's entry.
__global__ void k_prune_secular(int n, int N, const double *__restrict__ V, const double *__restrict__ W,
                                const double *__restrict__ Ahat, const int *__restrict__ list,
                                double *__restrict__ lam)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    const int m = warp;
    if (n == 2) {
        if (lane == 0) {
            const int o = list[1 - m];
            lam[m] = Ahat[(size_t)o * N + o];
        }
        return;
    }
    const double l1 = W[0];
    const double z0 = V[m];
    const double z02 = z0 * z0;
    double hi = W[1] - l1;
    if (z02 == 0.0 || !(hi > 0.0)) {
        if (lane == 0) lam[m] = l1;
        return;
    }
    double lo = 0.0;
    for (int it = 0; it < 200; it++) {
        const double mid = 0.5 * (lo + hi);
        if (!(mid > lo && mid < hi)) break;
        double s = 0.0;
        for (int i = 1 + lane; i < n; i += 32) {
            const double zi = V[m + (size_t)i * n];
            s += zi * zi / ((W[i] - l1) - mid);
        }
        s = __shfl_sync(0xffffffffu, warp_sum(s), 0) - z02 / mid;
        if (s < 0.0) lo = mid;
        else hi = mid;
    }
    if (lane == 0) lam[m] = l1 + 0.5 * (lo + hi);
}

// Upstream of lambda_min(Ahat) with respect to Gamma:
//   G[i][j] = vt_i vt_j - delta_ij lam v_i^2 / gamma_ii,  vt_i = v_i / sqrt(gamma_ii).
__global__ void k_lmin_upstream(int N, const double *__restrict__ gamma, const double *__restrict__ v, double lam,
                                double *__restrict__ G)
{
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)N * N) return;
    const int i = (int)(e / N), j = (int)(e - (long)i * N);
    const double gi = gamma[(size_t)i * N + i], gj = gamma[(size_t)j * N + j];
    double g = v[i] * v[j] / (sqrt(gi) * sqrt(gj));
    if (i == j) g -= lam * v[i] * v[i] / gi;
    G[e] = g;
}

// every eigenvector (pruning reads them all)
int select_all(const double *, int n, void *, int *first)
{
    *first = 0;
    return n;
}

}  // namespace

}  // namespace modal

using namespace modal;

extern "C" {

modal_status modal_basis_prune(modal_ctx *c, int N, const double *gamma, int nfail, const int *faillist, int *order,
                               double *lambda_min)
{
    if (!c || N < 1 || !order || !lambda_min || nfail < 0 || nfail >= N || (nfail > 0 && !faillist)) {
        set_error("modal_basis_prune: bad arguments (N=%d, nfail=%d)", N, nfail);
        return MODAL_ERR_ARG;
    }
    if (!gamma && !(c->have_gamma && c->N == N)) {
        set_error("modal_basis_prune: pass gamma or compute the FP64 Gamma of N=%d modes first", N);
        return MODAL_ERR_STATE;
    }
    std::vector<char> failed(N, 0);
    for (int j = 0; j < nfail; j++) {
        const int f = faillist[j];
        if (f < 0 || f >= N || failed[f]) {
            set_error("modal_basis_prune: fail-list entry %d (= %d) out of range or repeated", j, f);
            return MODAL_ERR_ARG;
        }
        failed[f] = 1;
    }
    std::vector<int> list;
    for (int i = 0; i < N; i++)
        if (!failed[i]) list.push_back(i);
    const int n0 = (int)list.size();
    MODAL_CUDA(cudaSetDevice(c->device));
    StageTimer t(c, MODAL_T_PRUNE);
    const size_t NN = (size_t)N * N, nn0 = (size_t)n0 * n0;
    // layout: Ahat [N][N] | gamma copy [N][N] | A [n0][n0] | V [n0][n0] | W [n0] | lam [n0] | list [n0]
    const size_t o_ahat = 0, o_g = o_ahat + NN, o_a = o_g + NN, o_v = o_a + nn0, o_w = o_v + nn0, o_lam = o_w + n0,
                 o_end = o_lam + n0;
    MODAL_TRY(ensure(c->prune, sizeof(double) * o_end + sizeof(int) * (2 + (size_t)n0) + 256));
    double *base = c->prune.as<double>();
    double *Ahat = base + o_ahat, *A = base + o_a, *Vv = base + o_v, *W = base + o_w, *lam = base + o_lam;
    int *dlist = reinterpret_cast<int *>(base + o_end) + 2;
    const double *g = gamma ? base + o_g : c->gamma.as<double>();
    if (gamma) MODAL_CUDA(cudaMemcpyAsync(base + o_g, gamma, sizeof(double) * NN, cudaMemcpyHostToDevice, c->stream));
    k_prune_normalise<<<ceil_div((long)NN, 256), 256, 0, c->stream>>>(N, g, Ahat);
    MODAL_TRY(launched(c, "prune_normalise"));
    std::vector<double> hl(n0);
    int step = 0;
    for (int n = n0; n >= 2; n--, step++) {
        MODAL_CUDA(cudaMemcpyAsync(dlist, list.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
        if (n > 2) {
            k_prune_gather<<<ceil_div((long)n * n, 256), 256, 0, c->stream>>>(n, N, Ahat, dlist, A);
            MODAL_TRY(launched(c, "prune_gather"));
            int nv = 0, first = 0;
            MODAL_TRY(syev_dev(c, n, A, W, Vv, select_all, nullptr, &nv, &first));
        }
        k_prune_secular<<<ceil_div((long)n * 32, 256), 256, 0, c->stream>>>(n, N, Vv, W, Ahat, dlist, lam);
        MODAL_TRY(launched(c, "prune_secular"));
        MODAL_CUDA(cudaMemcpyAsync(hl.data(), lam, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
        MODAL_CUDA(cudaStreamSynchronize(c->stream));
        // first maximum (basis_optimisation_mpi.c:287-297)
        int index = 0;
        double best = hl[0];
        for (int i = 1; i < n; i++)
            if (hl[i] > best) { best = hl[i]; index = i; }
        order[step] = list[index];
        lambda_min[step] = best;
        list.erase(list.begin() + index);
    }
    order[step] = list[0];
    lambda_min[step] = 1.0;  // the reference prints 1 for the last mode (:326-343)
    return MODAL_OK;
}

modal_status modal_lambda_min(modal_ctx *c, double *lambda_min, double *eigvec, double *dlam_dq)
{
    if (!c || !lambda_min) { set_error("modal_lambda_min: NULL argument"); return MODAL_ERR_ARG; }
    if (!c->have_gamma) { set_error("modal_lambda_min: compute the FP64 Gamma first"); return MODAL_ERR_STATE; }
    MODAL_CUDA(cudaSetDevice(c->device));
    const int N = c->N;
    const size_t NN = (size_t)N * N;
    StageTimer t(c, MODAL_T_ADJOINT);
    // layout: A [N][N] | G [N][N] | V [N][N] | W [N] | dq [L][P]
    const size_t LP = (size_t)c->L * c->P;
    const size_t o_a = 0, o_gu = NN, o_v = 2 * NN, o_w = 3 * NN, o_dq = o_w + N, o_end = o_dq + LP;
    MODAL_TRY(ensure(c->prune, sizeof(double) * o_end + 64));
    double *base = c->prune.as<double>();
    double *A = base + o_a, *G = base + o_gu, *Vv = base + o_v, *W = base + o_w, *dq = base + o_dq;
    k_prune_normalise<<<ceil_div((long)NN, 256), 256, 0, c->stream>>>(N, c->gamma.as<double>(), A);
    MODAL_TRY(launched(c, "prune_normalise"));
    int nv = 0, first = 0;
    MODAL_TRY(syev_dev(c, N, A, W, Vv, select_all, nullptr, &nv, &first));
    double lam = 0.0;
    MODAL_CUDA(cudaMemcpyAsync(&lam, W, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    *lambda_min = lam;
    // eigenvector of the smallest eigenvalue: row 0 of the result
    if (eigvec) MODAL_CUDA(cudaMemcpyAsync(eigvec, Vv, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream));
    if (dlam_dq) {
        if (!c->have_glint) { set_error("modal_lambda_min: no quadrature state for the gradient"); return MODAL_ERR_STATE; }
        k_lmin_upstream<<<ceil_div((long)NN, 256), 256, 0, c->stream>>>(N, c->gamma.as<double>(), Vv, lam, G);
        MODAL_TRY(launched(c, "lmin_upstream"));
        MODAL_CUDA(cudaMemsetAsync(dq, 0, sizeof(double) * LP, c->stream));
        MODAL_TRY(gamma_vjp_accum_dev(c, G, dq));
        MODAL_CUDA(cudaMemcpyAsync(dlam_dq, dq, sizeof(double) * LP, cudaMemcpyDeviceToHost, c->stream));
    }
    t.stop();
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}

}  // extern "C"
