// ortho.cu -- FP64 orthogonalisation of Gamma and the alpha solve on the GPU.
//
// Cholesky branch of ortho_late_mpi.c:759-843:
//   norm_i = sqrt(gamma_ii), ghat = gamma_ij / (norm_i norm_j)
//   ghat = L L^T                      (blocked right-looking Cholesky, lower)
//   orthol[i][j]  = norm_i L_ij       (i >= j, 0 above)
//   lambdal[i][j] = (L^{-1})_ij / norm_j
// The reference builds lambdal from gsl_linalg_LU_invert of the upper factor
// L^T with the identity permutation and transposes it (:821-841); that is
// (L^{-1})^T transposed back, i.e. L^{-1}.  Here L^{-1} comes from a blocked
// forward substitution L X = I.
//
// A non-positive pivot (ghat not positive definite) is recorded as the
// smallest failing row in a device status word; the host then reports
// MODAL_ERR_NOT_PD or takes the PCA branch (eig.cu).
//
// Alpha solve (eigenmodetoday_mpi.c:148-162, 286-316):
//   alpha = lambdal^T (lambdal beta),  modesR = lambdainv^T alpha with
//   lambdainv the lower triangle of orthol (or the PCA lambdainv).
#include <algorithm>
#include <climits>
#include "common.cuh"

namespace modal {

// --------------------------------------------------------------------------
// FP64 tiled GEMM (64x64 tile, K step 16, 4x4 outputs per thread).
// --------------------------------------------------------------------------
constexpr int GT = 64, GK = 16;

template <bool TA, bool TB>
__global__ void __launch_bounds__(256) k_dgemm(int M, int N, int K, double alpha, const double *__restrict__ A, int lda,
                                               const double *__restrict__ B, int ldb, double beta, double *C, int ldc,
                                               int lower, long cstride)
{
    const int bm = blockIdx.y * GT, bn = blockIdx.x * GT;
    if (lower && bn > bm + GT - 1) return;
    // slice z of gridDim.z sums k in [kbeg, kend) into C + z * cstride
    const int kbeg = (int)((long)K * blockIdx.z / gridDim.z), kend = (int)((long)K * (blockIdx.z + 1) / gridDim.z);
    C += (size_t)blockIdx.z * cstride;
    __shared__ double As[GK][GT + 1];
    __shared__ double Bs[GK][GT + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0.0;

    for (int k0 = kbeg; k0 < kend; k0 += GK) {
#pragma unroll
        for (int t = 0; t < (GK * GT) / 256; t++) {
            int e = tid + 256 * t;
            int kk, mm;
            if (TA) { mm = e % GT; kk = e / GT; }
            else { kk = e % GK; mm = e / GK; }
            int m = bm + mm, k = k0 + kk;
            double v = 0.0;
            if (m < M && k < kend) v = TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
            As[kk][mm] = v;
        }
#pragma unroll
        for (int t = 0; t < (GK * GT) / 256; t++) {
            int e = tid + 256 * t;
            int kk, nn;
            if (TB) { kk = e % GK; nn = e / GK; }
            else { nn = e % GT; kk = e / GT; }
            int n = bn + nn, k = k0 + kk;
            double v = 0.0;
            if (n < N && k < kend) v = TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n];
            Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; kk++) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        int m = bm + ty + 16 * i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int n = bn + tx + 16 * j;
            if (n >= N || (lower && n > m)) continue;
            double *c = C + (size_t)m * ldc + n;
            *c = (beta == 0.0) ? alpha * acc[i][j] : fma(alpha, acc[i][j], beta * *c);
        }
    }
}

static modal_status dgemm_launch(modal_ctx *ctx, dim3 grid, int M, int N, int K, double alpha, const double *A, int lda,
                                 bool transA, const double *B, int ldb, bool transB, double beta, double *C, int ldc,
                                 int lower, long cstride)
{
    if (!transA && !transB) k_dgemm<false, false><<<grid, 256, 0, ctx->stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lower, cstride);
    else if (!transA && transB) k_dgemm<false, true><<<grid, 256, 0, ctx->stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lower, cstride);
    else if (transA && !transB) k_dgemm<true, false><<<grid, 256, 0, ctx->stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lower, cstride);
    else k_dgemm<true, true><<<grid, 256, 0, ctx->stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lower, cstride);
    return launched(ctx, "dgemm");
}

modal_status dgemm(modal_ctx *ctx, int M, int N, int K, double alpha, const double *A, int lda, bool transA,
                   const double *B, int ldb, bool transB, double beta, double *C, int ldc, int lower)
{
    if (M <= 0 || N <= 0) return MODAL_OK;
    dim3 grid(ceil_div(N, GT), ceil_div(M, GT));
    return dgemm_launch(ctx, grid, M, N, K, alpha, A, lda, transA, B, ldb, transB, beta, C, ldc, lower, 0);
}

// C (+)= op(A) op(B) with K split over KS slices of the tiled kernel, for products
// whose M x N tile grid is too small to fill the GPU but whose K is long (the
// primordial grid's point sums).  The KS partial products land in a buffer and
// are added in a fixed order.
__global__ void k_splitk_sum(int M, int N, int KS, const double *__restrict__ part, double *__restrict__ C, int ldc,
                             int lower, int accumulate)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)M * N) return;
    const int m = (int)(e / N), n = (int)(e - (size_t)m * N);
    if (lower && n > m) return;
    double v = accumulate ? C[(size_t)m * ldc + n] : 0.0;
    for (int p = 0; p < KS; p++) v += part[(size_t)p * M * N + e];
    C[(size_t)m * ldc + n] = v;
}

modal_status dgemm_splitk(modal_ctx *ctx, int M, int N, int K, const double *A, int lda, bool transA, const double *B,
                          int ldb, bool transB, double *C, int ldc, int lower, bool accumulate)
{
    if (M <= 0 || N <= 0 || K <= 0) return MODAL_OK;
    int nsm = 0;
    MODAL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
    long tiles = (long)ceil_div(M, GT) * ceil_div(N, GT);
    if (lower) tiles = (tiles + ceil_div(M, GT)) / 2;
    int KS = (int)std::min<long>(std::max<long>(1, ceil_div(2L * nsm, tiles)), std::max(1, K / 256));
    KS = std::min(KS, 64);
    if (KS == 1) return dgemm(ctx, M, N, K, 1.0, A, lda, transA, B, ldb, transB, accumulate ? 1.0 : 0.0, C, ldc, lower);
    MODAL_TRY(ensure(ctx->gemm_part, sizeof(double) * (size_t)KS * M * N));
    double *part = ctx->gemm_part.as<double>();
    MODAL_TRY(dgemm_launch(ctx, dim3(ceil_div(N, GT), ceil_div(M, GT), KS), M, N, K, 1.0, A, lda, transA, B, ldb, transB,
                           0.0, part, N, lower, (long)M * N));
    k_splitk_sum<<<ceil_div((long)M * N, 256), 256, 0, ctx->stream>>>(M, N, KS, part, C, ldc, lower, accumulate ? 1 : 0);
    return launched(ctx, "splitk_sum");
}

// --------------------------------------------------------------------------
// Skinny FP64 products C[S][N] = A[S][K] op(B) for S <= 16 rows (the alpha
// solve's S shapes against N x N matrices).  The large operand is read once,
// coalesced; K is split over KS CTAs per column block for enough parallelism
// and the partial sums are added in a fixed order (deterministic).
// --------------------------------------------------------------------------
constexpr int SK_S = 16, SK_KCH = 128, SK_KS = 8;

// B row-major [K][ldb]: grid (ceil(N / 64), KS); 256 threads = 64 columns x 4 k-lanes.
// R: rows held per thread (S <= R <= SK_S).
template <int R>
__global__ void __launch_bounds__(256) k_skinny_nn(int S, int N, int K, const double *__restrict__ A, int lda,
                                                   const double *__restrict__ B, int ldb, double *__restrict__ part)
{
    __shared__ double As[SK_KCH][R];
    __shared__ double red[3][R][64];
    const int col = threadIdx.x & 63, kl = threadIdx.x >> 6, n = blockIdx.x * 64 + col;
    const int k0 = (int)((long)K * blockIdx.y / gridDim.y), k1 = (int)((long)K * (blockIdx.y + 1) / gridDim.y);
    double acc[R];
#pragma unroll
    for (int s = 0; s < R; s++) acc[s] = 0.0;
    for (int kc = k0; kc < k1; kc += SK_KCH) {
        const int len = min(SK_KCH, k1 - kc);
        for (int e = threadIdx.x; e < SK_KCH * R; e += 256) {
            const int kk = e / R, s = e - kk * R;
            As[kk][s] = (kk < len && s < S) ? A[(size_t)s * lda + kc + kk] : 0.0;
        }
        __syncthreads();
        if (n < N)
            for (int kk = kl; kk < len; kk += 4) {
                const double b = B[(size_t)(kc + kk) * ldb + n];
#pragma unroll
                for (int s = 0; s < R; s++) acc[s] = fma(As[kk][s], b, acc[s]);
            }
        __syncthreads();
    }
    if (kl > 0)
#pragma unroll
        for (int s = 0; s < R; s++) red[kl - 1][s][col] = acc[s];
    __syncthreads();
    if (kl == 0 && n < N)
#pragma unroll
        for (int s = 0; s < R; s++)
            if (s < S) part[((size_t)blockIdx.y * S + s) * N + n] = ((acc[s] + red[0][s][col]) + red[1][s][col]) + red[2][s][col];
}

// B row-major [N][ldb] used transposed: grid (ceil(N / 16), KS); warp w takes rows
// n = 16 x + 2 w and 2 w + 1, lanes run over k.
template <int R>
__global__ void __launch_bounds__(256) k_skinny_nt(int S, int N, int K, const double *__restrict__ A, int lda,
                                                   const double *__restrict__ B, int ldb, double *__restrict__ part)
{
    __shared__ double As[R][SK_KCH];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * 16 + 2 * warp;
    const int k0 = (int)((long)K * blockIdx.y / gridDim.y), k1 = (int)((long)K * (blockIdx.y + 1) / gridDim.y);
    double acc[2][R];
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
        for (int s = 0; s < R; s++) acc[r][s] = 0.0;
    for (int kc = k0; kc < k1; kc += SK_KCH) {
        const int len = min(SK_KCH, k1 - kc);
        for (int e = threadIdx.x; e < SK_KCH * R; e += 256) {
            const int s = e / SK_KCH, kk = e - s * SK_KCH;
            As[s][kk] = (kk < len && s < S) ? A[(size_t)s * lda + kc + kk] : 0.0;
        }
        __syncthreads();
        for (int kk = lane; kk < len; kk += 32) {
            double b[2];
#pragma unroll
            for (int r = 0; r < 2; r++) b[r] = (n0 + r < N) ? B[(size_t)(n0 + r) * ldb + kc + kk] : 0.0;
#pragma unroll
            for (int s = 0; s < R; s++) {
                const double a = As[s][kk];
                acc[0][s] = fma(a, b[0], acc[0][s]);
                acc[1][s] = fma(a, b[1], acc[1][s]);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
        for (int s = 0; s < R; s++) {
            double v = acc[r][s];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            acc[r][s] = v;
        }
    if (lane == 0)
#pragma unroll
        for (int r = 0; r < 2; r++)
#pragma unroll
            for (int s = 0; s < R; s++)
                if (n0 + r < N && s < S) part[((size_t)blockIdx.y * S + s) * N + n0 + r] = acc[r][s];
}

__global__ void k_skinny_sum(int S, int N, int KS, const double *__restrict__ part, double *__restrict__ C, int ldc,
                             int accumulate)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)S * N) return;
    const int s = (int)(e / N), n = (int)(e - (size_t)s * N);
    double v = accumulate ? C[(size_t)s * ldc + n] : 0.0;
    for (int p = 0; p < KS; p++) v += part[(size_t)p * S * N + e];
    C[(size_t)s * ldc + n] = v;
}

// C (+)= A op(B) (alpha 1) with A [S][K]; S > 32 goes to the tiled kernel.
modal_status dgemm_rows(modal_ctx *ctx, int S, int N, int K, const double *A, int lda, const double *B, int ldb,
                        bool transB, double *C, int ldc, bool accumulate)
{
    // many rows: the FP64-accurate tensor-core product (8 slices), ~10x the FP64 rate at S = 512, N = 11480
    if (S > 2 * SK_S)
        return oz_gemm(ctx, S, N, K, 1.0, A, lda, false, B, ldb, transB, accumulate ? 1.0 : 0.0, C, ldc, 0, 8);
    if (S <= 0 || N <= 0) return MODAL_OK;
    MODAL_TRY(ensure(ctx->gemm_part, sizeof(double) * (size_t)SK_KS * SK_S * N));
    double *part = ctx->gemm_part.as<double>();
    for (int s0 = 0; s0 < S; s0 += SK_S) {
        const int Sc = std::min(SK_S, S - s0);
        const double *As = A + (size_t)s0 * lda;
        auto run = [&](auto nt, auto nn) {
            if (transB) nt<<<dim3(ceil_div(N, 16), SK_KS), 256, 0, ctx->stream>>>(Sc, N, K, As, lda, B, ldb, part);
            else nn<<<dim3(ceil_div(N, 64), SK_KS), 256, 0, ctx->stream>>>(Sc, N, K, As, lda, B, ldb, part);
        };
        if (Sc <= 2) run(k_skinny_nt<2>, k_skinny_nn<2>);
        else if (Sc <= 4) run(k_skinny_nt<4>, k_skinny_nn<4>);
        else if (Sc <= 8) run(k_skinny_nt<8>, k_skinny_nn<8>);
        else run(k_skinny_nt<SK_S>, k_skinny_nn<SK_S>);
        MODAL_TRY(launched(ctx, "skinny_gemm"));
        k_skinny_sum<<<ceil_div((long)Sc * N, 256), 256, 0, ctx->stream>>>(Sc, N, SK_KS, part, C + (size_t)s0 * ldc, ldc,
                                                                            accumulate ? 1 : 0);
        MODAL_TRY(launched(ctx, "skinny_sum"));
    }
    return MODAL_OK;
}

// --------------------------------------------------------------------------
// Normalisation (ortho_late_mpi.c:759-773).
// --------------------------------------------------------------------------
__global__ void k_norm(int N, const double *__restrict__ g, double *__restrict__ norm)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) norm[i] = sqrt(g[(size_t)i * N + i]);
}

__global__ void k_normalise(int N, const double *__restrict__ g, const double *__restrict__ norm, double *__restrict__ a)
{
    size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)N * N) return;
    int i = (int)(e / N), j = (int)(e % N);
    a[e] = g[e] / (norm[i] * norm[j]);
}

// --------------------------------------------------------------------------
// Cholesky of one nb x nb diagonal block in shared memory (right-looking).
// info[0] = smallest failing pivot row (INT_MAX when none).
// --------------------------------------------------------------------------
constexpr int NB = 64;
constexpr size_t TRI_SMEM = sizeof(double) * 2 * NB * (NB + 1);  // two 64 x 65 FP64 tiles

__global__ void __launch_bounds__(256) k_potrf_diag(double *A, int N, int kb, int nb, int *info)
{
    __shared__ double s[NB][NB + 1];
    __shared__ int bad;
    const int tid = threadIdx.x;
    if (tid == 0) bad = 0;
    for (int e = tid; e < nb * nb; e += 256) {
        int i = e / nb, j = e % nb;
        s[i][j] = A[(size_t)(kb + i) * N + kb + j];
    }
    __syncthreads();
    for (int j = 0; j < nb; j++) {
        if (tid == 0) {
            double d = s[j][j];
            if (!(d > 0.0)) {
                if (!bad) atomicMin(info, kb + j);
                bad = 1;
            }
            s[j][j] = sqrt(d);
        }
        __syncthreads();
        const double ljj = s[j][j];
        for (int i = j + 1 + tid; i < nb; i += 256) s[i][j] /= ljj;
        __syncthreads();
        const int m = nb - j - 1;  // trailing size
        for (int e = tid; e < m * m; e += 256) {
            int i = j + 1 + e / m, c = j + 1 + e % m;
            if (c <= i) s[i][c] -= s[i][j] * s[c][j];
        }
        __syncthreads();
    }
    for (int e = tid; e < nb * nb; e += 256) {
        int i = e / nb, j = e % nb;
        if (j <= i) A[(size_t)(kb + i) * N + kb + j] = s[i][j];
    }
}

// Panel below the diagonal block: row r of A21 := row r of A21 * L11^{-T}.
// One thread per row; 64 rows per CTA; rows staged in shared memory.
__global__ void __launch_bounds__(64) k_trsm_panel(double *A, int N, int kb, int nb)
{
    extern __shared__ double dsm[];
    double (*L11)[NB + 1] = reinterpret_cast<double (*)[NB + 1]>(dsm);
    double (*R)[NB + 1] = reinterpret_cast<double (*)[NB + 1]>(dsm + NB * (NB + 1));
    const int tid = threadIdx.x;
    const int r0 = kb + nb + blockIdx.x * 64;
    for (int e = tid; e < nb * nb; e += 64) {
        int i = e / nb, j = e % nb;
        L11[i][j] = A[(size_t)(kb + i) * N + kb + j];
    }
    for (int e = tid; e < 64 * nb; e += 64) {
        int rr = e / nb, c = e % nb;
        int r = r0 + rr;
        R[rr][c] = (r < N) ? A[(size_t)r * N + kb + c] : 0.0;
    }
    __syncthreads();
    if (r0 + tid < N) {
        for (int c = 0; c < nb; c++) {
            double s = R[tid][c];
            for (int t = 0; t < c; t++) s -= R[tid][t] * L11[c][t];
            R[tid][c] = s / L11[c][c];
        }
    }
    __syncthreads();
    for (int e = tid; e < 64 * nb; e += 64) {
        int rr = e / nb, c = e % nb;
        int r = r0 + rr;
        if (r < N) A[(size_t)r * N + kb + c] = R[rr][c];
    }
}

// --------------------------------------------------------------------------
// X = L^{-1} by blocked forward substitution on L X = I.
// Step for row block r: X[rb:rb+nb, 0:rb+nb] = L_rr^{-1} B[rb:rb+nb, 0:rb+nb]
// (one thread per column), then B[rb+nb:, 0:rb+nb] -= L[rb+nb:, rb:rb+nb] X[rb:rb+nb, 0:rb+nb].
// --------------------------------------------------------------------------
__global__ void k_eye(int N, double *X)
{
    size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)N * N) return;
    X[e] = ((e / N) == (e % N)) ? 1.0 : 0.0;
}

__global__ void __launch_bounds__(64) k_trsv_diag(const double *L, double *X, int N, int rb, int nb, int ncols)
{
    extern __shared__ double dsm[];
    double (*Ld)[NB + 1] = reinterpret_cast<double (*)[NB + 1]>(dsm);
    double (*Xs)[64 + 1] = reinterpret_cast<double (*)[64 + 1]>(dsm + NB * (NB + 1));
    const int tid = threadIdx.x;
    const int c0 = blockIdx.x * 64;
    for (int e = tid; e < nb * nb; e += 64) {
        int i = e / nb, j = e % nb;
        Ld[i][j] = L[(size_t)(rb + i) * N + rb + j];
    }
    for (int e = tid; e < nb * 64; e += 64) {
        int i = e / 64, cc = e % 64;
        int c = c0 + cc;
        Xs[i][cc] = (c < ncols) ? X[(size_t)(rb + i) * N + c] : 0.0;
    }
    __syncthreads();
    if (c0 + tid < ncols) {
        for (int i = 0; i < nb; i++) {
            double s = Xs[i][tid];
            for (int t = 0; t < i; t++) s -= Ld[i][t] * Xs[t][tid];
            Xs[i][tid] = s / Ld[i][i];
        }
    }
    __syncthreads();
    for (int e = tid; e < nb * 64; e += 64) {
        int i = e / 64, cc = e % 64;
        int c = c0 + cc;
        if (c < ncols) X[(size_t)(rb + i) * N + c] = Xs[i][cc];
    }
}

// orthol = D^{1/2} L (lower), lambdal = X D^{-1/2} (lower).
__global__ void k_chol_outputs(int N, const double *__restrict__ Lm, const double *__restrict__ X,
                               const double *__restrict__ norm, double *__restrict__ orthol, double *__restrict__ lambdal)
{
    size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)N * N) return;
    int i = (int)(e / N), j = (int)(e % N);
    orthol[e] = (i >= j) ? norm[i] * Lm[e] : 0e0;
    lambdal[e] = (i >= j) ? X[e] / norm[j] : 0.0;
}

modal_status eig_pca_dev(modal_ctx *ctx);  // eig.cu

modal_status cholesky_dev(modal_ctx *ctx, int *fail_row)
{
    const int N = ctx->N;
    double *A = ctx->chol.as<double>();
    int *info = ctx->info.as<int>();
    const int big = INT_MAX;
    MODAL_CUDA(cudaFuncSetAttribute(k_trsm_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TRI_SMEM));
    MODAL_CUDA(cudaMemcpyAsync(info, &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    int h = INT_MAX;
    for (int kb = 0; kb < N; kb += NB) {
        int nb = (N - kb < NB) ? (N - kb) : NB;
        k_potrf_diag<<<1, 256, 0, ctx->stream>>>(A, N, kb, nb, info);
        MODAL_TRY(launched(ctx, "potrf_diag"));
        // every 4 panels: stop early once a pivot has failed (the PCA branch follows)
        if ((kb / NB) % 4 == 3) {
            MODAL_CUDA(cudaMemcpyAsync(&h, info, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            MODAL_CUDA(cudaStreamSynchronize(ctx->stream));
            if (h != INT_MAX) break;
        }
        int rest = N - kb - nb;
        if (rest > 0) {
            k_trsm_panel<<<ceil_div(rest, 64), 64, TRI_SMEM, ctx->stream>>>(A, N, kb, nb);
            MODAL_TRY(launched(ctx, "trsm_panel"));
            double *A21 = A + (size_t)(kb + nb) * N + kb;
            double *A22 = A + (size_t)(kb + nb) * N + kb + nb;
            // large trailing blocks on the tensor cores (FP64-accurate slices): the
            // FP64 tiled kernel runs at the FP64 rate, about 1.2 ms per update at 4900 rows
            if (rest >= 1024) MODAL_TRY(oz_gemm(ctx, rest, rest, nb, -1.0, A21, N, false, A21, N, true, 1.0, A22, N, 1, 8));
            else MODAL_TRY(dgemm(ctx, rest, rest, nb, -1.0, A21, N, false, A21, N, true, 1.0, A22, N, 1));
        }
    }
    MODAL_CUDA(cudaMemcpyAsync(&h, info, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MODAL_CUDA(cudaStreamSynchronize(ctx->stream));
    *fail_row = (h == INT_MAX) ? -1 : h;
    return MODAL_OK;
}

modal_status trtri_dev(modal_ctx *ctx)
{
    const int N = ctx->N;
    const double *Lm = ctx->chol.as<double>();
    double *X = ctx->linv.as<double>();
    size_t NN = (size_t)N * N;
    MODAL_CUDA(cudaFuncSetAttribute(k_trsv_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TRI_SMEM));
    k_eye<<<ceil_div((long)NN, 256), 256, 0, ctx->stream>>>(N, X);
    MODAL_TRY(launched(ctx, "eye"));
    for (int rb = 0; rb < N; rb += NB) {
        int nb = (N - rb < NB) ? (N - rb) : NB;
        int ncols = rb + nb;
        k_trsv_diag<<<ceil_div(ncols, 64), 64, TRI_SMEM, ctx->stream>>>(Lm, X, N, rb, nb, ncols);
        MODAL_TRY(launched(ctx, "trsv_diag"));
        int rest = N - rb - nb;
        if (rest > 0)
            MODAL_TRY(dgemm(ctx, rest, ncols, nb, -1.0, Lm + (size_t)(rb + nb) * N + rb, N, false,
                            X + (size_t)rb * N, N, false, 1.0, X + (size_t)(rb + nb) * N, N, 0));
    }
    return MODAL_OK;
}

modal_status ortho_dev(modal_ctx *ctx, int pca_flag)
{
    const int N = ctx->N;
    size_t NN = (size_t)N * N;
    MODAL_TRY(ensure(ctx->norm, sizeof(double) * N));
    MODAL_TRY(ensure(ctx->chol, sizeof(double) * NN));
    MODAL_TRY(ensure(ctx->orthol, sizeof(double) * NN));
    MODAL_TRY(ensure(ctx->lambdal, sizeof(double) * NN));
    MODAL_TRY(ensure(ctx->info, 4 * sizeof(int)));
    k_norm<<<ceil_div(N, 256), 256, 0, ctx->stream>>>(N, ctx->gamma.as<double>(), ctx->norm.as<double>());
    MODAL_TRY(launched(ctx, "norm"));
    k_normalise<<<ceil_div((long)NN, 256), 256, 0, ctx->stream>>>(N, ctx->gamma.as<double>(), ctx->norm.as<double>(),
                                                                     ctx->chol.as<double>());
    MODAL_TRY(launched(ctx, "normalise"));
    ctx->have_ortho = false;
    if (pca_flag != 0) {
        int fail = -1;
        MODAL_TRY(cholesky_dev(ctx, &fail));
        if (fail < 0) {
            MODAL_TRY(ensure(ctx->linv, sizeof(double) * NN));
            MODAL_TRY(trtri_dev(ctx));
            k_chol_outputs<<<ceil_div((long)NN, 256), 256, 0, ctx->stream>>>(
                N, ctx->chol.as<double>(), ctx->linv.as<double>(), ctx->norm.as<double>(), ctx->orthol.as<double>(),
                ctx->lambdal.as<double>());
            MODAL_TRY(launched(ctx, "chol_outputs"));
            ctx->ortho_branch = 0;
            ctx->ortho_rank = N;
            ctx->have_ortho = true;
            return MODAL_OK;
        }
        // not positive definite: re-normalise (the factorisation overwrote it) and take the PCA branch
        k_normalise<<<ceil_div((long)NN, 256), 256, 0, ctx->stream>>>(N, ctx->gamma.as<double>(),
                                                                         ctx->norm.as<double>(), ctx->chol.as<double>());
        MODAL_TRY(launched(ctx, "normalise"));
        ctx->ortho_rank = fail;  // first failing pivot, reported if PCA is unavailable
    }
    MODAL_TRY(eig_pca_dev(ctx));
    ctx->ortho_branch = 1;
    ctx->have_ortho = true;
    return MODAL_OK;
}

// --------------------------------------------------------------------------
// Alpha solve for S shapes: y = beta lambdal^T, alpha = y lambdal,
// modesR = alpha lambdainv, where lambdainv is the lower triangle of orthol
// (eigenmodetoday_mpi.c:148-160, 303-316): orthol itself on the Cholesky
// branch, the copy in linv otherwise (k_pca_outputs, or lambdainv_dev for an
// orthogonalisation loaded by modal_set_ortho).
// --------------------------------------------------------------------------
__global__ void k_lower_triangle(int N, const double *__restrict__ a, double *__restrict__ t)
{
    size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)N * N) return;
    int i = (int)(e / N), j = (int)(e % N);
    t[e] = (i >= j) ? a[e] : 0.0;
}

modal_status lambdainv_dev(modal_ctx *ctx)
{
    const size_t NN = (size_t)ctx->N * ctx->N;
    MODAL_TRY(ensure(ctx->linv, sizeof(double) * NN));
    k_lower_triangle<<<ceil_div((long)NN, 256), 256, 0, ctx->stream>>>(ctx->N, ctx->orthol.as<double>(),
                                                                        ctx->linv.as<double>());
    return launched(ctx, "lower_triangle");
}

modal_status alpha_dev(modal_ctx *ctx, int S)
{
    const int N = ctx->N;
    MODAL_TRY(ensure(ctx->alpha, sizeof(double) * (size_t)S * N));
    MODAL_TRY(ensure(ctx->modesr, sizeof(double) * (size_t)S * N));
    MODAL_TRY(ensure(ctx->scratch2, sizeof(double) * (size_t)S * N));
    double *y = ctx->scratch2.as<double>();
    const double *lam = ctx->lambdal.as<double>();
    MODAL_TRY(dgemm_rows(ctx, S, N, N, ctx->beta.as<double>(), N, lam, N, true, y, N, false));
    MODAL_TRY(dgemm_rows(ctx, S, N, N, y, N, lam, N, false, ctx->alpha.as<double>(), N, false));
    const double *lambdainv = ctx->ortho_branch == 0 ? ctx->orthol.as<double>() : ctx->linv.as<double>();
    MODAL_TRY(dgemm_rows(ctx, S, N, N, ctx->alpha.as<double>(), N, lambdainv, N, false, ctx->modesr.as<double>(), N,
                         false));
    return MODAL_OK;
}

}  // namespace modal
