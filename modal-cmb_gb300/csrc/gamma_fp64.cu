// gamma_fp64.cu -- plain FP64 form of the two contractions that build Gamma.
//
//  l-contraction (calculate_orthoMij_T, orthogonalisation_late.c:99-129):
//     M[i][j][k] = sum_{l=lmin}^{lmax} gl_Pl[k][l] q_i(l) q_j(l)
//  mu-contraction (calculate_orthol, orthogonalisation_late.c:239-336):
//     Gamma_mn = sum_k w_k/(48 pi) * sum of the six products
//                M[m_a][n_s(a)][k] over the permutations s of (0,1,2),
//  i.e. w_k/(48 pi) times the permanent of the 3x3 block of M(k) with rows
//  (m1,m2,m3) and columns (n1,n2,n3).  Device layouts: pl[l][k] (l-major),
//  mt[k][i][j] (mu-major, so one mu step of the whole P x P table is one
//  contiguous block).
#include "common.cuh"

namespace modal {

// --------------------------------------------------------------------------
// l-contraction, FP64 SIMT GEMM over l: out tile 64 (mu) x 32 (p<=q pairs).
// Summation over l in ascending order, as the reference.
// --------------------------------------------------------------------------
constexpr int MIJ_BK = 64, MIJ_BU = 32, MIJ_LC = 16;

__global__ void __launch_bounds__(256) k_mij_fp64(int nmu, int lmin, int lmax, int P, int npair,
                                                  const double *__restrict__ pl, const double *__restrict__ q,
                                                  const int2 *__restrict__ pairs, double *__restrict__ mt)
{
    __shared__ double sPl[MIJ_LC][MIJ_BK];
    __shared__ double sV[MIJ_LC][MIJ_BU];
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int k0 = blockIdx.x * MIJ_BK, u0 = blockIdx.y * MIJ_BU;
    const int L = lmax - lmin + 1;
    double acc[8];
#pragma unroll
    for (int r = 0; r < 8; r++) acc[r] = 0.0;

    for (int l0 = 0; l0 < L; l0 += MIJ_LC) {
#pragma unroll
        for (int t = 0; t < (MIJ_LC * MIJ_BK) / 256; t++) {
            int e = tid + 256 * t, lr = e / MIJ_BK, kc = e % MIJ_BK;
            int l = l0 + lr, k = k0 + kc;
            sPl[lr][kc] = (l < L && k < nmu) ? pl[(size_t)(lmin + l) * nmu + k] : 0.0;
        }
#pragma unroll
        for (int t = 0; t < (MIJ_LC * MIJ_BU) / 256; t++) {
            int e = tid + 256 * t, lr = e / MIJ_BU, uc = e % MIJ_BU;
            int l = l0 + lr, u = u0 + uc;
            double v = 0.0;
            if (l < L && u < npair) {
                int2 pq = pairs[u];
                v = q[(size_t)l * P + pq.x] * q[(size_t)l * P + pq.y];
            }
            sV[lr][uc] = v;
        }
        __syncthreads();
#pragma unroll
        for (int lr = 0; lr < MIJ_LC; lr++) {
            double vv = sV[lr][tx];
#pragma unroll
            for (int r = 0; r < 8; r++) acc[r] = fma(sPl[lr][ty + 8 * r], vv, acc[r]);
        }
        __syncthreads();
    }
    const int u = u0 + tx;
    if (u >= npair) return;
    const int2 pq = pairs[u];
#pragma unroll
    for (int r = 0; r < 8; r++) {
        int k = k0 + ty + 8 * r;
        if (k < nmu) {
            double *blk = mt + (size_t)k * P * P;
            blk[pq.x * P + pq.y] = acc[r];
            blk[pq.y * P + pq.x] = acc[r];
        }
    }
}

// M table [nmu][P][P] of a basis q[L][P] on lmin..lmax (T or E) into out.
modal_status mij_table_dev(modal_ctx *ctx, const double *q, int lmin, int lmax, int P, DevBuf &out)
{
    const int npair = P * (P + 1) / 2;
    MODAL_TRY(ensure(out, sizeof(double) * (size_t)ctx->nmu * P * P));
    MODAL_TRY(ensure(ctx->scratch, sizeof(int2) * npair));
    int2 *h = new int2[npair];
    int u = 0;
    for (int p = 0; p < P; p++)
        for (int qq = p; qq < P; qq++) h[u++] = make_int2(p, qq);
    cudaError_t e = cudaMemcpyAsync(ctx->scratch.ptr, h, sizeof(int2) * npair, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    delete[] h;
    if (e != cudaSuccess) { set_error("mij pairs: %s", cudaGetErrorString(e)); return MODAL_ERR_CUDA; }
    dim3 grid(ceil_div(ctx->nmu, MIJ_BK), ceil_div(npair, MIJ_BU));
    k_mij_fp64<<<grid, 256, 0, ctx->stream>>>(ctx->nmu, lmin, lmax, P, npair, ctx->pl.as<double>(), q,
                                              ctx->scratch.as<int2>(), out.as<double>());
    return launched(ctx, "mij_fp64");
}

modal_status mij_dev(modal_ctx *ctx)
{
    return mij_table_dev(ctx, ctx->q.as<double>(), ctx->lmin, ctx->lmax, ctx->P, ctx->mt);
}

modal_status mt_ready(modal_ctx *ctx)
{
    if (ctx->have_mt) return MODAL_OK;
    StageTimer t(ctx, MODAL_T_MIJ);
    MODAL_TRY(mij_dev(ctx));
    ctx->have_mt = true;
    return MODAL_OK;
}

// --------------------------------------------------------------------------
// mu-contraction, FP64.  One CTA per 32x32 tile of (m,n) with tile(m) <= tile(n);
// thread (tx,ty) owns n = n0+tx and m = m0+ty+8r, r < 4.  A chunk of KC mu
// steps of the whole P x P table is staged in shared memory; per (pair, mu):
// 9 shared loads, the permanent in 9 FP64 ops and one FMA with the weight.
// Summation over mu in ascending order.
// --------------------------------------------------------------------------
__global__ void k_wgt48(int nmu, const double *w, double *wg)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nmu) wg[k] = w[k] / (48e0 * 3.14159265358979323846);
}

__global__ void __launch_bounds__(256) k_gamma_fp64(int N, int P, int nmu, int KC, const int *__restrict__ triples,
                                                    const double *__restrict__ mt, const double *__restrict__ wg,
                                                    double *__restrict__ gamma)
{
    const int tm = blockIdx.y, tn = blockIdx.x;
    if (tm > tn) return;
    extern __shared__ double smem[];
    double *sW = smem;       // [KC]
    double *sA = smem + KC;  // [KC][P*P]
    const int PP = P * P;
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int n = tn * 32 + tx;
    int nb0 = 0, nb1 = 0, nb2 = 0;
    if (n < N) { nb0 = triples[3 * n]; nb1 = triples[3 * n + 1]; nb2 = triples[3 * n + 2]; }
    int mo[4][3];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        int m = tm * 32 + ty + 8 * r;
        if (m < N) { mo[r][0] = triples[3 * m] * P; mo[r][1] = triples[3 * m + 1] * P; mo[r][2] = triples[3 * m + 2] * P; }
        else { mo[r][0] = mo[r][1] = mo[r][2] = 0; }
    }
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k0 = 0; k0 < nmu; k0 += KC) {
        const int kc = min(KC, nmu - k0);
        const double *src = mt + (size_t)k0 * PP;
        for (int e = tid; e < kc * PP; e += 256) sA[e] = src[e];
        if (tid < kc) sW[tid] = wg[k0 + tid];
        __syncthreads();
        for (int kk = 0; kk < kc; kk++) {
            const double *A = sA + kk * PP;
            const double wk = sW[kk];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const double *r1 = A + mo[r][0], *r2 = A + mo[r][1], *r3 = A + mo[r][2];
                double a11 = r1[nb0], a12 = r1[nb1], a13 = r1[nb2];
                double a21 = r2[nb0], a22 = r2[nb1], a23 = r2[nb2];
                double a31 = r3[nb0], a32 = r3[nb1], a33 = r3[nb2];
                double t1 = fma(a23, a32, a22 * a33);
                double t2 = fma(a23, a31, a21 * a33);
                double t3 = fma(a22, a31, a21 * a32);
                double pm = fma(a13, t3, fma(a12, t2, a11 * t1));
                acc[r] = fma(wk, pm, acc[r]);
            }
        }
        __syncthreads();
    }
    if (n >= N) return;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        int m = tm * 32 + ty + 8 * r;
        if (m < N && m <= n) {
            gamma[(size_t)m * N + n] = acc[r];
            gamma[(size_t)n * N + m] = acc[r];
        }
    }
}

modal_status gamma_fp64_dev(modal_ctx *ctx, int mu0, int nmu)
{
    const int N = ctx->N, P = ctx->P;
    MODAL_TRY(mt_ready(ctx));
    MODAL_TRY(ensure(ctx->gamma, sizeof(double) * (size_t)N * N));
    MODAL_TRY(ensure(ctx->scratch2, sizeof(double) * nmu));
    k_wgt48<<<ceil_div(nmu, 256), 256, 0, ctx->stream>>>(nmu, ctx->w.as<double>() + mu0, ctx->scratch2.as<double>());
    MODAL_TRY(launched(ctx, "wgt48"));
    int KC = (96 * 1024) / (P * P * 8);
    if (KC < 1) KC = 1;
    if (KC > 32) KC = 32;
    if (ctx->gamma_kc > 0 && sizeof(double) * ((size_t)ctx->gamma_kc * (1 + (size_t)P * P)) <= 200 * 1024)
        KC = ctx->gamma_kc;  // tuned (modal_autotune)
    size_t smem = sizeof(double) * ((size_t)KC + (size_t)KC * P * P);
    if (smem > 200 * 1024) { set_error("gamma_fp64: P=%d too large for the shared-memory tile", P); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaFuncSetAttribute(k_gamma_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int nt = ceil_div(N, 32);
    dim3 grid(nt, nt);
    k_gamma_fp64<<<grid, 256, smem, ctx->stream>>>(N, P, nmu, KC, ctx->triples.as<int>(),
                                                   ctx->mt.as<double>() + (size_t)mu0 * P * P,
                                                   ctx->scratch2.as<double>(), ctx->gamma.as<double>());
    return launched(ctx, "gamma_fp64");
}

}  // namespace modal
