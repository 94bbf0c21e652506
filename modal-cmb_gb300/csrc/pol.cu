// pol.cu -- polarised Gamma: results[1..3] of calculate_orthol with
// do_polarisation (orthogonalisation_late.c:239-336), FP64.
//
// With an E basis q_E[L_E][P_E] on lmin_E..lmax_E the l-contraction gives a
// second table M_E (calculate_orthoMij_E, :131-157) on the same quadrature,
// whose n_mu and P_l table then cover max(lmax_T, lmax_E) (:33-37).  Mode
// triples follow find_perm_late_XXX: TTE (T,T,E), TEE (T,E,E), EEE (E,E,E).
//   TTE_mn = sum_k w_k/(16 pi) (MT[a0][b0] MT[a1][b1] + MT[a1][b0] MT[a0][b1]) ME[a2][b2]
//   TEE_mn = sum_k w_k/(16 pi) MT[a0][b0] (ME[a1][b1] ME[a2][b2] + ME[a2][b1] ME[a1][b2])
//   EEE_mn = sum_k w_k/(48 pi) perm3(ME[a_x][b_y])
// Each is symmetric in (m, n): the kernel computes the tiles with
// tile(m) <= tile(n) and mirrors, as k_gamma_fp64 does for TTT.
#include <algorithm>
#include <vector>
#include "common.cuh"

namespace modal {

namespace {

constexpr double kPi = 3.14159265358979323846;

// FORM 1: TTE, 2: TEE, 3: EEE.  One CTA per 32x32 tile; KC mu steps of both
// tables staged in shared memory per pass.
template <int FORM>
__global__ void __launch_bounds__(256) k_gamma_pol(int N, int PT, int PE, int nmu, int KC,
                                                   const int *__restrict__ tri, const double *__restrict__ mtT,
                                                   const double *__restrict__ mtE, const double *__restrict__ w,
                                                   double *__restrict__ gamma)
{
    const int tm = blockIdx.y, tn = blockIdx.x;
    if (tm > tn) return;
    extern __shared__ double smem[];
    const int PTT = (FORM == 3) ? 0 : PT * PT, PEE = PE * PE;
    double *sW = smem;              // [KC]
    double *sT = smem + KC;         // [KC][PT*PT]
    double *sE = sT + KC * PTT;     // [KC][PE*PE]
    // stride of each leg's table: legs in T use PT, legs in E use PE
    constexpr bool t0 = (FORM != 3), t1 = (FORM == 1);
    const int s0 = t0 ? PT : PE, s1 = t1 ? PT : PE;
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int n = tn * 32 + tx;
    int b0 = 0, b1 = 0, b2 = 0;
    if (n < N) { b0 = tri[3 * n]; b1 = tri[3 * n + 1]; b2 = tri[3 * n + 2]; }
    int ao[4][3];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const int m = tm * 32 + ty + 8 * r;
        if (m < N) { ao[r][0] = tri[3 * m] * s0; ao[r][1] = tri[3 * m + 1] * s1; ao[r][2] = tri[3 * m + 2] * PE; }
        else { ao[r][0] = ao[r][1] = ao[r][2] = 0; }
    }
    const double wscale = (FORM == 3) ? 1.0 / (48.0 * kPi) : 1.0 / (16.0 * kPi);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k0 = 0; k0 < nmu; k0 += KC) {
        const int kc = min(KC, nmu - k0);
        if (FORM != 3)
            for (int e = tid; e < kc * PTT; e += 256) sT[e] = mtT[(size_t)k0 * PTT + e];
        for (int e = tid; e < kc * PEE; e += 256) sE[e] = mtE[(size_t)k0 * PEE + e];
        if (tid < kc) sW[tid] = w[k0 + tid] * wscale;
        __syncthreads();
        for (int kk = 0; kk < kc; kk++) {
            const double *T = sT + kk * PTT, *E = sE + kk * PEE;
            const double wk = sW[kk];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                double v;
                if (FORM == 1) {
                    const double *r0 = T + ao[r][0], *r1 = T + ao[r][1];
                    v = fma(r0[b0], r1[b1], r1[b0] * r0[b1]) * E[ao[r][2] + b2];
                } else if (FORM == 2) {
                    const double *e1 = E + ao[r][1], *e2 = E + ao[r][2];
                    v = T[ao[r][0] + b0] * fma(e1[b1], e2[b2], e2[b1] * e1[b2]);
                } else {
                    const double *r1 = E + ao[r][0], *r2 = E + ao[r][1], *r3 = E + ao[r][2];
                    const double a11 = r1[b0], a12 = r1[b1], a13 = r1[b2];
                    const double a21 = r2[b0], a22 = r2[b1], a23 = r2[b2];
                    const double a31 = r3[b0], a32 = r3[b1], a33 = r3[b2];
                    v = fma(a13, fma(a22, a31, a21 * a32), fma(a12, fma(a23, a31, a21 * a33), a11 * fma(a23, a32, a22 * a33)));
                }
                acc[r] = fma(wk, v, acc[r]);
            }
        }
        __syncthreads();
    }
    if (n >= N) return;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const int m = tm * 32 + ty + 8 * r;
        if (m < N && m <= n) {
            gamma[(size_t)m * N + n] = acc[r];
            gamma[(size_t)n * N + m] = acc[r];
        }
    }
}

}  // namespace

}  // namespace modal

using namespace modal;

extern "C" {

modal_status modal_set_basis_e(modal_ctx *c, int lmin_e, int lmax_e, int P_e, const double *qe)
{
    if (!c || lmin_e < 0 || lmax_e < lmin_e || P_e < 1 || P_e > 64 || !qe) {
        set_error("modal_set_basis_e: lmin=%d lmax=%d P=%d (1 <= P <= 64)", lmin_e, lmax_e, P_e);
        return MODAL_ERR_ARG;
    }
    MODAL_CUDA(cudaSetDevice(c->device));
    const int L_e = lmax_e - lmin_e + 1;
    MODAL_TRY(ensure(c->qe, sizeof(double) * (size_t)L_e * P_e));
    MODAL_CUDA(cudaMemcpyAsync(c->qe.ptr, qe, sizeof(double) * (size_t)L_e * P_e, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    c->lmin_e = lmin_e;
    c->lmax_e = lmax_e;
    c->L_e = L_e;
    c->P_e = P_e;
    c->have_basis_e = true;
    // the quadrature and every table now cover max(lmax_T, lmax_E)
    c->have_glint = c->have_gamma = c->have_ortho = c->have_beta = false;
    c->have_pol = c->have_gamma_pol = false;
    return MODAL_OK;
}

modal_status modal_set_modes_pol(modal_ctx *c, const int *tte, const int *tee, const int *eee)
{
    if (!c || !tte || !tee || !eee) { set_error("modal_set_modes_pol: NULL argument"); return MODAL_ERR_ARG; }
    if (!c->have_modes || !c->have_basis_e) {
        set_error("modal_set_modes_pol: set the T basis and modes and the E basis first");
        return MODAL_ERR_STATE;
    }
    const int N = c->N, PT = c->P, PE = c->P_e;
    const int *lists[3] = {tte, tee, eee};
    // legs in T: TTE 0,1; TEE 0; EEE none
    const int nT[3] = {2, 1, 0};
    for (int f = 0; f < 3; f++)
        for (long e = 0; e < 3L * N; e++) {
            const int v = lists[f][e], lim = (e % 3) < nT[f] ? PT : PE;
            if (v < 0 || v >= lim) {
                set_error("modal_set_modes_pol: %s mode %ld leg %ld index %d outside [0,%d)",
                          f == 0 ? "TTE" : (f == 1 ? "TEE" : "EEE"), e / 3, e % 3, v, lim);
                return MODAL_ERR_ARG;
            }
        }
    MODAL_CUDA(cudaSetDevice(c->device));
    MODAL_TRY(ensure(c->tri_pol, sizeof(int) * 9 * (size_t)N));
    for (int f = 0; f < 3; f++)
        MODAL_CUDA(cudaMemcpyAsync(c->tri_pol.as<int>() + 3 * (size_t)N * f, lists[f], sizeof(int) * 3 * (size_t)N,
                                   cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    c->have_pol = true;
    c->have_gamma_pol = false;
    return MODAL_OK;
}

modal_status modal_gamma_pol(modal_ctx *c, double *gamma_tte, double *gamma_tee, double *gamma_eee)
{
    if (!c) { set_error("modal_gamma_pol: ctx is NULL"); return MODAL_ERR_ARG; }
    if (!c->have_pol) { set_error("modal_gamma_pol: set the polarised modes first"); return MODAL_ERR_STATE; }
    MODAL_CUDA(cudaSetDevice(c->device));
    if (!c->have_glint) MODAL_TRY(modal_init_glint(c));
    MODAL_TRY(mt_ready(c));
    const int N = c->N, PT = c->P, PE = c->P_e, nmu = c->nmu;
    const size_t NN = (size_t)N * N;
    MODAL_TRY(ensure(c->gamma_pol, sizeof(double) * 3 * NN));
    const size_t per_mu = (size_t)PT * PT + (size_t)PE * PE;
    int KC = (int)std::max<size_t>(1, std::min<size_t>(32, (96 * 1024) / (per_mu * 8 + 8)));
    const size_t smem = sizeof(double) * ((size_t)KC + (size_t)KC * per_mu);
    if (smem > 200 * 1024) { set_error("modal_gamma_pol: P_T=%d, P_E=%d too large for the tile", PT, PE); return MODAL_ERR_ARG; }
    const int nt = ceil_div(N, 32);
    const dim3 grid(nt, nt);
    {
        StageTimer t(c, MODAL_T_GAMMA);
        auto run = [&](auto kern, int f) -> modal_status {
            MODAL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            kern<<<grid, 256, smem, c->stream>>>(N, PT, PE, nmu, KC, c->tri_pol.as<int>() + 3 * (size_t)N * f,
                                                 c->mt.as<double>(), c->me.as<double>(), c->w.as<double>(),
                                                 c->gamma_pol.as<double>() + f * NN);
            return launched(c, "gamma_pol");
        };
        MODAL_TRY(run(k_gamma_pol<1>, 0));
        MODAL_TRY(run(k_gamma_pol<2>, 1));
        MODAL_TRY(run(k_gamma_pol<3>, 2));
    }
    double *outs[3] = {gamma_tte, gamma_tee, gamma_eee};
    for (int f = 0; f < 3; f++)
        if (outs[f])
            MODAL_CUDA(cudaMemcpyAsync(outs[f], c->gamma_pol.as<double>() + f * NN, sizeof(double) * NN,
                                       cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    c->have_gamma_pol = true;
    return MODAL_OK;
}

}  // extern "C"
