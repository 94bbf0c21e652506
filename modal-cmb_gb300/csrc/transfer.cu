// transfer.cu -- late x primordial transfer Gamma, FP64 on the GPU.
//
// Default path of gamma_mpi.c (calculate_gamma.c):
//   TTweight_l = (2l+1)^{5/6} b_l / sqrt(b_l^2 C_l + N_l)                     (:76-88)
//   M[p][q][x][k] = sum_l P_l(mu_k) TTweight_l q~_p(l,x) q_q(l)                (:254-303)
//   g(m,n,x)      = sum_k w_k perm3(M[p_a][q_b][x][k]), (p) = prim triple of n,
//                   (q) = late triple of m                                       (:512-555)
//   y_x = x^2 g(m,n,x), set to 0 at the first 10 grid points when |y| > 1e-18
//   Gamma_t[m][n] = integrate_cubic_spline(x, y) dphi^2 / (8 pi)                 (:773-934)
// The spline integral is linear in y for fixed nodes: I(y) = sum_x c_x y_x with
// c_x the integral of the spline through the unit vector e_x, computed once on
// the host with the reference's own spline recurrences.  The kernel folds the
// x loop and that weighted sum into one pass per (m, n) tile.
// Device layouts: qt[x][p][l] (l = 0..lmax), mt2[x][k][p][q] (mu-major per x).
#include <algorithm>
#include <cmath>
#include <vector>
#include "common.cuh"

namespace modal {

// Integral over [x0, x_{n-1}] of the cubic spline of integrate_cubic_spline
// (calculate_gamma.c:845-934) through (x, y).
static double spline_integral(const double *x, const double *y, int n)
{
    if (n < 2) return 0.0;
    std::vector<double> a(n, 0.0), b(n, 0.0), c(n, 0.0);
    c[0] = x[1] - x[0];
    b[1] = (y[1] - y[0]) / c[0];
    for (int i = 1; i < n - 1; i++) {
        c[i] = x[i + 1] - x[i];
        a[i] = 2.0 * (c[i - 1] + c[i]);
        b[i + 1] = (y[i + 1] - y[i]) / c[i];
        b[i] = b[i + 1] - b[i];
    }
    a[0] = -c[0];
    a[n - 1] = -c[n - 2];
    b[0] = 0.0;
    b[n - 1] = 0.0;
    if (n > 2) {
        b[0] = b[2] / (x[3] - x[1]) - b[1] / (x[2] - x[0]);
        b[n - 1] = b[n - 2] / (x[n - 1] - x[n - 3]) - b[n - 3] / (x[n - 2] - x[n - 4]);
        b[0] = b[0] * c[0] * c[0] / (x[3] - x[0]);
        b[n - 1] = -b[n - 1] * c[n - 2] * c[n - 2] / (x[n - 1] - x[n - 4]);
    }
    for (int i = 1; i < n; i++) {
        double h = c[i - 1] / a[i - 1];
        a[i] -= h * c[i - 1];
        b[i] -= h * b[i - 1];
    }
    b[n - 1] /= a[n - 1];
    for (int i = n - 2; i >= 0; i--) b[i] = (b[i] - c[i] * b[i + 1]) / a[i];
    for (int i = 0; i < n - 1; i++) {
        a[i] = (y[i + 1] - y[i]) / c[i] - c[i] * (b[i + 1] + 2.0 * b[i]);
        c[i] = (b[i + 1] - b[i]) / c[i];
        b[i] = 3.0 * b[i];
    }
    double in = 0.0;
    for (int i = 0; i < n - 1; i++) {
        double d = x[i + 1] - x[i];
        in += d * (y[i] + d * (a[i] / 2.0 + d * (b[i] / 3.0 + d * c[i] / 4.0)));
    }
    return in;
}

// v_l = TTweight_l / (2l+1)^{2/3}: the P_l table on the device carries (2l+1)^{2/3}.
__global__ void k_transfer_weight(int lmax, const double *__restrict__ cl, double *__restrict__ v)
{
    int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l > lmax) return;
    v[l] = (l > 1) ? pow(2e0 * l + 1e0, 5e0 / 6e0) * (1.0 / sqrt(cl[l])) / pow(2e0 * l + 1e0, 2e0 / 3e0) : 0e0;
}

// mt2[x][k][p][q] = sum_l pl[l][k] v_l qt[x][p][l] q[l-lmin][q]; tile 64 mu x 32 (p,q), l ascending.
constexpr int TR_BK = 64, TR_BU = 32, TR_LC = 16;

// With v2/qt2 (polarised E side): the transfer factor is v_l qt - v2_l qt2.
// qt and qt2 rows have stride qstride (lmax_T + 1).
__global__ void __launch_bounds__(256) k_mij_transfer(int nmu, int lmin, int lmax, int P, int Pp,
                                                      const double *__restrict__ pl, const double *__restrict__ q,
                                                      const double *__restrict__ v, const double *__restrict__ qt,
                                                      double *__restrict__ mt2, const double *__restrict__ v2 = nullptr,
                                                      const double *__restrict__ qt2 = nullptr, int qstride = 0)
{
    __shared__ double sPl[TR_LC][TR_BK];
    __shared__ double sV[TR_LC][TR_BU];
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int k0 = blockIdx.x * TR_BK, u0 = blockIdx.y * TR_BU, xi = blockIdx.z;
    const int L = lmax - lmin + 1, nu = Pp * P;
    if (qstride == 0) qstride = lmax + 1;
    const double *qtx = qt + (size_t)xi * Pp * qstride;
    const double *qtx2 = qt2 ? qt2 + (size_t)xi * Pp * qstride : nullptr;
    double acc[8];
#pragma unroll
    for (int r = 0; r < 8; r++) acc[r] = 0.0;
    for (int l0 = 0; l0 < L; l0 += TR_LC) {
#pragma unroll
        for (int t = 0; t < (TR_LC * TR_BK) / 256; t++) {
            int e = tid + 256 * t, lr = e / TR_BK, kc = e % TR_BK;
            int l = l0 + lr, k = k0 + kc;
            sPl[lr][kc] = (l < L && k < nmu) ? pl[(size_t)(lmin + l) * nmu + k] : 0.0;
        }
#pragma unroll
        for (int t = 0; t < (TR_LC * TR_BU) / 256; t++) {
            int e = tid + 256 * t, lr = e / TR_BU, uc = e % TR_BU;
            int l = l0 + lr, u = u0 + uc;
            double val = 0.0;
            if (l < L && u < nu) {
                int p = u / P, qq = u - p * P;
                double t = v[lmin + l] * qtx[(size_t)p * qstride + lmin + l];
                if (qtx2) t -= v2[lmin + l] * qtx2[(size_t)p * qstride + lmin + l];
                val = t * q[(size_t)l * P + qq];
            }
            sV[lr][uc] = val;
        }
        __syncthreads();
#pragma unroll
        for (int lr = 0; lr < TR_LC; lr++) {
            double vv = sV[lr][tx];
#pragma unroll
            for (int r = 0; r < 8; r++) acc[r] = fma(sPl[lr][ty + 8 * r], vv, acc[r]);
        }
        __syncthreads();
    }
    const int u = u0 + tx;
    if (u >= nu) return;
#pragma unroll
    for (int r = 0; r < 8; r++) {
        int k = k0 + ty + 8 * r;
        if (k < nmu) mt2[((size_t)xi * nmu + k) * nu + u] = acc[r];
    }
}

// One CTA per 32 (n: primordial) x 32 (m: late) tile; thread (tx, ty) owns
// n = n0 + tx and m = m0 + ty + 8 r.
// blockIdx.z takes the radial samples [z xs, min(xsize, (z + 1) xs)); its partial
// sum goes to out + z N Nprim (k_sum_groups adds the groups in a fixed order).
__global__ void __launch_bounds__(256) k_gamma_transfer(int N, int Nprim, int P, int Pp, int nmu, int xsize, int xs, int KC,
                                                        const int *__restrict__ triples, const int *__restrict__ prim,
                                                        const double *__restrict__ mt2, const double *__restrict__ w,
                                                        const double *__restrict__ xvec, const double *__restrict__ cx,
                                                        double scale, double *__restrict__ out)
{
    extern __shared__ double smt[];
    double *sW = smt;        // [KC]
    double *sA = smt + KC;   // [KC][Pp*P]
    const int nu = Pp * P;
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int n = blockIdx.x * 32 + tx;
    int po[3] = {0, 0, 0};
    if (n < Nprim) { po[0] = prim[3 * n] * P; po[1] = prim[3 * n + 1] * P; po[2] = prim[3 * n + 2] * P; }
    int qm[4][3];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        int m = blockIdx.y * 32 + ty + 8 * r;
        for (int b = 0; b < 3; b++) qm[r][b] = (m < N) ? triples[3 * m + b] : 0;
    }
    double res[4] = {0.0, 0.0, 0.0, 0.0};
    const int xb = blockIdx.z * xs, xe = min(xsize, xb + xs);
    out += (size_t)blockIdx.z * N * Nprim;
    for (int xi = xb; xi < xe; xi++) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        const double *src0 = mt2 + (size_t)xi * nmu * nu;
        for (int k0 = 0; k0 < nmu; k0 += KC) {
            const int kc = min(KC, nmu - k0);
            const double *src = src0 + (size_t)k0 * nu;
            for (int e = tid; e < kc * nu; e += 256) sA[e] = src[e];
            if (tid < kc) sW[tid] = w[k0 + tid];
            __syncthreads();
            for (int kk = 0; kk < kc; kk++) {
                const double *A = sA + kk * nu;
                const double wk = sW[kk];
                const double *r1 = A + po[0], *r2 = A + po[1], *r3 = A + po[2];
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    double a11 = r1[qm[r][0]], a12 = r1[qm[r][1]], a13 = r1[qm[r][2]];
                    double a21 = r2[qm[r][0]], a22 = r2[qm[r][1]], a23 = r2[qm[r][2]];
                    double a31 = r3[qm[r][0]], a32 = r3[qm[r][1]], a33 = r3[qm[r][2]];
                    double t1 = fma(a23, a32, a22 * a33);
                    double t2 = fma(a23, a31, a21 * a33);
                    double t3 = fma(a22, a31, a21 * a32);
                    acc[r] = fma(wk, fma(a13, t3, fma(a12, t2, a11 * t1)), acc[r]);
                }
            }
            __syncthreads();
        }
        const double x2 = xvec[xi] * xvec[xi], c = cx[xi];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            double y = x2 * acc[r];
            if (xi < 10 && fabs(y) > 1e-18) y = 0.0;  // calculate_gamma.c:803-804
            res[r] = fma(c, y, res[r]);
        }
    }
    if (n >= Nprim) return;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        int m = blockIdx.y * 32 + ty + 8 * r;
        if (m < N) out[(size_t)m * Nprim + n] = res[r] * scale;
    }
}

// out[e] = sum over the G groups of out[g stride + e], g ascending (in place).
__global__ void k_sum_groups(long n, int G, long stride, double *__restrict__ out)
{
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    double s = out[e];
    for (int g = 1; g < G; g++) s += out[(size_t)g * stride + e];
    out[e] = s;
}

// Polarised points (gamma_2d_pt_TTE/TEE/EEE, calculate_gamma.c:558-687): the
// 3x3 block has rows = primordial legs and columns = late legs, column b taken
// from the T table (b < nT: FORM 1 TTE nT = 2, FORM 2 TEE nT = 1) or the E
// table (FORM 3 EEE: all E); its permanent, weighted, summed over mu.
template <int FORM>
__global__ void __launch_bounds__(256) k_gamma_transfer_pol(int N, int Nprim, int P, int PE, int Pp, int nmu,
                                                            int xsize, int xs, long gstride, int KC,
                                                            const int *__restrict__ triples,
                                                            const int *__restrict__ prim,
                                                            const double *__restrict__ mtT,
                                                            const double *__restrict__ mtE,
                                                            const double *__restrict__ w,
                                                            const double *__restrict__ xvec,
                                                            const double *__restrict__ cx, double scale,
                                                            double *__restrict__ out)
{
    constexpr int nT = (FORM == 1) ? 2 : (FORM == 2 ? 1 : 0);
    extern __shared__ double smt[];
    const int nuT = (nT > 0) ? Pp * P : 0, nuE = Pp * PE;
    double *sW = smt;               // [KC]
    double *sT = smt + KC;          // [KC][Pp*P]
    double *sE = sT + KC * nuT;     // [KC][Pp*PE]
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int n = blockIdx.x * 32 + tx;
    int pa[3] = {0, 0, 0};
    if (n < Nprim) { pa[0] = prim[3 * n]; pa[1] = prim[3 * n + 1]; pa[2] = prim[3 * n + 2]; }
    int qm[4][3];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        int m = blockIdx.y * 32 + ty + 8 * r;
        for (int b = 0; b < 3; b++) qm[r][b] = (m < N) ? triples[3 * m + b] : 0;
    }
    double res[4] = {0.0, 0.0, 0.0, 0.0};
    const int xb = blockIdx.z * xs, xe = min(xsize, xb + xs);  // this CTA's radial samples (as k_gamma_transfer)
    out += (size_t)blockIdx.z * gstride;
    for (int xi = xb; xi < xe; xi++) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        for (int k0 = 0; k0 < nmu; k0 += KC) {
            const int kc = min(KC, nmu - k0);
            if (nT > 0)
                for (int e = tid; e < kc * nuT; e += 256) sT[e] = mtT[((size_t)xi * nmu + k0) * nuT + e];
            for (int e = tid; e < kc * nuE; e += 256) sE[e] = mtE[((size_t)xi * nmu + k0) * nuE + e];
            if (tid < kc) sW[tid] = w[k0 + tid];
            __syncthreads();
            for (int kk = 0; kk < kc; kk++) {
                const double *T = sT + kk * nuT, *E = sE + kk * nuE;
                const double wk = sW[kk];
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    double a[3][3];
#pragma unroll
                    for (int x = 0; x < 3; x++)
#pragma unroll
                        for (int b = 0; b < 3; b++)
                            a[x][b] = (b < nT) ? T[pa[x] * P + qm[r][b]] : E[pa[x] * PE + qm[r][b]];
                    const double t1 = fma(a[1][2], a[2][1], a[1][1] * a[2][2]);
                    const double t2 = fma(a[1][2], a[2][0], a[1][0] * a[2][2]);
                    const double t3 = fma(a[1][1], a[2][0], a[1][0] * a[2][1]);
                    acc[r] = fma(wk, fma(a[0][2], t3, fma(a[0][1], t2, a[0][0] * t1)), acc[r]);
                }
            }
            __syncthreads();
        }
        const double x2 = xvec[xi] * xvec[xi], c = cx[xi];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            double y = x2 * acc[r];
            if (xi < 10 && fabs(y) > 1e-18) y = 0.0;  // calculate_gamma.c:803-804 (and :812-826)
            res[r] = fma(c, y, res[r]);
        }
    }
    if (n >= Nprim) return;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        int m = blockIdx.y * 32 + ty + 8 * r;
        if (m < N) out[(size_t)m * Nprim + n] = res[r] * scale;
    }
}

}  // namespace modal

using namespace modal;

extern "C" modal_status modal_set_transfer(modal_ctx *c, int Pp, int xsize, const double *xvec, const double *qtilde,
                                           int Nprim, const int *prim)
{
    if (!c || !c->have_basis) { set_error("modal_set_transfer: set the basis first"); return MODAL_ERR_STATE; }
    if (Pp < 1 || Pp > 64 || xsize < 4 || Nprim < 1 || !xvec || !qtilde || !prim) {
        set_error("modal_set_transfer: Pp=%d xsize=%d (>= 4 points) Nprim=%d", Pp, xsize, Nprim);
        return MODAL_ERR_ARG;
    }
    for (long e = 0; e < 3L * Nprim; e++)
        if (prim[e] < 0 || prim[e] >= Pp) { set_error("modal_set_transfer: primordial mode index %d outside [0,%d)", prim[e], Pp); return MODAL_ERR_ARG; }
    for (int i = 1; i < xsize; i++)
        if (!(xvec[i] > xvec[i - 1])) { set_error("modal_set_transfer: x grid must increase"); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    // spline weights c_x = integral of the reference spline through e_x
    std::vector<double> cx(xsize), e(xsize, 0.0);
    for (int i = 0; i < xsize; i++) {
        e[i] = 1.0;
        cx[i] = spline_integral(xvec, e.data(), xsize);
        e[i] = 0.0;
    }
    const size_t nq = (size_t)xsize * Pp * (c->lmax + 1);
    MODAL_TRY(ensure(c->tr_x, sizeof(double) * 2 * xsize));
    MODAL_TRY(ensure(c->tr_qt, sizeof(double) * nq));
    MODAL_TRY(ensure(c->tr_prim, sizeof(int) * 3 * (size_t)Nprim));
    MODAL_CUDA(cudaMemcpyAsync(c->tr_x.ptr, xvec, sizeof(double) * xsize, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(c->tr_x.as<double>() + xsize, cx.data(), sizeof(double) * xsize, cudaMemcpyHostToDevice,
                               c->stream));
    MODAL_CUDA(cudaMemcpyAsync(c->tr_qt.ptr, qtilde, sizeof(double) * nq, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(c->tr_prim.ptr, prim, sizeof(int) * 3 * Nprim, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    c->tr_Pp = Pp;
    c->tr_xsize = xsize;
    c->tr_Nprim = Nprim;
    return MODAL_OK;
}

extern "C" modal_status modal_gamma_transfer(modal_ctx *c, double deltaphi, double *gamma_t)
{
    if (!c || !c->have_modes || !c->have_spec || c->tr_xsize < 4) {
        set_error("modal_gamma_transfer: set basis, modes, spectrum and transfer functions first");
        return MODAL_ERR_STATE;
    }
    MODAL_CUDA(cudaSetDevice(c->device));
    if (!c->have_glint) MODAL_TRY(modal_init_glint(c));
    const int P = c->P, Pp = c->tr_Pp, xsize = c->tr_xsize, nmu = c->nmu, N = c->N, Nprim = c->tr_Nprim;
    const int nu = Pp * P;
    MODAL_TRY(ensure(c->tr_mt, sizeof(double) * (size_t)xsize * nmu * nu));
    MODAL_TRY(ensure(c->tr_v, sizeof(double) * (c->lmax + 1)));
    MODAL_TRY(ensure(c->tr_out, sizeof(double) * (size_t)N * Nprim));
    StageTimer t(c, MODAL_T_GAMMA);
    k_transfer_weight<<<ceil_div(c->lmax + 1, 256), 256, 0, c->stream>>>(c->lmax, c->cl.as<double>(), c->tr_v.as<double>());
    MODAL_TRY(launched(c, "transfer_weight"));
    dim3 gm(ceil_div(nmu, TR_BK), ceil_div(nu, TR_BU), xsize);
    k_mij_transfer<<<gm, 256, 0, c->stream>>>(nmu, c->lmin, c->lmax, P, Pp, c->pl.as<double>(), c->q.as<double>(),
                                              c->tr_v.as<double>(), c->tr_qt.as<double>(), c->tr_mt.as<double>());
    MODAL_TRY(launched(c, "mij_transfer"));
    int KC = (96 * 1024) / (nu * 8);
    if (KC < 1) KC = 1;
    if (KC > 32) KC = 32;
    const size_t smem = sizeof(double) * ((size_t)KC + (size_t)KC * nu);
    if (smem > 200 * 1024) { set_error("modal_gamma_transfer: Pp*P=%d too large for the tile", nu); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaFuncSetAttribute(k_gamma_transfer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // the (primordial x late) tiles alone fill about two thirds of the SMs at the
    // benchmark sizes: split the radial samples into groups so that the grid holds
    // about 16 CTAs per SM (measured: 4 -> 67 ms, 8 -> 59 ms, 16 -> 57 ms at l <= 600),
    // and add the groups' partial sums afterwards
    int nsm = 0;
    MODAL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    const long tiles = (long)ceil_div(Nprim, 32) * ceil_div(N, 32);
    int XG = (int)std::min<long>(xsize, std::max<long>(1, (16L * nsm + tiles - 1) / tiles));
    const int xs = ceil_div(xsize, XG);
    XG = ceil_div(xsize, xs);
    MODAL_TRY(ensure(c->tr_out, sizeof(double) * (size_t)XG * N * Nprim));
    dim3 gg(ceil_div(Nprim, 32), ceil_div(N, 32), XG);
    const double scale = deltaphi * deltaphi / (8.0 * 3.14159265358979323846);
    k_gamma_transfer<<<gg, 256, smem, c->stream>>>(N, Nprim, P, Pp, nmu, xsize, xs, KC, c->triples.as<int>(),
                                                   c->tr_prim.as<int>(), c->tr_mt.as<double>(), c->w.as<double>(),
                                                   c->tr_x.as<double>(), c->tr_x.as<double>() + xsize, scale,
                                                   c->tr_out.as<double>());
    MODAL_TRY(launched(c, "gamma_transfer"));
    if (XG > 1) {
        const long n = (long)N * Nprim;
        k_sum_groups<<<ceil_div(n, 256), 256, 0, c->stream>>>(n, XG, n, c->tr_out.as<double>());
        MODAL_TRY(launched(c, "sum_groups"));
    }
    t.stop();
    if (gamma_t)
        MODAL_CUDA(cudaMemcpyAsync(gamma_t, c->tr_out.ptr, sizeof(double) * (size_t)N * Nprim, cudaMemcpyDeviceToHost,
                                   c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}

// E-side weights of calculate_gamma.c:142-183 on the host, divided by the
// (2l+1)^{2/3} the device P_l table carries:
//   EEweight_l = (2l+1)^{5/6} b_E / sqrt(s_TT (s_TT s_EE - s_TE^2))
//   wq_l = EEweight_l s_TT,  wl_l = EEweight_l (sqrt(fE/fT) b_TE^2 C_TE + N_TE)
// so that the effective E transfer function is wq_l q~_E - wl_l q~_T.
extern "C" modal_status modal_set_transfer_pol(modal_ctx *c, const double *qtilde_e, const modal_pol_spectra *sp)
{
    if (!c || !qtilde_e || !sp) { set_error("modal_set_transfer_pol: NULL argument"); return MODAL_ERR_ARG; }
    if (c->tr_xsize < 4 || !c->have_pol) {
        set_error("modal_set_transfer_pol: call modal_set_transfer, modal_set_basis_e and modal_set_modes_pol first");
        return MODAL_ERR_STATE;
    }
    if (c->lmax_e > c->lmax) {
        set_error("modal_set_transfer_pol: lmax_E=%d must not exceed lmax_T=%d", c->lmax_e, c->lmax);
        return MODAL_ERR_ARG;
    }
    const double *arr[9] = {sp->cl_tt, sp->cl_te, sp->cl_ee, sp->beam_tt, sp->beam_te, sp->beam_ee,
                            sp->noise_tt, sp->noise_te, sp->noise_ee};
    for (const double *a : arr)
        if (!a) { set_error("modal_set_transfer_pol: a spectrum array is NULL"); return MODAL_ERR_ARG; }
    if (!(sp->fsky_t > 0.0) || !(sp->fsky_e > 0.0)) { set_error("modal_set_transfer_pol: fsky must be > 0"); return MODAL_ERR_ARG; }
    const int lmax = c->lmax;
    std::vector<double> wq(lmax + 1, 0.0), wl(lmax + 1, 0.0);
    for (int l = std::max(c->lmin_e, 2); l <= c->lmax_e; l++) {
        const double s2 = sp->beam_tt[l] * sp->beam_tt[l] * sp->cl_tt[l] + sp->noise_tt[l];
        const double s3 = sp->beam_tt[l] * sp->beam_ee[l] * sp->cl_te[l] + sp->noise_te[l];
        const double s4 = sp->beam_ee[l] * sp->beam_ee[l] * sp->cl_ee[l] + sp->noise_ee[l];
        const double den = s2 * (s2 * s4 - s3 * s3);
        if (!(den > 0.0)) { set_error("modal_set_transfer_pol: TT/TE/EE covariance not positive at l=%d", l); return MODAL_ERR_ARG; }
        const double eew = std::pow(2.0 * l + 1.0, 5.0 / 6.0) * (sp->beam_ee[l] / std::sqrt(den));
        const double lk = std::sqrt(sp->fsky_e / sp->fsky_t) * sp->beam_te[l] * sp->beam_te[l] * sp->cl_te[l] + sp->noise_te[l];
        const double f = std::pow(2.0 * l + 1.0, 2.0 / 3.0);
        wq[l] = eew * s2 / f;
        wl[l] = eew * lk / f;
    }
    MODAL_CUDA(cudaSetDevice(c->device));
    const size_t nq = (size_t)c->tr_xsize * c->tr_Pp * (lmax + 1);
    MODAL_TRY(ensure(c->tr_qte, sizeof(double) * nq));
    MODAL_TRY(ensure(c->tr_we, sizeof(double) * 2 * (lmax + 1)));
    MODAL_CUDA(cudaMemcpyAsync(c->tr_qte.ptr, qtilde_e, sizeof(double) * nq, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(c->tr_we.ptr, wq.data(), sizeof(double) * (lmax + 1), cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(c->tr_we.as<double>() + (lmax + 1), wl.data(), sizeof(double) * (lmax + 1),
                               cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    c->tr_pol = true;
    return MODAL_OK;
}

extern "C" modal_status modal_gamma_transfer_pol(modal_ctx *c, double deltaphi, double *gamma_tte, double *gamma_tee,
                                                 double *gamma_eee)
{
    if (!c || !c->have_modes || !c->have_spec || c->tr_xsize < 4 || !c->tr_pol || !c->have_pol) {
        set_error("modal_gamma_transfer_pol: set basis, modes, spectrum, transfer functions and their E side first");
        return MODAL_ERR_STATE;
    }
    MODAL_CUDA(cudaSetDevice(c->device));
    if (!c->have_glint) MODAL_TRY(modal_init_glint(c));
    const int P = c->P, PE = c->P_e, Pp = c->tr_Pp, xsize = c->tr_xsize, nmu = c->nmu, N = c->N, Nprim = c->tr_Nprim;
    const int nuT = Pp * P, nuE = Pp * PE;
    const size_t NP = (size_t)N * Nprim;
    MODAL_TRY(ensure(c->tr_mt, sizeof(double) * (size_t)xsize * nmu * nuT));
    MODAL_TRY(ensure(c->tr_mte, sizeof(double) * (size_t)xsize * nmu * nuE));
    MODAL_TRY(ensure(c->tr_v, sizeof(double) * (c->lmax + 1)));
    MODAL_TRY(ensure(c->tr_out, sizeof(double) * 3 * NP));
    const size_t per_mu = (size_t)nuT + nuE;
    const int KC = (int)std::max<size_t>(1, std::min<size_t>(32, (96 * 1024) / (per_mu * 8 + 8)));
    const size_t smem = sizeof(double) * ((size_t)KC + (size_t)KC * per_mu);
    if (smem > 200 * 1024) { set_error("modal_gamma_transfer_pol: Pp*(P+P_E)=%zu too large for the tile", per_mu); return MODAL_ERR_ARG; }
    StageTimer t(c, MODAL_T_GAMMA);
    k_transfer_weight<<<ceil_div(c->lmax + 1, 256), 256, 0, c->stream>>>(c->lmax, c->cl.as<double>(), c->tr_v.as<double>());
    MODAL_TRY(launched(c, "transfer_weight"));
    dim3 gT(ceil_div(nmu, TR_BK), ceil_div(nuT, TR_BU), xsize), gE(ceil_div(nmu, TR_BK), ceil_div(nuE, TR_BU), xsize);
    k_mij_transfer<<<gT, 256, 0, c->stream>>>(nmu, c->lmin, c->lmax, P, Pp, c->pl.as<double>(), c->q.as<double>(),
                                              c->tr_v.as<double>(), c->tr_qt.as<double>(), c->tr_mt.as<double>());
    MODAL_TRY(launched(c, "mij_transfer"));
    const double *wq = c->tr_we.as<double>(), *wl = wq + (c->lmax + 1);
    k_mij_transfer<<<gE, 256, 0, c->stream>>>(nmu, c->lmin_e, c->lmax_e, PE, Pp, c->pl.as<double>(), c->qe.as<double>(),
                                              wq, c->tr_qte.as<double>(), c->tr_mte.as<double>(), wl,
                                              c->tr_qt.as<double>(), c->lmax + 1);
    MODAL_TRY(launched(c, "mij_transfer_e"));
    int nsm = 0;
    MODAL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    const long tiles = (long)ceil_div(Nprim, 32) * ceil_div(N, 32);
    int XG = (int)std::min<long>(xsize, std::max<long>(1, (16L * nsm + tiles - 1) / tiles));
    const int xs = ceil_div(xsize, XG);
    XG = ceil_div(xsize, xs);
    MODAL_TRY(ensure(c->tr_out, sizeof(double) * 3 * (size_t)XG * NP));  // group g of form f at (3 g + f) NP
    dim3 gg(ceil_div(Nprim, 32), ceil_div(N, 32), XG);
    const double scale = deltaphi * deltaphi / (8.0 * 3.14159265358979323846);
    auto run = [&](auto kern, int f) -> modal_status {
        MODAL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<gg, 256, smem, c->stream>>>(N, Nprim, P, PE, Pp, nmu, xsize, xs, 3 * (long)NP, KC,
                                           c->tri_pol.as<int>() + 3 * (size_t)N * f,
                                           c->tr_prim.as<int>(), c->tr_mt.as<double>(), c->tr_mte.as<double>(),
                                           c->w.as<double>(), c->tr_x.as<double>(), c->tr_x.as<double>() + xsize, scale,
                                           c->tr_out.as<double>() + f * NP);
        MODAL_TRY(launched(c, "gamma_transfer_pol"));
        if (XG > 1) {
            k_sum_groups<<<ceil_div((long)NP, 256), 256, 0, c->stream>>>((long)NP, XG, 3 * (long)NP,
                                                                          c->tr_out.as<double>() + f * NP);
            MODAL_TRY(launched(c, "sum_groups"));
        }
        return MODAL_OK;
    };
    MODAL_TRY(run(k_gamma_transfer_pol<1>, 0));
    MODAL_TRY(run(k_gamma_transfer_pol<2>, 1));
    MODAL_TRY(run(k_gamma_transfer_pol<3>, 2));
    t.stop();
    double *outs[3] = {gamma_tte, gamma_tee, gamma_eee};
    for (int f = 0; f < 3; f++)
        if (outs[f])
            MODAL_CUDA(cudaMemcpyAsync(outs[f], c->tr_out.as<double>() + f * NP, sizeof(double) * NP,
                                       cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}
