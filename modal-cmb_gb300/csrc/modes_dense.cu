// modes_dense.cu -- projection of a dense, tabulated bispectrum onto the modes.
//
// Reference serial form (calculate_modes.c):
//   modify_bispectrum (:6-45): b[i][j][k] <- c_i c_j c_k h~^2(l_i,l_j,l_k) (1.55e-8)^2 b[i][j][k]
//     on even-parity, triangle-satisfying (l_i,l_j,l_k), 0 elsewhere, with
//     c_i = beam_i / ((2 l_i + 1)^{1/6} sqrt(beam_i^2 C_i + N_i)) when C_i != 0 and l_i != 0;
//   calculate_modes (:47-79): beta_r = sum_{i<=j<=k<size, b != 0} m(i,j,k) plijk_TTT(r,i,j,k) b[i][j][k]
//     with m = 1, 3, 6 the number of distinct orderings, the array index used as l.
// Same sum factorisation as the tetrapyd projection (project.cu): one CTA per
// slab i, rows j, contiguous k; F_i[b][c] = sum_j q_b(j) sum_k f(i,j,k) q_c(k).
#include "common.cuh"

namespace modal {

__global__ void k_project_B(int L, int P, int S, const double *__restrict__ q, const double *__restrict__ Fbuf,
                            double *__restrict__ B);
__global__ void k_project_beta(int N, int P, int S, const int *__restrict__ triples, const double *__restrict__ B,
                               double *__restrict__ beta);

__global__ void k_modify_bispectrum(int size, const int *__restrict__ vec, const double *__restrict__ c,
                                    double *__restrict__ b)
{
    const long n = (long)size * size * size;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const int k = (int)(e % size), j = (int)((e / size) % size), i = (int)(e / ((long)size * size));
        const int l1 = vec[i], l2 = vec[j], l3 = vec[k];
        double out = 0.0;
        if (((l1 + l2 + l3) % 2) == 0 && l1 + l2 >= l3 && l2 + l3 >= l1 && l3 + l1 >= l2) {
            double s1 = l1 + l2 + l3 + 1.0, s3 = l1 + l2 + l3 + 1.0 / 3.0, s6 = l1 + l2 + l3 + 1.0 / 6.0;
            double s13 = l2 + l3 - l1 + 1.0 / 3.0, s23 = l3 + l1 - l2 + 1.0 / 3.0, s33 = l1 + l2 - l3 + 1.0 / 3.0;
            double s16 = l2 + l3 - l1 + 1.0 / 6.0, s26 = l3 + l1 - l2 + 1.0 / 6.0, s36 = l1 + l2 - l3 + 1.0 / 6.0;
            const double ipi = 0.318309886183790671537767526745028724;
            double geo = (ipi * ipi / 2.0 * ((2.0 * l1 + 1.0) * (2.0 * l2 + 1.0) * (2.0 * l3 + 1.0)) / s1) *
                         (s3 / (s13 * s23 * s33)) * sqrt(s16 * s26 * s36 / s6);
            double x1 = b[e] * 1.55e-8 * 1.55e-8;
            out = c[i] * c[j] * c[k] * geo * x1;
        }
        b[e] = out;
    }
}

__global__ void k_modify_c(int size, const int *__restrict__ vec, const double *__restrict__ cl,
                           const double *__restrict__ beam, const double *__restrict__ noise, double *__restrict__ c)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= size) return;
    double v = 0.0;
    if (cl[i] != 0 && vec[i] != 0)
        v = beam[i] / (pow(2.0 * vec[i] + 1.0, 1.0 / 6.0) * sqrt(beam[i] * beam[i] * cl[i] + noise[i]));
    c[i] = v;
}

constexpr int DJC = 8;

// One CTA per slab i (index = l), rows j >= i, k >= j, all < kmax+1 = min(lmax, size-1)+1.
template <int FPT>
__global__ void __launch_bounds__(256) k_modes_slab_fp64(int lmin, int kmax, int size, int P, int KW,
                                                          const double *__restrict__ q, const double *__restrict__ b,
                                                          double *__restrict__ Fbuf)
{
    extern __shared__ double sm[];
    double *f = sm;              // [DJC][KW]
    double *H = sm + DJC * KW;   // [DJC][P]
    const int slab = blockIdx.x;
    const int i = lmin + slab;
    const int tid = threadIdx.x, PP = P * P;
    double Facc[FPT];
#pragma unroll
    for (int t = 0; t < FPT; t++) Facc[t] = 0.0;
    for (int j0 = i; j0 <= kmax; j0 += DJC) {
        for (int e = tid; e < DJC * KW; e += 256) {
            int jj = e / KW, kk = e - jj * KW, j = j0 + jj, k = j + kk;
            double v = 0.0;
            if (j <= kmax && k <= kmax) {
                double bv = b[((size_t)i * size + j) * size + k];
                double m = (i == j && j == k) ? 1.0 : ((i == j || j == k) ? 3.0 : 6.0);
                v = (bv != 0.0) ? m * bv : 0.0;
            }
            f[e] = v;
        }
        __syncthreads();
        for (int e = tid; e < DJC * P; e += 256) {
            int jj = e / P, c = e - jj * P, j = j0 + jj;
            double acc = 0.0;
            if (j <= kmax) {
                const double *fr = f + jj * KW;
                const double *qc = q + (size_t)(j - lmin) * P + c;
                const int nk = kmax - j + 1;
                for (int kk = 0; kk < nk; kk++) acc = fma(fr[kk], qc[(size_t)kk * P], acc);
            }
            H[e] = acc;
        }
        __syncthreads();
#pragma unroll
        for (int t = 0; t < FPT; t++) {
            int e = tid + 256 * t;
            if (e < PP) {
                int bb = e / P, c = e - bb * P;
                double a = 0.0;
                for (int jj = 0; jj < DJC; jj++) {
                    int j = j0 + jj;
                    if (j <= kmax) a = fma(q[(size_t)(j - lmin) * P + bb], H[jj * P + c], a);
                }
                Facc[t] += a;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int t = 0; t < FPT; t++) {
        int e = tid + 256 * t;
        if (e < PP) Fbuf[(size_t)slab * PP + e] = Facc[t];
    }
}

}  // namespace modal

using namespace modal;

extern "C" modal_status modal_modify_bispectrum(int size, const int *vec, const double *cl, const double *beam,
                                                const double *noise, double *b)
{
    if (size < 1 || !vec || !cl || !beam || !noise || !b) {
        set_error("modal_modify_bispectrum: size=%d, NULL argument", size);
        return MODAL_ERR_ARG;
    }
    modal_ctx *c = nullptr;
    MODAL_TRY(modal_ctx_create(0, &c));
    modal_status st = MODAL_OK;
    const size_t n = (size_t)size * size * size;
    DevBuf dv, dcl, dbeam, dnoise, dc, db;
    auto run = [&]() -> modal_status {
        MODAL_TRY(ensure(dv, sizeof(int) * size));
        MODAL_TRY(ensure(dcl, sizeof(double) * size));
        MODAL_TRY(ensure(dbeam, sizeof(double) * size));
        MODAL_TRY(ensure(dnoise, sizeof(double) * size));
        MODAL_TRY(ensure(dc, sizeof(double) * size));
        MODAL_TRY(ensure(db, sizeof(double) * n));
        MODAL_CUDA(cudaMemcpyAsync(dv.ptr, vec, sizeof(int) * size, cudaMemcpyHostToDevice, c->stream));
        MODAL_CUDA(cudaMemcpyAsync(dcl.ptr, cl, sizeof(double) * size, cudaMemcpyHostToDevice, c->stream));
        MODAL_CUDA(cudaMemcpyAsync(dbeam.ptr, beam, sizeof(double) * size, cudaMemcpyHostToDevice, c->stream));
        MODAL_CUDA(cudaMemcpyAsync(dnoise.ptr, noise, sizeof(double) * size, cudaMemcpyHostToDevice, c->stream));
        MODAL_CUDA(cudaMemcpyAsync(db.ptr, b, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        k_modify_c<<<ceil_div(size, 128), 128, 0, c->stream>>>(size, dv.as<int>(), dcl.as<double>(),
                                                              dbeam.as<double>(), dnoise.as<double>(), dc.as<double>());
        MODAL_TRY(launched(c, "modify_c"));
        long blocks = std::min<long>(ceil_div((long)n, 256), 152L * 16);
        k_modify_bispectrum<<<(int)blocks, 256, 0, c->stream>>>(size, dv.as<int>(), dc.as<double>(), db.as<double>());
        MODAL_TRY(launched(c, "modify_bispectrum"));
        MODAL_CUDA(cudaMemcpyAsync(b, db.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
        MODAL_CUDA(cudaStreamSynchronize(c->stream));
        return MODAL_OK;
    };
    st = run();
    DevBuf *bufs[] = {&dv, &dcl, &dbeam, &dnoise, &dc, &db};
    for (DevBuf *x : bufs) release(*x);
    modal_ctx_destroy(c);
    return st;
}

extern "C" modal_status modal_calculate_modes(modal_ctx *c, int size, const double *b, double *beta)
{
    if (!c || !c->have_modes) { set_error("modal_calculate_modes: set basis and modes first"); return MODAL_ERR_STATE; }
    if (size < 1 || !b) { set_error("modal_calculate_modes: size=%d", size); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    const int lmin = c->lmin, P = c->P, N = c->N, PP = P * P;
    const int kmax = std::min(c->lmax, size - 1);
    MODAL_TRY(ensure(c->beta, sizeof(double) * (size_t)N));
    if (kmax < lmin) {
        MODAL_CUDA(cudaMemsetAsync(c->beta.ptr, 0, sizeof(double) * N, c->stream));
    } else {
        const int nsl = kmax - lmin + 1;
        const size_t n = (size_t)size * size * size;
        const size_t fbytes = sizeof(double) * (size_t)nsl * PP, bbytes = sizeof(double) * (size_t)P * PP;
        MODAL_TRY(ensure(c->scratch2, sizeof(double) * n));
        MODAL_TRY(ensure(c->scratch, fbytes + bbytes));
        MODAL_CUDA(cudaMemcpyAsync(c->scratch2.ptr, b, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        double *Fbuf = c->scratch.as<double>(), *B = Fbuf + (size_t)nsl * PP;
        const int KW = kmax - lmin + 1;
        const size_t smem = sizeof(double) * ((size_t)DJC * KW + (size_t)DJC * P);
        if (smem > 220 * 1024) { set_error("modal_calculate_modes: size too large for the slab tile"); return MODAL_ERR_ARG; }
        const int fpt = ceil_div(PP, 256);
        auto run = [&](auto kern) -> modal_status {
            MODAL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            kern<<<nsl, 256, smem, c->stream>>>(lmin, kmax, size, P, KW, c->q.as<double>(), c->scratch2.as<double>(), Fbuf);
            return launched(c, "modes_slab_fp64");
        };
        StageTimer t(c, MODAL_T_PROJECT);
        if (fpt <= 1) MODAL_TRY(run(k_modes_slab_fp64<1>));
        else if (fpt <= 4) MODAL_TRY(run(k_modes_slab_fp64<4>));
        else if (fpt <= 8) MODAL_TRY(run(k_modes_slab_fp64<8>));
        else if (fpt <= 16) MODAL_TRY(run(k_modes_slab_fp64<16>));
        else { set_error("modal_calculate_modes: P=%d too large", P); return MODAL_ERR_ARG; }
        k_project_B<<<ceil_div((long)P * PP, 256), 256, 0, c->stream>>>(nsl, P, 1, c->q.as<double>(), Fbuf, B);
        MODAL_TRY(launched(c, "project_B"));
        k_project_beta<<<ceil_div(N, 256), 256, 0, c->stream>>>(N, P, 1, c->triples.as<int>(), B, c->beta.as<double>());
        MODAL_TRY(launched(c, "project_beta"));
    }
    c->have_beta = true;
    c->beta_S = 1;
    if (beta) MODAL_CUDA(cudaMemcpyAsync(beta, c->beta.ptr, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}
