// adjoint.cu -- reverse-mode gradients with respect to the 1D basis values q_p(l), FP64.
//
// The reference has no derivatives: its basis optimisation (basis_optimisation_mpi.c:199-337)
// prunes modes greedily by the smallest eigenvalue of leave-one-out Gamma submatrices.
// Here the quantities of the hot path are differentiated with hand-written kernels.
//
//   M[p][q](k)  = sum_l pl_l(k) q_p(l) q_q(l),     pl_l(k) = (2l+1)^{2/3} P_l(mu_k)
//   Gamma_mn    = sum_k w_k/(48 pi) perm3(M[m_a][n_b](k))              (orthogonalisation_late.c:239-336)
//   B_e[q](k)   = sum_l pl_l(k) f~_e(l) q_q(l),    f~_e = w_l f_e, e = one leg (term t, axis a) of a separable shape
//   beta_sn     = sum_k w_k/(48 pi) sum_t perm3(B_{(s,t,a)}[n_b](k))    = <S_s, Q_n>
//   <S_s,S_s>   = sum_k w_k/(48 pi) sum_{t,t'} perm3(<f~_{t,a}, f~_{t',b}>_k)
// i.e. shape projection and shape norm in Gamma's own inner product (the exact
// Gauss-Legendre form of h^2 rather than the tetrapyd sum with the approximate
// geometric factor of calculate_mode_3D.c), w_l = (2l+1)^{1/6}/sqrt(C_l + N_l/b_l^2),
// zero for l < 2 (calculate_mode_3D.c:53-62).  With the symmetrised shape and
// symmetrised modes both products carry the same 1/(48 pi) perm3 normalisation.
//
// Vector-Jacobian products for an upstream G (dL/dGamma) and Gb (dL/dbeta):
//   dM[p][q](k) = sum_{m,n} G_mn w_k/(48 pi) sum_{a,b: m_a=p, n_b=q} cof_ab(M_mn(k))
//   cof_ab      = permanent of the 2x2 block of M_mn(k) without row a and column b
//   dq_r(l)    += sum_k pl_l(k) sum_q (dM[r][q](k) + dM[q][r](k)) q_q(l)
//   dB_e[q](k)  = sum_{s,n} Gb_sn w_k/(48 pi) sum_t sum_{a,b: e=(s,t,a), n_b=q} cof_ab(B(k))
//   dq_q(l)    += sum_k pl_l(k) sum_e f~_e(l) dB_e[q](k)
// The Gamma adjoint recomputes M(mu_k) from the Legendre table and q inside each
// CTA instead of reading a stored copy.  Objectives built on these:
//   alpha_s = Gamma^{-1} beta_s = lambda^T lambda beta_s  (the orthogonalisation's factor)
//   dL/dbeta_s = u_s, dL/dGamma = -sum_s u_s alpha_s^T,   u_s = Gamma^{-1} dL/dalpha_s
//   J = (1/S) sum_s (<S_s,S_s> - beta_s^T alpha_s) / <S_s,S_s>
//   dJ/dGamma = sum_s c_s alpha_s alpha_s^T, dJ/dbeta_s = -2 c_s alpha_s, c_s = 1/(S <S_s,S_s>).
#include <algorithm>
#include <vector>
#include "common.cuh"

namespace modal {

namespace {

constexpr double kInv48Pi = 1.0 / (48.0 * 3.14159265358979323846);

// out[k][c] = sum_{l=lmin}^{lmax} pl[l][k] vecs[ca[c]][l-lmin] vecs[cb[c]][l-lmin];
// vecs holds per-l rows [nvec][L].  Tile: 64 mu nodes x 32 columns, 16 l per stage.
constexpr int AJ_BK = 64, AJ_BC = 32, AJ_LC = 16;

__global__ void __launch_bounds__(256) k_lcontract(int nmu, int lmin, int lmax, int ncol, const double *__restrict__ pl,
                                                   const double *__restrict__ vecs, const int *__restrict__ ca,
                                                   const int *__restrict__ cb, double *__restrict__ out)
{
    __shared__ double sPl[AJ_LC][AJ_BK];
    __shared__ double sV[AJ_LC][AJ_BC];
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const int k0 = blockIdx.x * AJ_BK, c0 = blockIdx.y * AJ_BC;
    const int L = lmax - lmin + 1;
    double acc[8];
#pragma unroll
    for (int r = 0; r < 8; r++) acc[r] = 0.0;
    for (int l0 = 0; l0 < L; l0 += AJ_LC) {
#pragma unroll
        for (int t = 0; t < (AJ_LC * AJ_BK) / 256; t++) {
            const int e = tid + 256 * t, lr = e / AJ_BK, kc = e % AJ_BK;
            const int l = l0 + lr, k = k0 + kc;
            sPl[lr][kc] = (l < L && k < nmu) ? pl[(size_t)(lmin + l) * nmu + k] : 0.0;
        }
#pragma unroll
        for (int t = 0; t < (AJ_LC * AJ_BC) / 256; t++) {
            const int e = tid + 256 * t, lr = e / AJ_BC, cc = e % AJ_BC;
            const int l = l0 + lr, c = c0 + cc;
            sV[lr][cc] = (l < L && c < ncol) ? vecs[(size_t)ca[c] * L + l] * vecs[(size_t)cb[c] * L + l] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int lr = 0; lr < AJ_LC; lr++) {
            const double vv = sV[lr][tx];
#pragma unroll
            for (int r = 0; r < 8; r++) acc[r] = fma(sPl[lr][ty + 8 * r], vv, acc[r]);
        }
        __syncthreads();
    }
    const int c = c0 + tx;
    if (c >= ncol) return;
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const int k = k0 + ty + 8 * r;
        if (k < nmu) out[(size_t)k * ncol + c] = acc[r];
    }
}

__device__ __forceinline__ double perm3(const double a[3][3])
{
    return a[0][0] * (a[1][1] * a[2][2] + a[1][2] * a[2][1]) + a[0][1] * (a[1][0] * a[2][2] + a[1][2] * a[2][0]) +
           a[0][2] * (a[1][0] * a[2][1] + a[1][1] * a[2][0]);
}

// Permanent of a without row r and column c.
__device__ __forceinline__ double cof3(const double a[3][3], int r, int c)
{
    const int r1 = (r == 0) ? 1 : 0, r2 = (r == 2) ? 1 : 2;
    const int c1 = (c == 0) ? 1 : 0, c2 = (c == 2) ? 1 : 2;
    return a[r1][c1] * a[r2][c2] + a[r1][c2] * a[r2][c1];
}

// Per-shape leg bookkeeping on the device.  BK rows are [ncolB | ncolK] with row
// stride `stride`: B columns (e, q) at e*P + q, Gram columns of shape s at
// ncolB + kb[s] + i*(3T) + j.
struct LegInfo {
    int nshape, P, ncolB, stride;
    const int *leg0;   // [S] first leg of shape s
    const int *nterm;  // [S] separable terms of shape s
    const int *kb;     // [S] first Gram column of shape s
};

__global__ void __launch_bounds__(128) k_beta_gl(int N, int nmu, LegInfo li, const int *__restrict__ triples,
                                                 const double *__restrict__ w, const double *__restrict__ BK,
                                                 double *__restrict__ beta)
{
    const int s = blockIdx.y;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const int P = li.P, e0 = li.leg0[s], T = li.nterm[s];
    const int nb[3] = {triples[3 * n], triples[3 * n + 1], triples[3 * n + 2]};
    double acc = 0.0;
    for (int k = 0; k < nmu; k++) {
        const double *Bk = BK + (size_t)k * li.stride;
        double sk = 0.0;
        for (int t = 0; t < T; t++) {
            double a[3][3];
#pragma unroll
            for (int x = 0; x < 3; x++)
#pragma unroll
                for (int y = 0; y < 3; y++) a[x][y] = Bk[(e0 + 3 * t + x) * P + nb[y]];
            sk += perm3(a);
        }
        acc = fma(w[k] * kInv48Pi, sk, acc);
    }
    beta[(size_t)s * N + n] = acc;
}

// norm2[s] = <S_s,S_s>: one CTA per shape, threads over mu nodes, tree reduction.
__global__ void __launch_bounds__(128) k_norm_gl(int nmu, LegInfo li, const double *__restrict__ w,
                                                 const double *__restrict__ BK, double *__restrict__ norm2)
{
    __shared__ double red[128];
    const int s = blockIdx.x, T = li.nterm[s], T3 = 3 * T;
    double acc = 0.0;
    for (int k = threadIdx.x; k < nmu; k += blockDim.x) {
        const double *Kk = BK + (size_t)k * li.stride + li.ncolB + li.kb[s];
        double sk = 0.0;
        for (int t = 0; t < T; t++)
            for (int u = 0; u < T; u++) {
                double a[3][3];
#pragma unroll
                for (int x = 0; x < 3; x++)
#pragma unroll
                    for (int y = 0; y < 3; y++) a[x][y] = Kk[(3 * t + x) * T3 + 3 * u + y];
                sk += perm3(a);
            }
        acc = fma(w[k] * kInv48Pi, sk, acc);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) norm2[s] = red[0];
}

// Gamma adjoint, one CTA per mu node k.  M(k) is rebuilt in shared memory from the
// Legendre table and q (64 l per stage), then every (m, n) with G_mn != 0 scatters
// its nine weighted cofactors into dM(k) (shared-memory atomics).
constexpr int GV_LC = 64;

__global__ void __launch_bounds__(256) k_gamma_vjp(int N, int P, int nmu, int lmin, int lmax,
                                                   const int *__restrict__ triples, const double *__restrict__ pl,
                                                   const double *__restrict__ q, const double *__restrict__ w,
                                                   const double *__restrict__ G, double *__restrict__ dM)
{
    extern __shared__ double sm[];
    const int k = blockIdx.x, PP = P * P, L = lmax - lmin + 1;
    double *sM = sm, *sD = sM + PP, *sQ = sD + PP, *sPl = sQ + GV_LC * P;
    for (int e = threadIdx.x; e < PP; e += blockDim.x) { sM[e] = 0.0; sD[e] = 0.0; }
    for (int l0 = 0; l0 < L; l0 += GV_LC) {
        const int nl = min(GV_LC, L - l0);
        __syncthreads();
        for (int e = threadIdx.x; e < nl * P; e += blockDim.x) sQ[e] = q[(size_t)l0 * P + e];
        for (int e = threadIdx.x; e < nl; e += blockDim.x) sPl[e] = pl[(size_t)(lmin + l0 + e) * nmu + k];
        __syncthreads();
        for (int e = threadIdx.x; e < PP; e += blockDim.x) {
            const int p = e / P, r = e - p * P;
            if (r < p) continue;
            double acc = 0.0;
            for (int l = 0; l < nl; l++) acc = fma(sPl[l] * sQ[l * P + p], sQ[l * P + r], acc);
            sM[e] += acc;
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < PP; e += blockDim.x) {
        const int p = e / P, r = e - p * P;
        if (r < p) sM[e] = sM[r * P + p];
    }
    __syncthreads();
    const double wk = w[k] * kInv48Pi;
    const long NN = (long)N * N;
    for (long e = threadIdx.x; e < NN; e += blockDim.x) {
        const double g = G[e];
        if (g == 0.0) continue;
        const int m = (int)(e / N), n = (int)(e - (long)m * N);
        const int ma[3] = {triples[3 * m], triples[3 * m + 1], triples[3 * m + 2]};
        const int nb[3] = {triples[3 * n], triples[3 * n + 1], triples[3 * n + 2]};
        double a[3][3];
#pragma unroll
        for (int x = 0; x < 3; x++)
#pragma unroll
            for (int y = 0; y < 3; y++) a[x][y] = sM[ma[x] * P + nb[y]];
        const double gw = g * wk;
#pragma unroll
        for (int x = 0; x < 3; x++)
#pragma unroll
            for (int y = 0; y < 3; y++) atomicAdd(&sD[ma[x] * P + nb[y]], gw * cof3(a, x, y));
    }
    __syncthreads();
    for (int e = threadIdx.x; e < PP; e += blockDim.x) dM[(size_t)k * PP + e] = sD[e];
}

// Projection adjoint, one CTA per mu node k: B(k) staged in shared memory,
// dB(k) accumulated there.
__global__ void __launch_bounds__(256) k_beta_vjp(int N, int nmu, LegInfo li, int E, const int *__restrict__ triples,
                                                  const double *__restrict__ BK, const double *__restrict__ w,
                                                  const double *__restrict__ Gb, double *__restrict__ dB)
{
    extern __shared__ double sm[];
    const int k = blockIdx.x, P = li.P, EP = E * P;
    double *sB = sm, *sD = sm + EP;
    for (int e = threadIdx.x; e < EP; e += blockDim.x) { sB[e] = BK[(size_t)k * li.stride + e]; sD[e] = 0.0; }
    __syncthreads();
    const double wk = w[k] * kInv48Pi;
    const long SN = (long)li.nshape * N;
    for (long e = threadIdx.x; e < SN; e += blockDim.x) {
        const double g = Gb[e];
        if (g == 0.0) continue;
        const int s = (int)(e / N), n = (int)(e - (long)s * N);
        const int nb[3] = {triples[3 * n], triples[3 * n + 1], triples[3 * n + 2]};
        const int e0 = li.leg0[s], T = li.nterm[s];
        const double gw = g * wk;
        for (int t = 0; t < T; t++) {
            const int lg = e0 + 3 * t;
            double a[3][3];
#pragma unroll
            for (int x = 0; x < 3; x++)
#pragma unroll
                for (int y = 0; y < 3; y++) a[x][y] = sB[(lg + x) * P + nb[y]];
#pragma unroll
            for (int x = 0; x < 3; x++)
#pragma unroll
                for (int y = 0; y < 3; y++) atomicAdd(&sD[(lg + x) * P + nb[y]], gw * cof3(a, x, y));
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < EP; e += blockDim.x) dB[(size_t)k * EP + e] = sD[e];
}

// dq[l][r] += sum_c (Z[l][r*P+c] + Z[l][c*P+r]) q[l][c]      (Z = pl^T dM)
__global__ void k_dq_gamma(int L, int P, const double *__restrict__ Z, const double *__restrict__ q,
                           double *__restrict__ dq)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= L * P) return;
    const int l = e / P, r = e - l * P;
    const double *z = Z + (size_t)l * P * P;
    double acc = 0.0;
    for (int c = 0; c < P; c++) acc = fma(z[r * P + c] + z[c * P + r], q[(size_t)l * P + c], acc);
    dq[e] += acc;
}

// dq[l][c] += sum_e f~_e(l) Z2[l][e*P+c]      (Z2 = pl^T dB)
__global__ void k_dq_beta(int L, int P, int E, const double *__restrict__ Z2, const double *__restrict__ legs,
                          double *__restrict__ dq)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L * P) return;
    const int l = i / P, c = i - l * P;
    const double *z = Z2 + (size_t)l * E * P;
    double acc = 0.0;
    for (int e = 0; e < E; e++) acc = fma(legs[(size_t)e * L + l], z[e * P + c], acc);
    dq[i] += acc;
}

// vecs rows [0, P): basis columns q_p(l); rows [P, P+E): weighted legs w_l f_e(l).
__global__ void k_adj_vecs(int L, int lmin, int P, int E, const double *__restrict__ q, const double *__restrict__ wl,
                           const double *__restrict__ tab, const long *__restrict__ leg_off, double *__restrict__ vecs)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)(P + E) * L) return;
    const int r = (int)(i / L), l = (int)(i - (long)r * L);
    vecs[i] = (r < P) ? q[(size_t)l * P + r] : wl[lmin + l] * tab[leg_off[r - P] + lmin + l];
}

__global__ void k_leg_weight(int lmax, const double *__restrict__ cl, double *__restrict__ wl)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l <= lmax) wl[l] = (l < 2) ? 0.0 : pow(2.0 * l + 1.0, 1.0 / 6.0) / sqrt(cl[l]);
}

// out[s][n] = f * c[s] * a[s][n]
__global__ void k_scale_rows(int S, int N, const double *__restrict__ a, const double *__restrict__ c,
                             double *__restrict__ out, double f)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (long)S * N) out[i] = f * c[i / N] * a[i];
}

// Forward state of one adjoint call; device pointers index into ctx->adj.
struct AdjFwd {
    int S = 0, E = 0, ncolB = 0, ncolK = 0;
    LegInfo li{};
    double *BK = nullptr;     // [nmu][ncolB + ncolK]
    double *vecs = nullptr;   // [P + E][L]
    double *beta = nullptr;   // [S][N]
    double *norm2 = nullptr;  // [S]
};

inline size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

// Uploads the separable shape tables, builds the legs and runs the forward
// Gauss-Legendre projection: beta [S][N] and <S,S> [S] on the device.
modal_status adj_forward(modal_ctx *c, int S, const modal_shape *shapes, AdjFwd &f)
{
    const int lmin = c->lmin, lmax = c->lmax, L = c->L, P = c->P, N = c->N, nmu = c->nmu;
    std::vector<int> leg0(S), nterm(S), kb(S);
    std::vector<long> leg_off;
    long tab_total = 0;
    int E = 0, ncolK = 0;
    for (int s = 0; s < S; s++) {
        if (shapes[s].kind != MODAL_SHAPE_SEPARABLE || shapes[s].nterms < 1 || shapes[s].nterms > 64 || !shapes[s].tab) {
            set_error("adjoint: shape %d must be separable with 1..64 terms and a table", s);
            return MODAL_ERR_ARG;
        }
        leg0[s] = E;
        nterm[s] = shapes[s].nterms;
        kb[s] = ncolK;
        for (int t = 0; t < shapes[s].nterms; t++)
            for (int a = 0; a < 3; a++) leg_off.push_back(tab_total + ((long)t * 3 + a) * (lmax + 1));
        tab_total += (long)shapes[s].nterms * 3 * (lmax + 1);
        E += 3 * shapes[s].nterms;
        ncolK += 9 * shapes[s].nterms * shapes[s].nterms;
    }
    f.S = S;
    f.E = E;
    f.ncolB = E * P;
    f.ncolK = ncolK;
    const int ncol = f.ncolB + ncolK;
    std::vector<int> ca(ncol), cb(ncol);
    for (int e = 0; e < E; e++)
        for (int qq = 0; qq < P; qq++) { ca[e * P + qq] = P + e; cb[e * P + qq] = qq; }
    for (int s = 0; s < S; s++) {
        const int T3 = 3 * nterm[s];
        for (int i = 0; i < T3; i++)
            for (int j = 0; j < T3; j++) {
                ca[f.ncolB + kb[s] + i * T3 + j] = P + leg0[s] + i;
                cb[f.ncolB + kb[s] + i * T3 + j] = P + leg0[s] + j;
            }
    }
    size_t o = 0;
    const size_t o_tab = o; o += al256(sizeof(double) * (size_t)tab_total);
    const size_t o_loff = o; o += al256(sizeof(long) * (size_t)E);
    const size_t o_ca = o; o += al256(sizeof(int) * (size_t)ncol);
    const size_t o_cb = o; o += al256(sizeof(int) * (size_t)ncol);
    const size_t o_leg0 = o; o += al256(sizeof(int) * S);
    const size_t o_nt = o; o += al256(sizeof(int) * S);
    const size_t o_kb = o; o += al256(sizeof(int) * S);
    const size_t o_wl = o; o += al256(sizeof(double) * (lmax + 1));
    const size_t o_vecs = o; o += al256(sizeof(double) * (size_t)(P + E) * L);
    const size_t o_BK = o; o += al256(sizeof(double) * (size_t)nmu * ncol);
    const size_t o_beta = o; o += al256(sizeof(double) * (size_t)S * N);
    const size_t o_n2 = o; o += al256(sizeof(double) * S);
    MODAL_TRY(ensure(c->adj, o));
    uint8_t *b = c->adj.as<uint8_t>();
    size_t off = 0;
    for (int s = 0; s < S; s++) {
        const size_t n = (size_t)shapes[s].nterms * 3 * (lmax + 1);
        MODAL_CUDA(cudaMemcpyAsync(b + o_tab + off * sizeof(double), shapes[s].tab, n * sizeof(double),
                                   cudaMemcpyHostToDevice, c->stream));
        off += n;
    }
    MODAL_CUDA(cudaMemcpyAsync(b + o_loff, leg_off.data(), sizeof(long) * E, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(b + o_ca, ca.data(), sizeof(int) * ncol, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(b + o_cb, cb.data(), sizeof(int) * ncol, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(b + o_leg0, leg0.data(), sizeof(int) * S, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(b + o_nt, nterm.data(), sizeof(int) * S, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(b + o_kb, kb.data(), sizeof(int) * S, cudaMemcpyHostToDevice, c->stream));
    double *wl = reinterpret_cast<double *>(b + o_wl);
    f.vecs = reinterpret_cast<double *>(b + o_vecs);
    f.BK = reinterpret_cast<double *>(b + o_BK);
    f.beta = reinterpret_cast<double *>(b + o_beta);
    f.norm2 = reinterpret_cast<double *>(b + o_n2);
    k_leg_weight<<<ceil_div(lmax + 1, 256), 256, 0, c->stream>>>(lmax, c->cl.as<double>(), wl);
    MODAL_TRY(launched(c, "leg_weight"));
    k_adj_vecs<<<ceil_div((long)(P + E) * L, 256), 256, 0, c->stream>>>(
        L, lmin, P, E, c->q.as<double>(), wl, reinterpret_cast<const double *>(b + o_tab),
        reinterpret_cast<const long *>(b + o_loff), f.vecs);
    MODAL_TRY(launched(c, "adj_vecs"));
    const dim3 g1(ceil_div(nmu, AJ_BK), ceil_div(ncol, AJ_BC));
    if (g1.y > 65535) { set_error("adjoint: %d projection columns exceed one launch", ncol); return MODAL_ERR_ARG; }
    k_lcontract<<<g1, 256, 0, c->stream>>>(nmu, lmin, lmax, ncol, c->pl.as<double>(), f.vecs,
                                           reinterpret_cast<const int *>(b + o_ca),
                                           reinterpret_cast<const int *>(b + o_cb), f.BK);
    MODAL_TRY(launched(c, "lcontract_legs"));
    f.li.nshape = S;
    f.li.P = P;
    f.li.ncolB = f.ncolB;
    f.li.stride = ncol;
    f.li.leg0 = reinterpret_cast<const int *>(b + o_leg0);
    f.li.nterm = reinterpret_cast<const int *>(b + o_nt);
    f.li.kb = reinterpret_cast<const int *>(b + o_kb);
    const dim3 g2(ceil_div(N, 128), S);
    k_beta_gl<<<g2, 128, 0, c->stream>>>(N, nmu, f.li, c->triples.as<int>(), c->w.as<double>(), f.BK, f.beta);
    MODAL_TRY(launched(c, "beta_gl"));
    k_norm_gl<<<S, 128, 0, c->stream>>>(nmu, f.li, c->w.as<double>(), f.BK, f.norm2);
    MODAL_TRY(launched(c, "norm_gl"));
    // the host-side tables above are pageable and go out of scope on return
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}

// dq (device [L][P], accumulated) += VJP of Gamma for the upstream G [N][N] (device).
modal_status gamma_vjp_dev(modal_ctx *c, const double *G, double *dq)
{
    const int P = c->P, PP = P * P, nmu = c->nmu, L = c->L;
    const size_t smem = sizeof(double) * (2 * (size_t)PP + (size_t)GV_LC * P + GV_LC);
    if (smem > 200 * 1024) { set_error("adjoint: P=%d too large for the Gamma adjoint", P); return MODAL_ERR_ARG; }
    MODAL_TRY(ensure(c->adj2, sizeof(double) * ((size_t)nmu * PP + (size_t)L * PP)));
    double *dM = c->adj2.as<double>(), *Z = dM + (size_t)nmu * PP;
    MODAL_CUDA(cudaFuncSetAttribute(k_gamma_vjp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_gamma_vjp<<<nmu, 256, smem, c->stream>>>(c->N, P, nmu, c->lmin, c->lmax, c->triples.as<int>(),
                                               c->pl.as<double>(), c->q.as<double>(), c->w.as<double>(), G, dM);
    MODAL_TRY(launched(c, "gamma_vjp"));
    // Z[l][pq] = sum_k pl[lmin+l][k] dM[k][pq]
    MODAL_TRY(dgemm(c, L, PP, nmu, 1.0, c->pl.as<double>() + (size_t)c->lmin * nmu, nmu, false, dM, PP, false, 0.0, Z,
                    PP, 0));
    k_dq_gamma<<<ceil_div((long)L * P, 256), 256, 0, c->stream>>>(L, P, Z, c->q.as<double>(), dq);
    return launched(c, "dq_gamma");
}

// dq (device, accumulated) += VJP of beta for the upstream Gb [S][N] (device).
modal_status beta_vjp_dev(modal_ctx *c, const AdjFwd &f, const double *Gb, double *dq)
{
    const int P = c->P, nmu = c->nmu, L = c->L, E = f.E, EP = E * P;
    const size_t smem = sizeof(double) * 2 * (size_t)EP;
    if (smem > 200 * 1024) {
        set_error("adjoint: %d shape legs x P=%d exceed one CTA's shared memory", E, P);
        return MODAL_ERR_ARG;
    }
    MODAL_TRY(ensure(c->adj2, sizeof(double) * ((size_t)nmu * EP + (size_t)L * EP)));
    double *dB = c->adj2.as<double>(), *Z2 = dB + (size_t)nmu * EP;
    MODAL_CUDA(cudaFuncSetAttribute(k_beta_vjp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_beta_vjp<<<nmu, 256, smem, c->stream>>>(c->N, nmu, f.li, E, c->triples.as<int>(), f.BK, c->w.as<double>(), Gb,
                                              dB);
    MODAL_TRY(launched(c, "beta_vjp"));
    MODAL_TRY(dgemm(c, L, EP, nmu, 1.0, c->pl.as<double>() + (size_t)c->lmin * nmu, nmu, false, dB, EP, false, 0.0,
                    Z2, EP, 0));
    k_dq_beta<<<ceil_div((long)L * P, 256), 256, 0, c->stream>>>(L, P, E, Z2, f.vecs + (size_t)P * L, dq);
    return launched(c, "dq_beta");
}

// Sizes ctx->adj2 once for both adjoints of a call, so that neither reallocates
// it while the other's kernels are queued.
modal_status adj2_reserve(modal_ctx *c, const AdjFwd &f)
{
    const size_t PP = (size_t)c->P * c->P, EP = (size_t)f.E * c->P;
    return ensure(c->adj2, sizeof(double) * ((size_t)c->nmu + c->L) * std::max(PP, EP));
}

// out[s] = Gamma^{-1} in[s] = lambda^T (lambda in[s]) for S rows; tmp [S][N].
modal_status apply_ginv(modal_ctx *c, int S, const double *in, double *tmp, double *out)
{
    const int N = c->N;
    const double *lam = c->lambdal.as<double>();
    MODAL_TRY(dgemm(c, S, N, N, 1.0, in, N, false, lam, N, true, 0.0, tmp, N, 0));
    return dgemm(c, S, N, N, 1.0, tmp, N, false, lam, N, false, 0.0, out, N, 0);
}

modal_status adj_ready(modal_ctx *c, const char *who, int S, const modal_shape *shapes)
{
    if (!c) { set_error("%s: ctx is NULL", who); return MODAL_ERR_ARG; }
    if (!c->have_modes || !c->have_spec) {
        set_error("%s: set basis, modes and spectrum first", who);
        return MODAL_ERR_STATE;
    }
    if (S < 1 || !shapes) { set_error("%s: S=%d, shapes=%p", who, S, (const void *)shapes); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    if (!c->have_glint) MODAL_TRY(modal_init_glint(c));
    return MODAL_OK;
}

}  // namespace

modal_status gamma_vjp_accum_dev(modal_ctx *c, const double *G, double *dq) { return gamma_vjp_dev(c, G, dq); }

}  // namespace modal

using namespace modal;

extern "C" {

modal_status modal_project_gl(modal_ctx *c, int S, const modal_shape *shapes, double *beta, double *norm2)
{
    MODAL_TRY(adj_ready(c, "modal_project_gl", S, shapes));
    AdjFwd f;
    {
        StageTimer t(c, MODAL_T_PROJECT);
        MODAL_TRY(adj_forward(c, S, shapes, f));
    }
    if (beta)
        MODAL_CUDA(cudaMemcpyAsync(beta, f.beta, sizeof(double) * (size_t)S * c->N, cudaMemcpyDeviceToHost, c->stream));
    if (norm2) MODAL_CUDA(cudaMemcpyAsync(norm2, f.norm2, sizeof(double) * S, cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}

modal_status modal_gamma_vjp(modal_ctx *c, const double *dL_dgamma, double *dL_dq)
{
    if (!c || !dL_dgamma || !dL_dq) { set_error("modal_gamma_vjp: NULL argument"); return MODAL_ERR_ARG; }
    if (!c->have_modes) { set_error("modal_gamma_vjp: set basis and modes first"); return MODAL_ERR_STATE; }
    MODAL_CUDA(cudaSetDevice(c->device));
    if (!c->have_glint) MODAL_TRY(modal_init_glint(c));
    const int N = c->N, L = c->L, P = c->P;
    MODAL_TRY(ensure(c->adj3, sizeof(double) * ((size_t)N * N + (size_t)L * P)));
    double *G = c->adj3.as<double>(), *dq = G + (size_t)N * N;
    MODAL_CUDA(cudaMemcpyAsync(G, dL_dgamma, sizeof(double) * (size_t)N * N, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemsetAsync(dq, 0, sizeof(double) * (size_t)L * P, c->stream));
    {
        StageTimer t(c, MODAL_T_ADJOINT);
        MODAL_TRY(gamma_vjp_dev(c, G, dq));
    }
    MODAL_CUDA(cudaMemcpyAsync(dL_dq, dq, sizeof(double) * (size_t)L * P, cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}

modal_status modal_project_gl_vjp(modal_ctx *c, int S, const modal_shape *shapes, const double *dL_dbeta,
                                  double *dL_dq)
{
    MODAL_TRY(adj_ready(c, "modal_project_gl_vjp", S, shapes));
    if (!dL_dbeta || !dL_dq) { set_error("modal_project_gl_vjp: NULL argument"); return MODAL_ERR_ARG; }
    const int N = c->N, L = c->L, P = c->P;
    AdjFwd f;
    StageTimer t(c, MODAL_T_ADJOINT);
    MODAL_TRY(adj_forward(c, S, shapes, f));
    MODAL_TRY(ensure(c->adj3, sizeof(double) * ((size_t)S * N + (size_t)L * P)));
    double *Gb = c->adj3.as<double>(), *dq = Gb + (size_t)S * N;
    MODAL_CUDA(cudaMemcpyAsync(Gb, dL_dbeta, sizeof(double) * (size_t)S * N, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemsetAsync(dq, 0, sizeof(double) * (size_t)L * P, c->stream));
    MODAL_TRY(beta_vjp_dev(c, f, Gb, dq));
    t.stop();
    MODAL_CUDA(cudaMemcpyAsync(dL_dq, dq, sizeof(double) * (size_t)L * P, cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}

modal_status modal_alpha_gl(modal_ctx *c, int S, const modal_shape *shapes, double *alpha, const double *dL_dalpha,
                            double *dL_dq)
{
    MODAL_TRY(adj_ready(c, "modal_alpha_gl", S, shapes));
    if (!c->have_ortho) { set_error("modal_alpha_gl: orthogonalise first"); return MODAL_ERR_STATE; }
    if (!dL_dalpha != !dL_dq) {
        set_error("modal_alpha_gl: pass both dL_dalpha and dL_dq, or neither");
        return MODAL_ERR_ARG;
    }
    const int N = c->N, L = c->L, P = c->P;
    const size_t SN = (size_t)S * N;
    AdjFwd f;
    StageTimer t(c, MODAL_T_ADJOINT);
    MODAL_TRY(adj_forward(c, S, shapes, f));
    MODAL_TRY(ensure(c->adj3, sizeof(double) * ((size_t)N * N + (size_t)L * P + 4 * SN)));
    double *G = c->adj3.as<double>(), *dq = G + (size_t)N * N, *al = dq + (size_t)L * P, *tmp = al + SN,
           *g = tmp + SN, *u = g + SN;
    MODAL_TRY(apply_ginv(c, S, f.beta, tmp, al));
    if (alpha) MODAL_CUDA(cudaMemcpyAsync(alpha, al, sizeof(double) * SN, cudaMemcpyDeviceToHost, c->stream));
    if (dL_dalpha) {
        MODAL_CUDA(cudaMemcpyAsync(g, dL_dalpha, sizeof(double) * SN, cudaMemcpyHostToDevice, c->stream));
        MODAL_TRY(apply_ginv(c, S, g, tmp, u));
        // dL/dGamma[m][n] = -sum_s u[s][m] alpha[s][n];  dL/dbeta = u
        MODAL_TRY(dgemm(c, N, N, S, -1.0, u, N, true, al, N, false, 0.0, G, N, 0));
        MODAL_TRY(adj2_reserve(c, f));
        MODAL_CUDA(cudaMemsetAsync(dq, 0, sizeof(double) * (size_t)L * P, c->stream));
        MODAL_TRY(gamma_vjp_dev(c, G, dq));
        MODAL_TRY(beta_vjp_dev(c, f, u, dq));
        MODAL_CUDA(cudaMemcpyAsync(dL_dq, dq, sizeof(double) * (size_t)L * P, cudaMemcpyDeviceToHost, c->stream));
    }
    t.stop();
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}

modal_status modal_adjoint_residual(modal_ctx *c, int S, const modal_shape *shapes, double *J, double *dJ_dq)
{
    MODAL_TRY(adj_ready(c, "modal_adjoint_residual", S, shapes));
    if (!c->have_ortho) { set_error("modal_adjoint_residual: orthogonalise first"); return MODAL_ERR_STATE; }
    const int N = c->N, L = c->L, P = c->P;
    const size_t SN = (size_t)S * N;
    AdjFwd f;
    StageTimer t(c, MODAL_T_ADJOINT);
    MODAL_TRY(adj_forward(c, S, shapes, f));
    MODAL_TRY(ensure(c->adj3, sizeof(double) * ((size_t)N * N + (size_t)L * P + 3 * SN + S)));
    double *G = c->adj3.as<double>(), *dq = G + (size_t)N * N, *al = dq + (size_t)L * P, *tmp = al + SN,
           *ca = tmp + SN, *dcs = ca + SN;
    MODAL_TRY(apply_ginv(c, S, f.beta, tmp, al));
    std::vector<double> hn2(S), hb(SN), ha(SN);
    MODAL_CUDA(cudaMemcpyAsync(hn2.data(), f.norm2, sizeof(double) * S, cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(hb.data(), f.beta, sizeof(double) * SN, cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(ha.data(), al, sizeof(double) * SN, cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    double Jv = 0.0;
    std::vector<double> cs(S);
    for (int s = 0; s < S; s++) {
        if (!(hn2[s] > 0.0)) {
            set_error("modal_adjoint_residual: shape %d has <S,S> = %g", s, hn2[s]);
            return MODAL_ERR_ARG;
        }
        double ba = 0.0;
        for (int n = 0; n < N; n++) ba += hb[(size_t)s * N + n] * ha[(size_t)s * N + n];
        Jv += (hn2[s] - ba) / hn2[s];
        cs[s] = 1.0 / ((double)S * hn2[s]);
    }
    if (J) *J = Jv / S;
    if (dJ_dq) {
        MODAL_CUDA(cudaMemcpyAsync(dcs, cs.data(), sizeof(double) * S, cudaMemcpyHostToDevice, c->stream));
        // dJ/dGamma = sum_s c_s alpha_s alpha_s^T
        k_scale_rows<<<ceil_div((long)SN, 256), 256, 0, c->stream>>>(S, N, al, dcs, ca, 1.0);
        MODAL_TRY(launched(c, "scale_alpha"));
        MODAL_TRY(dgemm(c, N, N, S, 1.0, al, N, true, ca, N, false, 0.0, G, N, 0));
        // dJ/dbeta_s = -2 c_s alpha_s
        k_scale_rows<<<ceil_div((long)SN, 256), 256, 0, c->stream>>>(S, N, al, dcs, ca, -2.0);
        MODAL_TRY(launched(c, "scale_alpha"));
        MODAL_TRY(adj2_reserve(c, f));
        MODAL_CUDA(cudaMemsetAsync(dq, 0, sizeof(double) * (size_t)L * P, c->stream));
        MODAL_TRY(gamma_vjp_dev(c, G, dq));
        MODAL_TRY(beta_vjp_dev(c, f, ca, dq));
        MODAL_CUDA(cudaMemcpyAsync(dJ_dq, dq, sizeof(double) * (size_t)L * P, cudaMemcpyDeviceToHost, c->stream));
    }
    t.stop();
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}

}  // extern "C"
