// gamma_split.cu -- split-precision tensor-core form of Gamma: both contractions
// on the tcgen05 tensor cores, FP64 accuracy by exact integer slices.
//
// Gamma_mn = sum_k w_k/(48 pi) perm3(M(k)[m_a][n_b])   (orthogonalisation_late.c:239-336)
// is lifted to a GEMM over pairs.  With u = (a,b), a <= b, a pair of basis
// indices (U = P(P+1)/2 of them) and X_u(k) = M_ab(mu_k):
//     T[u][v][t] = sum_k X_u(k) * (w_k/(48 pi) X_v(k) X_t(k))      (fully symmetric)
//     Gamma_mn   = sum over the six orderings s of T[(m1,n_s1)][(m2,n_s2)][(m3,n_s3)]
// T is only needed for u <= v <= t.
//
// 1. l-contraction (calculate_orthoMij_T, orthogonalisation_late.c:99-129) as a
//    GEMM: X[u][k] = sum_l q_a(l) q_b(l) gl_Pl[k][l], rows (a, b) of the pair
//    products against the P_l table, on the tensor cores (ozgemm.cu, 8 slices).
// 2. mu-contraction: T[u][(v,t)] = sum_k X_u(k) Y_vt(k), Y_vt(k) = w_k/(48 pi)
//    X_v(k) X_t(k), one GEMM [U x K] x [K x U(U+1)/2] on the tensor cores with
//    7 slices; X and Y are sliced straight from FP64 (Y is never stored in
//    FP64).  Output tiles whose smallest u exceeds every v of their column tile
//    are skipped.
// 3. Gamma_mn gathered in FP64 from the six sorted-triple entries of T.
//
// Each slice product is summed exactly in FP32 tensor memory over blocks of 512
// nodes (the digits are 7-bit integers), so the rounding of the whole form is
// that of FP64 arithmetic plus the 7-slice truncation (about 2^-49 of the row
// scales): the split Gamma agrees with the plain FP64 Gamma to ~1e-14.
#include <algorithm>
#include <vector>
#include "common.cuh"
#include "dfbits.cuh"

namespace modal {

namespace {

constexpr int SP_SLICES_X = 8;   // l-contraction
constexpr int SP_SLICES_G = 7;   // mu-contraction
constexpr int SP_TILE = 128;

// Qp[u][l] = q[l][a] q[l][b] for the pair u = (a, b).
__global__ void k_pair_rows(int U, int L, int P, const int2 *__restrict__ pairs, const double *__restrict__ q,
                            double *__restrict__ Qp)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)U * L) return;
    const int u = (int)(e / L), l = (int)(e - (size_t)u * L);
    const int2 ab = pairs[u];
    Qp[e] = q[(size_t)l * P + ab.x] * q[(size_t)l * P + ab.y];
}

// weights w_k/(48 pi), zero beyond the node range
__global__ void k_wgt48(int nmu, int Kpad, const double *__restrict__ w, double *__restrict__ wk)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < Kpad) wk[k] = (k < nmu) ? w[k] / (48e0 * 3.14159265358979323846) : 0.0;
}

// Z[v][k] = wk[k] X_v(k) for k < K, 0 beyond: the first factor of every Y row
// of pair v (the product (wk X_v) X_t rounds as wk X_v X_t evaluated left to right).
__global__ void k_weight_rows(int U, int K, int Kpad, const double *__restrict__ X, const double *__restrict__ wk,
                              double *__restrict__ Z)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)U * Kpad) return;
    const int k = (int)(e % Kpad);
    Z[e] = (k < K) ? wk[k] * X[e] : 0.0;
}

// Digits of the rows Y_vt(k) = (wk[k] X_v(k)) X_t(k) = Z_v(k) X_t(k) (one FP64
// product), one warp per row: the row's exponent from its maximum, then s
// balanced 7-bit digits of y 2^{6 - e + 7(s-1)} rounded to an integer (the
// ozgemm.cu layout: out[p][r][k], FP16).  Rows >= UV are zero.  The maximum
// and the scaled rounding run on the bit patterns (integer instructions), so
// the FP64 pipe sees one multiply per element and pass.
__global__ void __launch_bounds__(256) k_slice_y(int UV, int UVpad, int K, int Kpad, const int2 *__restrict__ vt,
                                                 const double *__restrict__ X, const double *__restrict__ Z, long ldx,
                                                 int s, __half *__restrict__ out, int *__restrict__ ey)
{
    const long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= UVpad) return;
    const size_t plane = (size_t)UVpad * Kpad;
    __half *o = out + (size_t)r * Kpad;
    if (r >= UV) {
        for (int k = lane; k < Kpad; k += 32)
            for (int p = 0; p < s; p++) o[p * plane + k] = __int2half_rn(0);
        if (lane == 0) ey[r] = 0;
        return;
    }
    const int2 p2 = vt[r];
    const double *zv = Z + (size_t)p2.x * ldx, *xt = X + (size_t)p2.y * ldx;
    unsigned long long mb = 0ull;
    for (int k = lane; k < K; k += 32) mb = dfb::absmax_bits(mb, zv[k] * xt[k]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, off));
    const double m = __longlong_as_double((long long)mb);
    const int e = (m > 0.0 && isfinite(m)) ? ilogb(m) + 1 : 0;
    if (lane == 0) ey[r] = e;
    const int sh = 6 - e + 7 * (s - 1);
    for (int k = lane; k < Kpad; k += 32) {
        const double y = (k < K) ? zv[k] * xt[k] : 0.0;
        long long F;
        if (!dfb::scaled_rint(y, sh, &F)) {
            const double ys = ldexp(y, sh);
            F = isfinite(ys) ? __double2ll_rn(ys) : 0ll;
        }
        for (int p = s - 1; p > 0; p--) {
            const long long d = ((F + 64) & 127) - 64;
            o[p * plane + k] = __int2half_rn((int)d);
            F = (F - d) >> 7;
        }
        o[k] = __int2half_rn((int)F);
    }
}

// Gamma_mn = sum over the six orderings of T[lo][vt(mid, hi)] (sorted pair
// indices lo <= mid <= hi; vt(v, t) = vbase[v] + t - v, the row order of Y).
// One thread per (m, n) of a 32 x 32 tile with tile(m) <= tile(n).
__global__ void __launch_bounds__(256) k_gamma_gather64(int N, int P, int U, long ldT, const int *__restrict__ triples,
                                                        const int *__restrict__ pidx, const long long *__restrict__ vbase,
                                                        const double *__restrict__ T, double *__restrict__ gamma)
{
    const int tm = blockIdx.y, tn = blockIdx.x;
    if (tm > tn) return;
    extern __shared__ unsigned char gsm[];
    long long *sbase = reinterpret_cast<long long *>(gsm);
    int *sp = reinterpret_cast<int *>(sbase + U);
    for (int e = threadIdx.x; e < U; e += 256) sbase[e] = vbase[e];
    for (int e = threadIdx.x; e < P * P; e += 256) sp[e] = pidx[e];
    __syncthreads();
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int n = tn * 32 + tx;
    if (n >= N) return;
    const int n0 = triples[3 * n], n1 = triples[3 * n + 1], n2 = triples[3 * n + 2];
    const int perm[6][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}, {1, 0, 2}, {0, 2, 1}};
    for (int r = 0; r < 4; r++) {
        const int m = tm * 32 + ty + 8 * r;
        if (m >= N || m > n) continue;
        const int mm[3] = {triples[3 * m], triples[3 * m + 1], triples[3 * m + 2]};
        const int nn[3] = {n0, n1, n2};
        double g = 0.0;
#pragma unroll
        for (int s = 0; s < 6; s++) {
            const int x = sp[mm[0] * P + nn[perm[s][0]]];
            const int y = sp[mm[1] * P + nn[perm[s][1]]];
            const int z = sp[mm[2] * P + nn[perm[s][2]]];
            const int lo = min(x, min(y, z)), hi = max(x, max(y, z)), mid = x + y + z - lo - hi;
            g += T[(size_t)lo * ldT + sbase[mid] + (hi - mid)];
        }
        gamma[(size_t)m * N + n] = g;
        gamma[(size_t)n * N + m] = g;
    }
}

}  // namespace

modal_status gamma_split_dev(modal_ctx *ctx, int mu0, int nmu)
{
    const int P = ctx->P, N = ctx->N, L = ctx->L;
    const int U = P * (P + 1) / 2;
    const int Upad = ceil_div(U, SP_TILE) * SP_TILE;
    const long UV = (long)U * (U + 1) / 2;
    const long UVpad = (long)ceil_div(UV, SP_TILE) * SP_TILE;
    const int Kpad = ceil_div(nmu, 64) * 64;

    // host tables: pairs, pair index, (v,t) rows and their bases, output tiles
    std::vector<int2> pairs(U);
    std::vector<int> pidx((size_t)P * P);
    {
        int u = 0;
        for (int p = 0; p < P; p++)
            for (int q = p; q < P; q++) { pairs[u] = make_int2(p, q); pidx[p * P + q] = pidx[q * P + p] = u; u++; }
    }
    std::vector<long long> vbase(U);
    std::vector<int2> vtp(UV);
    {
        long r = 0;
        for (int v = 0; v < U; v++) {
            vbase[v] = r;
            for (int t = v; t < U; t++) vtp[r++] = make_int2(v, t);
        }
    }
    std::vector<int2> tiles;
    for (long j = 0; j < UVpad / SP_TILE; j++) {
        const long last = std::min(UV - 1, (j + 1) * SP_TILE - 1);
        const int vmax = vtp[last].x;
        for (int i = 0; i * SP_TILE <= vmax && i < Upad / SP_TILE; i++) tiles.push_back(make_int2(i, (int)j));
    }

    // device buffers, laid out in ctx->split (one allocation)
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t o = 0;
    // the host tables first: their offsets depend on P alone
    const size_t o_pairs = o; o += al((size_t)U * sizeof(int2));
    const size_t o_pidx = o; o += al((size_t)P * P * 4);
    const size_t o_vbase = o; o += al((size_t)U * 8);
    const size_t o_vtp = o; o += al((size_t)UV * sizeof(int2));
    const size_t o_qp = o; o += al((size_t)U * L * 8);
    const size_t o_x = o; o += al((size_t)U * Kpad * 8);
    const size_t o_wk = o; o += al((size_t)Kpad * 8);
    const size_t o_xs = o; o += al((size_t)SP_SLICES_G * Upad * Kpad * 2);
    const size_t o_ex = o; o += al((size_t)Upad * 4);
    const size_t o_ys = o; o += al((size_t)SP_SLICES_G * UVpad * Kpad * 2);
    const size_t o_ey = o; o += al((size_t)UVpad * 4);
    const size_t o_T = o; o += al((size_t)U * UV * 8);
    const size_t o_z = o; o += al((size_t)U * Kpad * 8);
    MODAL_TRY(ensure(ctx->split, o));
    uint8_t *b = ctx->split.as<uint8_t>();
    double *Qp = reinterpret_cast<double *>(b + o_qp), *X = reinterpret_cast<double *>(b + o_x);
    double *wk = reinterpret_cast<double *>(b + o_wk), *T = reinterpret_cast<double *>(b + o_T);
    // the host tables depend on P only; a reallocated buffer has lost them
    if (ctx->split_P != P || ctx->split_ptr != ctx->split.ptr || ctx->split_bytes != ctx->split.bytes) {
        MODAL_CUDA(cudaMemcpyAsync(b + o_pairs, pairs.data(), U * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream));
        MODAL_CUDA(cudaMemcpyAsync(b + o_pidx, pidx.data(), pidx.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
        MODAL_CUDA(cudaMemcpyAsync(b + o_vbase, vbase.data(), U * 8, cudaMemcpyHostToDevice, ctx->stream));
        MODAL_CUDA(cudaMemcpyAsync(b + o_vtp, vtp.data(), UV * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream));
        MODAL_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->split_P = P;
        ctx->split_ptr = ctx->split.ptr;
        ctx->split_bytes = ctx->split.bytes;
    }
    MODAL_TRY(oz_reset(ctx));
    OzOpts oz;
    oz.check = false;
    // 1. X = (pair products of q) x P_l table^T over the node range, on the tensor cores
    {
        StageTimer tm(ctx, MODAL_T_MIJ);
        k_pair_rows<<<ceil_div((long)U * L, 256), 256, 0, ctx->stream>>>(U, L, P, reinterpret_cast<const int2 *>(b + o_pairs),
                                                                          ctx->q.as<double>(), Qp);
        MODAL_TRY(launched(ctx, "pair_rows"));
        oz.slices = SP_SLICES_X;
        const double *pl = ctx->pl.as<double>() + (size_t)ctx->lmin * ctx->nmu + mu0;
        MODAL_TRY(oz_gemm_ex(ctx, U, nmu, L, 1.0, Qp, L, false, pl, ctx->nmu, false, 0.0, X, Kpad, oz));
    }
    // 2. slices of X and of Y = w X_v X_t, then T = X Y^T on the tensor cores
    k_wgt48<<<ceil_div(Kpad, 256), 256, 0, ctx->stream>>>(nmu, Kpad, ctx->w.as<double>() + mu0, wk);
    MODAL_TRY(launched(ctx, "wgt48"));
    OzOperand xs{reinterpret_cast<__half *>(b + o_xs), reinterpret_cast<int *>(b + o_ex), U, Upad};
    OzOperand ys{reinterpret_cast<__half *>(b + o_ys), reinterpret_cast<int *>(b + o_ey), (int)UV, (int)UVpad};
    MODAL_TRY(oz_slice(ctx, U, nmu, X, Kpad, false, SP_SLICES_G, Upad, Kpad, xs.slices, xs.ex));
    double *Z = reinterpret_cast<double *>(b + o_z);
    k_weight_rows<<<ceil_div((long)U * Kpad, 256), 256, 0, ctx->stream>>>(U, nmu, Kpad, X, wk, Z);
    MODAL_TRY(launched(ctx, "weight_rows"));
    k_slice_y<<<ceil_div(UVpad * 32, 256), 256, 0, ctx->stream>>>((int)UV, (int)UVpad, nmu, Kpad,
                                                                   reinterpret_cast<const int2 *>(b + o_vtp), X, Z, Kpad,
                                                                   SP_SLICES_G, ys.slices, ys.ex);
    MODAL_TRY(launched(ctx, "slice_y"));
    oz.slices = SP_SLICES_G;
    oz.ksplit = 1;
    {
        StageTimer tl(ctx, MODAL_T_LIFT);
        MODAL_TRY(oz_run(ctx, xs, ys, Kpad, SP_SLICES_G, &tiles, 1.0, 0.0, T, UV, oz));
    }
    // 3. Gamma from the sorted-triple entries of T
    MODAL_TRY(ensure(ctx->gamma, sizeof(double) * (size_t)N * N));
    const size_t gsm = (size_t)U * 8 + (size_t)P * P * 4;
    MODAL_CUDA(cudaFuncSetAttribute(k_gamma_gather64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsm));
    const int nt = ceil_div(N, 32);
    k_gamma_gather64<<<dim3(nt, nt), 256, gsm, ctx->stream>>>(N, P, U, UV, ctx->triples.as<int>(),
                                                                reinterpret_cast<const int *>(b + o_pidx),
                                                                reinterpret_cast<const long long *>(b + o_vbase), T,
                                                                ctx->gamma.as<double>());
    MODAL_TRY(launched(ctx, "gamma_gather64"));
    return oz_check(ctx);
}

}  // namespace modal
