// gl.cu -- Gauss-Legendre quadrature, the P_l(mu) table, the shifted Legendre
// basis and the asymptotic geometric factor, all FP64 on the GPU.
#include "common.cuh"

namespace modal {

// ---------------------------------------------------------------------------
// Gauss-Legendre nodes/weights (replaces asy, gl_integration.c:46-168; same
// ascending symmetric layout).  One thread per positive root.  Newton in
// theta (x = cos theta) from Tricomi's guess; P_n(cos theta) by the
// three-term recurrence in differences D_l = P_l - P_{l-1} with
// y = 1 - x = 2 sin^2(theta/2):
//     D_{l+1} = (l D_l - (2l+1) y P_l) / (l+1),  P_{l+1} = P_l + D_{l+1},
// which stays accurate next to x = 1, where the small endpoint weights carry
// a large share of the Gamma integrand.  w = 2 sin^2 theta / (n (P_{n-1} - x P_n))^2.
// Newton stops after 30 iterations at most.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void leg_diff(int n, double th, double &Pn, double &Q)
{
    double s = sin(0.5 * th);
    double y = 2.0 * s * s;
    double P = 1.0, D = 0.0;
    for (int l = 0; l < n; l++) {
        double Dn = (l * D - (2.0 * l + 1.0) * y * P) / (l + 1.0);
        P += Dn;
        D = Dn;
    }
    Pn = P;
    Q = -D + y * P;
}

__global__ void k_gl_nodes(int n, double *mu, double *w)
{
    const int half = n / 2;
    const int k = blockIdx.x * blockDim.x + threadIdx.x + 1;  // root index 1..half (+ middle)
    if (k <= half) {
        const double pi = 3.141592653589793238462643383279502884;
        double th = pi * (4.0 * k - 1.0) / (4.0 * n + 2.0);
        double x0 = (1.0 - (n - 1.0) / (8.0 * (double)n * n * n)) * cos(th);
        th = acos(x0);
        double Pn, Q;
        for (int it = 0; it < 30; it++) {
            leg_diff(n, th, Pn, Q);
            double dth = Pn * sin(th) / (n * Q);
            th += dth;
            if (fabs(dth) <= 1e-17 * th) break;
        }
        leg_diff(n, th, Pn, Q);
        double st = sin(th);
        double wk = 2.0 * st * st / ((double)n * n * Q * Q);
        double x = cos(th);
        mu[n - k] = x;
        mu[k - 1] = -x;
        w[n - k] = wk;
        w[k - 1] = wk;
    } else if (k == half + 1 && (n & 1)) {
        double Pn, Q;
        leg_diff(n, 1.5707963267948966192313216916397514, Pn, Q);
        mu[half] = 0.0;
        w[half] = 2.0 / ((double)n * n * Q * Q);
    }
}

modal_status gl_nodes_dev(modal_ctx *ctx, int n, double *d_mu, double *d_w)
{
    int threads = 64;
    int roots = n / 2 + 1;
    k_gl_nodes<<<ceil_div(roots, threads), threads, 0, ctx->stream>>>(n, d_mu, d_w);
    return launched(ctx, "gl_nodes");
}

// ---------------------------------------------------------------------------
// P_l table: pl[l][k] = (2l+1)^{2/3} P_l(mu_k), l = 0..lmax (gl_Pl of
// orthogonalisation_late.c:47-54, stored l-major so each step of the
// recurrence is one coalesced row).  P_l as gsl_sf_legendre_Pl: upward
// recurrence p_l = (x(2l-1)p_{l-1} - (l-1)p_{l-2})/l from P_0 = 1, P_1 = x,
// P_2 returned in closed form, exact values at x = +-1.  One thread per node;
// the (2l+1)^{2/3} factors come from a per-l table.
// ---------------------------------------------------------------------------
// pw[l] = (2l+1)^{2/3}
__global__ void k_pl_factors(int lmax, double *pw)
{
    int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l <= lmax) pw[l] = pow(2.0 * l + 1.0, 2.0 / 3.0);
}

// One thread per node, so that the n_mu independent recurrences spread over as
// many warps as possible: the recurrence is serial in l and GB300's FP64 rate
// per SM is low, so the length of the FP64 dependency chain, not the bytes
// written, sets the time (~1.45 ms for 3001 nodes to l = 2000: 33 GB/s of
// table).  The arithmetic is gsl_sf_legendre_Pl's upward recurrence exactly,
// (x (2l-1) P_{l-1} - (l-1) P_{l-2}) / l, with the integer factors read as
// doubles from shared memory (the same values, so the same bits; it saves
// three integer-to-FP64 conversions per step, 10%).  Folding the division into
// precomputed reciprocals is faster but moves the table by ~1e-12 at l = 500
// (the roundings accumulate coherently along l), which would show in Gamma's
// 1e-12 parity with the reference.
constexpr int PL_WPB = 1;  // warps per block (measured: 1 and 4 give the same time; the chains do not contend)
__global__ void __launch_bounds__(32 * PL_WPB) k_legendre_table(int nmu, int lmax, const double *__restrict__ mu,
                                                                const double *__restrict__ pw, double *__restrict__ pl)
{
    extern __shared__ double tab[];  // [lmax+1][3]: 2l - 1, l - 1, l
    for (int l = threadIdx.x; l <= lmax; l += blockDim.x) {
        tab[3 * l] = (double)(2 * l - 1);
        tab[3 * l + 1] = (double)(l - 1);
        tab[3 * l + 2] = (double)l;
    }
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nmu) return;
    const double x = mu[k];
    const bool xp1 = (x == 1.0), xm1 = (x == -1.0);
    pl[k] = pw[0];
    if (lmax >= 1) pl[(size_t)nmu + k] = pw[1] * x;
    double pm2 = 1.0, pm1 = x;
    for (int l = 2; l <= lmax; l++) {
        const double pr = (x * tab[3 * l] * pm1 - tab[3 * l + 1] * pm2) / tab[3 * l + 2];
        pm2 = pm1;
        pm1 = pr;
        double p = pr;
        if (l == 2) p = 0.5 * (3.0 * x * x - 1.0);
        else if (xp1) p = 1.0;
        else if (xm1) p = (l & 1) ? -1.0 : 1.0;
        pl[(size_t)l * nmu + k] = pw[l] * p;
    }
}

modal_status legendre_table_dev(modal_ctx *ctx, int nmu, int lmax, const double *d_mu, double *d_pl)
{
    MODAL_TRY(ensure(ctx->scratch2, sizeof(double) * (lmax + 1)));
    double *pw = ctx->scratch2.as<double>();
    k_pl_factors<<<ceil_div(lmax + 1, 256), 256, 0, ctx->stream>>>(lmax, pw);
    MODAL_TRY(launched(ctx, "pl_factors"));
    const size_t smem = sizeof(double) * 3 * (size_t)(lmax + 1);
    if (smem > 200 * 1024) { set_error("legendre table: lmax = %d too large", lmax); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaFuncSetAttribute(k_legendre_table, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_legendre_table<<<ceil_div(nmu, 32 * PL_WPB), 32 * PL_WPB, smem, ctx->stream>>>(nmu, lmax, d_mu, pw, d_pl);
    return launched(ctx, "legendre_table");
}

// ---------------------------------------------------------------------------
// Shifted Legendre basis (basis_functions.c:88-107): one thread per value.
// ---------------------------------------------------------------------------
__global__ void k_basis_legendre(int size, int pmax, double min, double max, const double *__restrict__ values,
                                 double *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= size) return;
    double *a = out + (size_t)i * (pmax + 1);
    double x = (values[i] - min) / (max - min);
    a[0] = 1e0;
    if (pmax > 0) a[1] = 2e0 * x - 1e0;
    double a1 = 2e0 * x - 1e0, am2 = 1e0, am1 = a1;
    for (int j = 2; j <= pmax; j++) {
        double v = ((2e0 * j - 1e0) * a1 * am1 - (j - 1e0) * am2) / (1e0 * j);
        a[j] = v;
        am2 = am1;
        am1 = v;
    }
}

// ---------------------------------------------------------------------------
// Asymptotic geometric factor (calculate_geometric.c:59-92).
// ---------------------------------------------------------------------------
__global__ void k_geometric(long npts, const int *__restrict__ pts, double *__restrict__ out)
{
    long n = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= npts) return;
    int l1 = pts[3 * n], l2 = pts[3 * n + 1], l3 = pts[3 * n + 2];
    double r = 0.0;
    if (((l1 + l2 + l3) % 2) == 0 && l1 + l2 >= l3 && l2 + l3 >= l1 && l3 + l1 >= l2) {
        double s1 = l1 + l2 + l3 + 1.0, s3 = l1 + l2 + l3 + 1.0 / 3.0, s6 = l1 + l2 + l3 + 1.0 / 6.0;
        double s13 = l2 + l3 - l1 + 1.0 / 3.0, s23 = l3 + l1 - l2 + 1.0 / 3.0, s33 = l1 + l2 - l3 + 1.0 / 3.0;
        double s16 = l2 + l3 - l1 + 1.0 / 6.0, s26 = l3 + l1 - l2 + 1.0 / 6.0, s36 = l1 + l2 - l3 + 1.0 / 6.0;
        const double ipi = 0.318309886183790671537767526745028724;
        double fact = ipi * ipi / 2.0;
        double p1 = fact * ((2.0 * l1 + 1.0) * (2.0 * l2 + 1.0) * (2.0 * l3 + 1.0)) / s1;
        double p2 = s3 / (s13 * s23 * s33);
        double p3 = sqrt(s16 * s26 * s36 / s6);
        r = p1 * p2 * p3;
    }
    out[n] = r;
}

// out[c][r] = in[r][c] for an R x C row-major FP64 matrix.
__global__ void k_transpose(const double *__restrict__ in, double *__restrict__ out, int R, int C)
{
    __shared__ double t[32][33];
    int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        int r = r0 + y, c = c0 + threadIdx.x;
        if (r < R && c < C) t[y][threadIdx.x] = in[(size_t)r * C + c];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        int c = c0 + y, r = r0 + threadIdx.x;
        if (r < R && c < C) out[(size_t)c * R + r] = t[threadIdx.x][y];
    }
}

modal_status transpose_dev(modal_ctx *ctx, const double *in, double *out, int R, int C)
{
    dim3 grid(ceil_div(C, 32), ceil_div(R, 32)), block(32, 8);
    k_transpose<<<grid, block, 0, ctx->stream>>>(in, out, R, C);
    return launched(ctx, "transpose");
}

modal_status basis_legendre_dev(modal_ctx *ctx, int size, int pmax, double min, double max, const double *d_values,
                                double *d_out)
{
    k_basis_legendre<<<ceil_div(size, 128), 128, 0, ctx->stream>>>(size, pmax, min, max, d_values, d_out);
    return launched(ctx, "basis_legendre");
}

modal_status geometric_dev(modal_ctx *ctx, long npts, const int *d_pts, double *d_out)
{
    k_geometric<<<ceil_div(npts, 256), 256, 0, ctx->stream>>>(npts, d_pts, d_out);
    return launched(ctx, "geometric");
}

}  // namespace modal
