// project.cu -- projection of bispectrum shapes onto the modes.
//
// Reference (calculate_mode_3D, calculate_mode_3D.c:217-264, over the walk of
// get_ijk_next_XXX, tetrapyd_tools.c:104-142):
//   beta_r = sum_{i<=j<=k<=lmax, k<=i+j, i+j+k even}
//            permsix(i,j,k) h~^2(i,j,k) prod (2l+1)^{-1/3} S(i,j,k) w_i w_j w_k
//            * plijk_TTT(r,i,j,k)
// with plijk_TTT the 1/6 sum of the six q-products (orthogonalisation_late.c:620-644).
//
// Sum factorisation: with f(i,j,k) the scalar weight above,
//   B[a][b][c] = sum_i q_a(i) sum_j q_b(j) sum_k f(i,j,k) q_c(k)
//   beta_r     = (1/6) sum over the six orderings s of B[p_s1][p_s2][p_s3]
// for mode r = (p1,p2,p3).  That is O(points * P) instead of O(points * N).
// One CTA per slab l1 = i; the tetrapyd rows j are processed JC at a time:
//   phase 1: f(i,j,k) for the JC rows into shared memory (shape evaluated here)
//   phase 2: H[j][c] = sum_k f(i,j,k) q_c(k)
//   phase 3: F_i[b][c] += sum_j q_b(j) H[j][c]          (registers)
// F_i goes to a [S][L][P*P] buffer; a second pass forms B and beta.
#include <algorithm>
#include <vector>
#include <cuda_bf16.h>
#include "common.cuh"
#include "tc_ptx.cuh"

namespace modal {

__device__ __forceinline__ double d_permsix(int i, int j, int k)
{
    if (i == k && i == j) return 1.0;
    if (i == j || j == k || i == k) return 3.0;
    return 6.0;
}

// calculate_geometric (calculate_geometric.c:59-92) for a point already known
// to satisfy parity and the triangle condition.
__device__ __forceinline__ double d_geo(int l1, int l2, int l3)
{
    double s1 = l1 + l2 + l3 + 1.0, s3 = l1 + l2 + l3 + 1.0 / 3.0, s6 = l1 + l2 + l3 + 1.0 / 6.0;
    double s13 = l2 + l3 - l1 + 1.0 / 3.0, s23 = l3 + l1 - l2 + 1.0 / 3.0, s33 = l1 + l2 - l3 + 1.0 / 3.0;
    double s16 = l2 + l3 - l1 + 1.0 / 6.0, s26 = l3 + l1 - l2 + 1.0 / 6.0, s36 = l1 + l2 - l3 + 1.0 / 6.0;
    const double ipi = 0.318309886183790671537767526745028724;
    double fact = ipi * ipi / 2.0;
    double p1 = fact * ((2.0 * l1 + 1.0) * (2.0 * l2 + 1.0) * (2.0 * l3 + 1.0)) / s1;
    double p2 = s3 / (s13 * s23 * s33);
    double p3 = sqrt(s16 * s26 * s36 / s6);
    return p1 * p2 * p3;
}

// s_n(i,j,k) / (wq_i wq_j wq_k) of calculate_sijk_TTT (calculate_gamma_3d.c:813-860):
// the trapezium integral (integrate, :783-811) over x of x^2 (1/6) sum over the six
// orderings of q~(i,a) q~(j,b) q~(k,c), with the reference's rule that drops any of
// the first 10 samples above 1e-18 applied to the weighted sample.  The weights
// wq come back through the projection's point weight.
__device__ double d_radial(const RadialArgs &ra, int n, int i, int j, int k)
{
    const int a1 = ra.prim[3 * n], a2 = ra.prim[3 * n + 1], a3 = ra.prim[3 * n + 2], L1 = ra.L1;
    const double wp = ra.wq[i] * ra.wq[j] * ra.wq[k];
    double r = 0.0, yprev = 0.0;
    for (int x = 0; x < ra.xsize; x++) {
        const double *qx = ra.qt + (size_t)x * ra.Pp * L1;
        const double *q1 = qx + (size_t)a1 * L1, *q2 = qx + (size_t)a2 * L1, *q3 = qx + (size_t)a3 * L1;
        const double p1 = q1[i], p2 = q2[i], p3 = q3[i], p4 = q1[j], p5 = q2[j], p6 = q3[j], p7 = q1[k], p8 = q2[k],
                     p9 = q3[k];
        const double sum = p1 * p5 * p9 + p2 * p6 * p7 + p3 * p4 * p8 + p3 * p5 * p7 + p2 * p4 * p9 + p1 * p6 * p8;
        double y = ra.x[x] * ra.x[x] * sum * (1.0 / 6.0);
        if (x < 10 && fabs(wp * y) > 1e-18) y = 0.0;
        if (x > 0) r += (ra.x[x] - ra.x[x - 1]) * (yprev + y) * 0.5;
        yprev = y;
    }
    return r;
}

// Trapezium weight of sample x: the sum over x of w_x y_x equals the reference's
// sum over intervals of (x_x - x_{x-1}) (y_{x-1} + y_x) / 2.
__device__ __forceinline__ double trap_w(const RadialArgs &ra, int x)
{
    const double lo = x >= 1 ? ra.x[x] - ra.x[x - 1] : 0.0, hi = x + 1 < ra.xsize ? ra.x[x + 1] - ra.x[x] : 0.0;
    return 0.5 * (lo + hi);
}

constexpr int RAD_X0 = 10;  // samples below this index follow the per-point zeroing rule

// The same radial shape, sum-factorised over the row.  The integrand of sample x
// is linear in q~(k, x): with the row factors
//   U[c][x] = x^2 / 6 (sum over the orderings with q~_{a_c} at k of the
//             q~(i, x) q~(j, x) products),
// y_x = sum_c U[c][x] q~_{a_c}(k, x).  The reference drops y_x for x < 10 when
// |wq_i wq_j wq_k y_x| > 1e-18; where the factorised y_x lies within 1e-10
// (relative) of that threshold, the decision is taken on y_x summed as the
// reference sums it.  tw: [X] trapezium weights; U: [3][X] for this row.
__device__ double d_radial_rows(const RadialArgs &ra, int n, int i, int j, int k, const double *U, const double *tw)
{
    const int a1 = ra.prim[3 * n], a2 = ra.prim[3 * n + 1], a3 = ra.prim[3 * n + 2], L1 = ra.L1, X = ra.xsize;
    const double wp = ra.wq[i] * ra.wq[j] * ra.wq[k];
    double r = 0.0;
    for (int x = 0; x < X; x++) {
        const double *qx = ra.qt + (size_t)x * ra.Pp * L1;
        double y = U[x] * qx[(size_t)a1 * L1 + k];
        y = fma(U[X + x], qx[(size_t)a2 * L1 + k], y);
        y = fma(U[2 * X + x], qx[(size_t)a3 * L1 + k], y);
        if (x < RAD_X0) {
            const double t = fabs(wp * y);
            bool drop = t > 1e-18;
            if (t > 1e-18 * (1.0 - 1e-10) && t < 1e-18 * (1.0 + 1e-10)) {
                const double *q1 = qx + (size_t)a1 * L1, *q2 = qx + (size_t)a2 * L1, *q3 = qx + (size_t)a3 * L1;
                const double p1 = q1[i], p2 = q2[i], p3 = q3[i], p4 = q1[j], p5 = q2[j], p6 = q3[j], p7 = q1[k],
                             p8 = q2[k], p9 = q3[k];
                const double sum =
                    p1 * p5 * p9 + p2 * p6 * p7 + p3 * p4 * p8 + p3 * p5 * p7 + p2 * p4 * p9 + p1 * p6 * p8;
                drop = fabs(wp * (ra.x[x] * ra.x[x] * sum * (1.0 / 6.0))) > 1e-18;
            }
            if (drop) continue;
        }
        r = fma(tw[x], y, r);
    }
    return r;
}

__device__ __forceinline__ double d_shape(const DShape &s, const double *__restrict__ tab, int stride, int i, int j, int k,
                                          const RadialArgs &ra)
{
    if (s.kind == SHAPE_RADIAL) return d_radial(ra, s.nterms, i, j, k);
    if (s.kind == MODAL_SHAPE_SEPARABLE) {
        double acc = 0.0;
        for (int t = 0; t < s.nterms; t++) {
            const double *f = tab + s.tab_off + (long)t * 3 * stride;
            const double *g = f + stride, *h = g + stride;
            double v = f[i] * g[j] * h[k] + f[i] * g[k] * h[j] + f[j] * g[i] * h[k] + f[j] * g[k] * h[i] +
                       f[k] * g[i] * h[j] + f[k] * g[j] * h[i];
            acc += v / 6.0;
        }
        return acc;
    }
    double L = (double)(i + j + k);
    double x1 = i / L - s.c1, x2 = j / L - s.c2, x3 = k / L - s.c3;
    return exp(-(x1 * x1 + x2 * x2 + x3 * x3) / (2.0 * s.sigma * s.sigma));
}

// A separable shape on a fixed row (i, j), FP64: with the row coefficients
//   c[t] = (f_t(i) g_t(j) + f_t(j) g_t(i), f_t(i) h_t(j) + f_t(j) h_t(i), g_t(i) h_t(j) + g_t(j) h_t(i))
// the value at k is (1/6) sum_t (c0 h_t(k) + c1 g_t(k) + c2 f_t(k)): three loads
// and three FMAs per term instead of the six-ordering sum.
constexpr int PJ_TCOEF64 = 8;  // terms per shape with row coefficients (more: d_shape)

__device__ __forceinline__ double d_sep_rows(const DShape &s, const double *__restrict__ tab, int stride, int k,
                                             const double *c)
{
    double acc = 0.0;
    for (int t = 0; t < s.nterms; t++) {
        const double *f = tab + s.tab_off + (long)t * 3 * stride;
        acc = fma(c[3 * t], f[2 * stride + k], acc);
        acc = fma(c[3 * t + 1], f[stride + k], acc);
        acc = fma(c[3 * t + 2], f[k], acc);
    }
    return acc * (1.0 / 6.0);
}

// v_l = (2l+1)^{-1/3} w_l, w_l = (2l+1)^{1/6}/sqrt(C_l + N_l/b_l^2), w_0 = w_1 = 0
// (calculate_mode_3D.c:53-62, get_weight :283-290).
__global__ void k_vl(int lmax, const double *__restrict__ cl, double *__restrict__ vl)
{
    int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l > lmax) return;
    vl[l] = (l < 2) ? 0.0 : pow(2.0 * l + 1.0, -1.0 / 3.0) * (pow(2.0 * l + 1.0, 1.0 / 6.0) / sqrt(cl[l]));
}

constexpr int JC = 8;

__host__ __device__ inline long long tet_tri_sum(long long u)
{
    // sum_{v=0}^{u} (floor(v/2) + 1): (a+1)^2 for u = 2a, (a+1)(a+2) for u = 2a+1
    if (u < 0) return 0;
    const long long a = u / 2;
    return (u & 1) ? (a + 1) * (a + 2) : (a + 1) * (a + 1);
}

// Points of rows i..j-1 of slab i (rows hold k = j + (i & 1) + 2m <= min(i + j, lmax)).
__host__ __device__ inline long long tet_row_offset(int i, int j, int lmax)
{
    const int ip = i & 1;
    const long long n1 = (i - ip) / 2 + 1;  // points of a row with i + j <= lmax
    const int J1 = lmax - i;                // last such row
    long long off = 0;
    const int e1 = (j - 1 < J1) ? j - 1 : J1;
    if (e1 >= i) off += (long long)(e1 - i + 1) * n1;
    const int s2 = (i > J1 + 1) ? i : J1 + 1;  // rows ending at k = lmax
    if (j - 1 >= s2) off += tet_tri_sum((long long)lmax - ip - s2) - tet_tri_sum((long long)lmax - ip - (j - 1) - 1);
    return off;
}

// base[s] = points of slabs lmin..lmin+s-1 (s = 0..L); one block.
__global__ void k_slab_base(int lmin, int lmax, long long *__restrict__ base)
{
    __shared__ long long part[256];
    const int L = lmax - lmin + 1, per = (L + 255) / 256, t = threadIdx.x;
    const int a = min(L, t * per), b = min(L, a + per);
    long long sum = 0;
    for (int s = a; s < b; s++) sum += tet_row_offset(lmin + s, lmax + 1, lmax);
    part[t] = sum;
    __syncthreads();
    for (int d = 1; d < 256; d <<= 1) {  // inclusive scan
        const long long v = (t >= d) ? part[t - d] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    long long run = part[t] - sum;  // exclusive
    for (int s = a; s < b; s++) {
        base[s] = run;
        run += tet_row_offset(lmin + s, lmax + 1, lmax);
    }
    if (t == 255) base[L] = part[255];
}

// FP64 form of the weight table: the same products in the same order as the
// FP64 point weight, so the projection is unchanged to the last bit.
__global__ void __launch_bounds__(256) k_weight_table_fp64(int lmin, int lmax, const double *__restrict__ vl,
                                                           const long long *__restrict__ base, double *__restrict__ Wd)
{
    const int i = lmin + blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j = i + blockIdx.y * 8 + warp;
    if (j > lmax) return;
    const int ip = i & 1, kend = min(i + j, lmax), k0 = j + ip;
    if (kend < k0) return;
    const int n = (kend - k0) / 2 + 1;
    double *row = Wd + base[blockIdx.x] + tet_row_offset(i, j, lmax);
    const double vi = vl[i], vj = vl[j];
    for (int m = lane; m < n; m += 32) {
        const int k = k0 + 2 * m;
        row[m] = d_permsix(i, j, k) * d_geo(i, j, k) * vi * vj * vl[k];
    }
}

template <int FPT>
__global__ void __launch_bounds__(256) k_project_slab_fp64(int lmin, int lmax, int P, int S, int KMAX,
                                                            const int *__restrict__ slab_order,
                                                            const double *__restrict__ q, const double *__restrict__ vl,
                                                            const DShape *__restrict__ shapes,
                                                            const double *__restrict__ tab,
                                                            const double *__restrict__ Wd,
                                                            const long long *__restrict__ sbase,
                                                            double *__restrict__ Fbuf, const RadialArgs ra)
{
    extern __shared__ double sm[];
    double *f = sm;               // [JC][KMAX]
    double *H = sm + JC * KMAX;   // [JC][P]
    double *Cf = H + JC * P;      // separable shapes: [JC][PJ_TCOEF64][3] row coefficients (d_sep_rows)
    double *V = Cf + JC * PJ_TCOEF64 * 3;  // radial shapes: [JC][3][X] row factors, then [X] trapezium weights
    const int XR = ra.xsize;
    double *TW = V + (size_t)JC * 3 * XR;
    const int slab = slab_order[blockIdx.x];
    const int i = lmin + slab;
    const int tid = threadIdx.x;
    const int PP = P * P, L = lmax - lmin + 1, stride = lmax + 1;
    const int par = i & 1;
    for (int s = 0; s < S; s++) {
        const DShape sh = shapes[s];
        double Facc[FPT];
#pragma unroll
        for (int t = 0; t < FPT; t++) Facc[t] = 0.0;
        const bool radial = sh.kind == SHAPE_RADIAL;
        const bool rowc = sh.kind == MODAL_SHAPE_SEPARABLE && sh.nterms <= PJ_TCOEF64;
        for (int j0 = i; j0 <= lmax; j0 += JC) {
            if (rowc) {
                for (int e = tid; e < JC * sh.nterms; e += 256) {
                    const int jj = e / sh.nterms, t = e - jj * sh.nterms, j = min(j0 + jj, lmax);
                    const double *f = tab + sh.tab_off + (long)t * 3 * stride, *g = f + stride, *h = g + stride;
                    double *c = Cf + ((size_t)jj * PJ_TCOEF64 + t) * 3;
                    c[0] = f[i] * g[j] + f[j] * g[i];  // with h(k)
                    c[1] = f[i] * h[j] + f[j] * h[i];  // with g(k)
                    c[2] = g[i] * h[j] + g[j] * h[i];  // with f(k)
                }
                __syncthreads();
            }
            if (radial) {
                const int a1 = ra.prim[3 * sh.nterms], a2 = ra.prim[3 * sh.nterms + 1], a3 = ra.prim[3 * sh.nterms + 2];
                for (int e = tid; e < JC * XR; e += 256) {
                    const int jj = e / XR, x = e - jj * XR, j = min(j0 + jj, lmax);
                    const double *qx = ra.qt + (size_t)x * ra.Pp * ra.L1;
                    const double p1 = qx[(size_t)a1 * ra.L1 + i], p2 = qx[(size_t)a2 * ra.L1 + i],
                                 p3 = qx[(size_t)a3 * ra.L1 + i], p4 = qx[(size_t)a1 * ra.L1 + j],
                                 p5 = qx[(size_t)a2 * ra.L1 + j], p6 = qx[(size_t)a3 * ra.L1 + j];
                    const double g = ra.x[x] * ra.x[x] * (1.0 / 6.0);
                    double *u = V + (size_t)jj * 3 * XR;
                    u[x] = g * (p2 * p6 + p3 * p5);           // with q~_{a1}(k)
                    u[XR + x] = g * (p3 * p4 + p1 * p6);      // with q~_{a2}(k)
                    u[2 * XR + x] = g * (p1 * p5 + p2 * p4);  // with q~_{a3}(k)
                }
                for (int x = tid; x < XR; x += 256) TW[x] = trap_w(ra, x);
                __syncthreads();
            }
            for (int e = tid; e < JC * KMAX; e += 256) {
                int jj = e / KMAX, kk = e - jj * KMAX, j = j0 + jj;
                double val = 0.0;
                if (j <= lmax) {
                    int k = j + par + 2 * kk, k1 = min(i + j, lmax);
                    if (k <= k1)
                        val = Wd[sbase[slab] + tet_row_offset(i, j, lmax) + kk] *
                              (radial ? d_radial_rows(ra, sh.nterms, i, j, k, V + (size_t)jj * 3 * XR, TW)
                               : rowc ? d_sep_rows(sh, tab, stride, k, Cf + (size_t)jj * PJ_TCOEF64 * 3)
                                      : d_shape(sh, tab, stride, i, j, k, ra));
                }
                f[e] = val;
            }
            __syncthreads();
            for (int e = tid; e < JC * P; e += 256) {
                int jj = e / P, c = e - jj * P, j = j0 + jj;
                double acc = 0.0;
                if (j <= lmax) {
                    int kf = j + par, k1 = min(i + j, lmax);
                    int nk = (k1 >= kf) ? (k1 - kf) / 2 + 1 : 0;
                    const double *fr = f + jj * KMAX;
                    const double *qc = q + (size_t)(kf - lmin) * P + c;
                    for (int kk = 0; kk < nk; kk++) acc = fma(fr[kk], qc[(size_t)2 * kk * P], acc);
                }
                H[e] = acc;
            }
            __syncthreads();
#pragma unroll
            for (int t = 0; t < FPT; t++) {
                int e = tid + 256 * t;
                if (e < PP) {
                    int b = e / P, c = e - b * P;
                    double a = 0.0;
                    for (int jj = 0; jj < JC; jj++) {
                        int j = j0 + jj;
                        if (j <= lmax) a = fma(q[(size_t)(j - lmin) * P + b], H[jj * P + c], a);
                    }
                    Facc[t] += a;
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int t = 0; t < FPT; t++) {
            int e = tid + 256 * t;
            if (e < PP) Fbuf[((size_t)s * L + slab) * PP + e] = Facc[t];
        }
    }
}

// B[s][a][bc] = sum_slab q[slab][a] Fbuf[s][slab][bc]
__global__ void k_project_B(int L, int P, int S, const double *__restrict__ q, const double *__restrict__ Fbuf,
                            double *__restrict__ B)
{
    const int PP = P * P;
    size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)S * P * PP) return;
    int s = (int)(e / ((size_t)P * PP));
    int rem = (int)(e - (size_t)s * P * PP);
    int a = rem / PP, bc = rem - a * PP;
    const double *F = Fbuf + (size_t)s * L * PP + bc;
    double acc = 0.0;
    for (int l = 0; l < L; l++) acc = fma(q[(size_t)l * P + a], F[(size_t)l * PP], acc);
    B[e] = acc;
}

// beta[s][r] = (1/6) sum of B over the six orderings of mode r's triple
__global__ void k_project_beta(int N, int P, int S, const int *__restrict__ triples, const double *__restrict__ B,
                               double *__restrict__ beta)
{
    size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)S * N) return;
    int s = (int)(e / N), r = (int)(e % N);
    int p1 = triples[3 * r], p2 = triples[3 * r + 1], p3 = triples[3 * r + 2];
    const double *b = B + (size_t)s * P * P * P;
#define BB(x, y, z) b[((size_t)(x) * P + (y)) * P + (z)]
    double v = BB(p1, p2, p3) + BB(p2, p3, p1) + BB(p3, p1, p2) + BB(p3, p2, p1) + BB(p2, p1, p3) + BB(p1, p3, p2);
#undef BB
    beta[e] = v / 6e0;
}


// ---------------------------------------------------------------------------
// Split-precision (FP32) form of the slab kernel, for many shapes per launch.
// Same sum factorisation; FP32 products with compensated (Kahan) FP32
// accumulation, because GB300's FP64 rate is 1/64 of FP32.
//   grid (slab, shape group of SG shapes), 8 warps; each warp takes two
//   tetrapyd rows j and j+2 (same k parity, overlapping k windows, so each
//   q_c(k) load serves both rows and all SG shapes); lanes own c.
//   Per 32-point block a lane evaluates h~^2 once and the SG shapes, the warp
//   then accumulates H_s[j][c] in FP32 and folds each block into a Kahan sum.
//   The 16 rows' H go through shared memory into F_s[b][c] (Kahan pairs in
//   shared memory); F_i is written in FP32 for the reduction over slabs.
// ---------------------------------------------------------------------------
struct FShape {
    int kind, nterms;
    long tab_off;
    float ch[3], cl[3];  // bump centre as hi + lo float pairs
    float inv2s2;
};

__device__ __forceinline__ void kahan_add(float &hi, float &lo, float x)
{
    float y = x - lo;
    float t = hi + y;
    lo = (t - hi) - y;
    hi = t;
}

__device__ __forceinline__ float geo_f(int l1, int l2, int l3)
{
    const float L3 = (float)(l1 + l2 + l3);
    const float a1 = (float)(l2 + l3 - l1), a2 = (float)(l3 + l1 - l2), a3 = (float)(l1 + l2 - l3);
    const float third = 1.f / 3.f, sixth = 1.f / 6.f;
    const float fact = 0.0506605918211689f;  // 1/(2 pi^2)
    float p1 = fact * ((2.f * l1 + 1.f) * (2.f * l2 + 1.f) * (2.f * l3 + 1.f)) / (L3 + 1.f);
    float p2 = (L3 + third) / ((a1 + third) * (a2 + third) * (a3 + third));
    float p3 = sqrtf((a1 + sixth) * (a2 + sixth) * (a3 + sixth) / (L3 + sixth));
    return p1 * p2 * p3;
}

__device__ __forceinline__ float permsix_f(int i, int j, int k)
{
    return (i == k && i == j) ? 1.f : ((i == j || j == k || i == k) ? 3.f : 6.f);
}

// ---------------------------------------------------------------------------
// The FP32 weight table.  The per-point weight of the projection,
//   W(i,j,k) = permsix(i,j,k) h~^2 geometric factor v_i v_j v_k,
// depends on neither the shape nor the basis.  The FP32 form computes it once
// per projection into an HBM table in walk order (slab i, row j >= i, then
// k = j + (i & 1) + 2m, m = 0..), so that every shape group streams it instead
// of recomputing the geometric factor (three divisions and a square root) per
// point.  Row offsets within a slab have a closed form; slab bases are a
// prefix sum over slabs.
// ---------------------------------------------------------------------------
// grid (L slabs, ceil(L / 8)); warp w of block y fills row j = i + 8 y + w.
__global__ void __launch_bounds__(256) k_weight_table(int lmin, int lmax, const float *__restrict__ vlf,
                                                      const long long *__restrict__ base, float *__restrict__ Wt)
{
    const int i = lmin + blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j = i + blockIdx.y * 8 + warp;
    if (j > lmax) return;
    const int ip = i & 1, kend = min(i + j, lmax), k0 = j + ip;
    if (kend < k0) return;
    const int n = (kend - k0) / 2 + 1;
    float *row = Wt + base[blockIdx.x] + tet_row_offset(i, j, lmax);
    const float vij = vlf[i] * vlf[j];
    for (int m = lane; m < n; m += 32) {
        const int k = k0 + 2 * m;
        row[m] = permsix_f(i, j, k) * geo_f(i, j, k) * vij * vlf[k];
    }
}

// FP32 separable tables, per shape: [parity of l][l / 2][term][f_t, g_t, h_t, 0]
// with H = (lmax + 2) / 2 entries per parity.  The k walk of a row keeps one
// parity, so a warp's lanes read consecutive 16-byte entries: one load per term
// gives f, g and h at k.
__device__ __forceinline__ float4 tab4(const FShape &s, const float *__restrict__ tab, int H, int t, int l)
{
    return __ldg(reinterpret_cast<const float4 *>(tab + s.tab_off) + ((long)((l & 1) * H + (l >> 1)) * s.nterms + t));
}

__device__ __forceinline__ float shape_f(const FShape &s, const float *__restrict__ tab, int H, int i, int j, int k)
{
    if (s.kind == MODAL_SHAPE_SEPARABLE) {
        float acc = 0.f;
        for (int t = 0; t < s.nterms; t++) {
            const float4 Ti = tab4(s, tab, H, t, i), Tj = tab4(s, tab, H, t, j), Tk = tab4(s, tab, H, t, k);
            float fi = Ti.x, fj = Tj.x, fk = Tk.x, gi = Ti.y, gj = Tj.y, gk = Tk.y, hi = Ti.z, hj = Tj.z, hk = Tk.z;
            acc += (fi * (gj * hk + gk * hj) + fj * (gi * hk + gk * hi) + fk * (gi * hj + gj * hi)) * (1.f / 6.f);
        }
        return acc;
    }
    // Gaussian bump: exp(-|(l1,l2,l3)/L - c|^2 / (2 sigma^2)).  l_m/L - c_m is
    // formed as (l_m - c_m L)/L with c_m = hi + lo and the exact FMA residual of
    // hi*L, so it is accurate relative to itself: the exponent (up to ~200 |x|^2
    // for sigma = 0.05) then keeps ~1e-7 relative accuracy in FP32.
    const float L = (float)(i + j + k), invL = 1.f / L;
    const float l3[3] = {(float)i, (float)j, (float)k};
    float a = 0.f;
#pragma unroll
    for (int m = 0; m < 3; m++) {
        const float p = s.ch[m] * L;
        const float e = fmaf(s.ch[m], L, -p);
        const float d = (((l3[m] - p) - e) - s.cl[m] * L) * invL;
        a = fmaf(d, d, a);
    }
    return expf(-a * s.inv2s2);
}

// A separable shape on a fixed row (i, j): sym sum_t f_t g_t h_t at (i, j, k) is
//   sum_t (al_t h_t(k) + be_t g_t(k) + ga_t f_t(k)) / 6,
//   al_t = f_t(i) g_t(j) + f_t(j) g_t(i), be_t = f_t(i) h_t(j) + f_t(j) h_t(i),
//   ga_t = g_t(i) h_t(j) + g_t(j) h_t(i),
// so the per-point work is three table reads and three FMAs per term.
constexpr int PJ_TCOEF = 4;  // terms per shape with precomputed row coefficients (more: shape_f)

__device__ __forceinline__ float3 sep_row_coef(const FShape &s, const float *__restrict__ tab, int H, int t, int i, int j)
{
    const float4 Ti = tab4(s, tab, H, t, i), Tj = tab4(s, tab, H, t, j);
    const float fi = Ti.x, fj = Tj.x, gi = Ti.y, gj = Tj.y, hi = Ti.z, hj = Tj.z;
    return make_float3(fi * gj + fj * gi, fi * hj + fj * hi, gi * hj + gj * hi);
}

// FP32 tables of the separable shapes, re-laid from the FP64 [term][f, g, h][l]
// tables; grid (ceil((lmax + 1) max_nterms / 256), S).
__global__ void k_tab_f32(int lmax, const DShape *__restrict__ shapes, const double *__restrict__ tab64,
                          float *__restrict__ tabf)
{
    const DShape d = shapes[blockIdx.y];
    if (d.kind != MODAL_SHAPE_SEPARABLE) return;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int l = e / d.nterms, t = e - l * d.nterms;
    if (l > lmax) return;
    const int stride = lmax + 1, H = (lmax + 2) / 2;
    const double *f = tab64 + d.tab_off + (long)t * 3 * stride;
    float4 v = make_float4((float)f[l], (float)f[stride + l], (float)f[2 * stride + l], 0.f);
    reinterpret_cast<float4 *>(tabf + d.tab_off_f)[(long)((l & 1) * H + (l >> 1)) * d.nterms + t] = v;
}

// Work item w = (slab rank w / G, shape group w % G), slabs heaviest first.
// counter == NULL: one item per CTA of a (L x G) grid.  counter != NULL: a
// persistent grid whose CTAs take items from *counter until nitems are done.
template <int SG, int CPL>
__global__ void __launch_bounds__(256, 2) k_project_slab_f32(int lmin, int lmax, int P, int S, int G, int nitems,
                                                           int *__restrict__ counter,
                                                           const int *__restrict__ slab_order,
                                                           const float *__restrict__ qf, const float *__restrict__ vlf,
                                                           const FShape *__restrict__ shapes,
                                                           const float *__restrict__ tabf,
                                                           const float *__restrict__ Wt,
                                                           const long long *__restrict__ sbase,
                                                           float *__restrict__ Fbuf)
{
    constexpr int JC = 16, CW = 32 * CPL;
    static_assert(SG % 4 == 0, "shape groups are read as float4");
    __shared__ float4 fsm[8][2][32][SG / 4];  // shape values per (warp, row, k, shape)
    __shared__ __align__(16) float Hs[JC][SG][CW];
    __shared__ __align__(16) float Qs[JC][CW];  // q_b(j) of the chunk's rows, zero beyond P and lmax
    __shared__ FShape sh[SG];
    __shared__ float4 coef[8][2][SG][PJ_TCOEF];  // row coefficients of separable shapes per (warp, row), one 16-byte load
    __shared__ int item;
    // F_i as Kahan pairs, element-major over the fold's 4 x 4 tiles: entry (4x + y) of
    // tile t at [(4x + y) NT + t], so the threads of a warp (consecutive tiles) touch
    // consecutive words.  NT = SG nb4^2 tiles, nb4 = ceil(P / 4); hi, then lo.
    extern __shared__ float Fsm[];
    for (int pass = 0;; pass++) {
    int w;
    if (counter) {
        __syncthreads();  // the previous item's last reads of Fsm are done
        if (threadIdx.x == 0) item = atomicAdd(counter, 1);
        __syncthreads();
        w = item;
        if (w >= nitems) return;
    } else {
        if (pass > 0) return;
        w = blockIdx.x * G + blockIdx.y;
    }
    const int slab = slab_order[w / G];
    const int i = lmin + slab;
    const int s0 = (w % G) * SG;
    const int sgv = min(SG, S - s0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int par = i & 1, PP = P * P, L = lmax - lmin + 1, H = (lmax + 2) / 2;
    if (threadIdx.x < SG) {
        FShape z = {1, 0, 0, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, 0.f};
        sh[threadIdx.x] = (threadIdx.x < sgv) ? shapes[s0 + threadIdx.x] : z;
    }
    const int nb4 = (P + 3) >> 2, NT = SG * nb4 * nb4;
    float *Fhi = Fsm, *Flo = Fsm + 16 * NT;
    for (int e = threadIdx.x; e < 32 * NT; e += 256) Fsm[e] = 0.f;
    __syncthreads();
    const int jo = (warp >> 1) * 4 + (warp & 1);  // rows jo and jo+2 of each chunk

    for (int j0 = i; j0 <= lmax; j0 += JC) {
        const int jA = j0 + jo, jB = jA + 2;
        float HAh[SG][CPL], HAl[SG][CPL], HBh[SG][CPL], HBl[SG][CPL];
#pragma unroll
        for (int s = 0; s < SG; s++)
#pragma unroll
            for (int cc = 0; cc < CPL; cc++) HAh[s][cc] = HAl[s][cc] = HBh[s][cc] = HBl[s][cc] = 0.f;
        if (jA <= lmax) {
            const bool hasB = jB <= lmax;
            const int kstart = jA + par;
            const int kendA = min(i + jA, lmax), kendB = hasB ? min(i + jB, lmax) : -1;
            const int kend = max(kendA, kendB);
            const int nk = (kend >= kstart) ? (kend - kstart) / 2 + 1 : 0;
            // this warp's two rows in the weight table (row B starts one lattice point later)
            const float *wA = Wt + sbase[slab] + tet_row_offset(i, jA, lmax);
            const float *wB = hasB ? Wt + sbase[slab] + tet_row_offset(i, jB, lmax) - 1 : wA;
            for (int e = lane; e < 2 * SG * PJ_TCOEF; e += 32) {
                const int row = e / (SG * PJ_TCOEF), rem = e - row * (SG * PJ_TCOEF);
                const int sx = rem / PJ_TCOEF, t = rem - sx * PJ_TCOEF;
                const int j = row ? jB : jA;
                float3 cv = make_float3(0.f, 0.f, 0.f);
                if (sx < sgv && sh[sx].kind == MODAL_SHAPE_SEPARABLE && t < sh[sx].nterms && j <= lmax)
                    cv = sep_row_coef(sh[sx], tabf, H, t, i, j);
                coef[warp][row][sx][t] = make_float4(cv.x, cv.y, cv.z, 0.f);
            }
            __syncwarp();
            for (int kb = 0; kb < nk; kb += 32) {
                const int kk = kb + lane, k = kstart + 2 * kk;
                float fa[SG], fb2[SG];
#pragma unroll
                for (int s = 0; s < SG; s++) fa[s] = fb2[s] = 0.f;
                if (kk < nk) {
                    // both rows share k: one table load per term serves the two
                    const bool inA = k <= kendA, inB = hasB && k >= jB + par && k <= kendB;
                    const float gA = inA ? wA[kk] : 0.f, gB = inB ? wB[kk] : 0.f;
#pragma unroll
                    for (int s = 0; s < SG; s++) {
                        if (s >= sgv) continue;
                        const FShape &sp = sh[s];
                        if (sp.kind == MODAL_SHAPE_SEPARABLE && sp.nterms <= PJ_TCOEF) {
                            float accA = 0.f, accB = 0.f;
                            for (int t = 0; t < sp.nterms; t++) {
                                const float4 T = tab4(sp, tabf, H, t, k);
                                const float4 cA = coef[warp][0][s][t], cB = coef[warp][1][s][t];
                                accA += fmaf(cA.x, T.z, fmaf(cA.y, T.y, cA.z * T.x)) * (1.f / 6.f);
                                accB += fmaf(cB.x, T.z, fmaf(cB.y, T.y, cB.z * T.x)) * (1.f / 6.f);
                            }
                            if (inA) fa[s] = gA * accA;
                            if (inB) fb2[s] = gB * accB;
                        } else {
                            if (inA) fa[s] = gA * shape_f(sp, tabf, H, i, jA, k);
                            if (inB) fb2[s] = gB * shape_f(sp, tabf, H, i, jB, k);
                        }
                    }
                }
#pragma unroll
                for (int s4 = 0; s4 < SG / 4; s4++) {
                    fsm[warp][0][lane][s4] = make_float4(fa[4 * s4], fa[4 * s4 + 1], fa[4 * s4 + 2], fa[4 * s4 + 3]);
                    fsm[warp][1][lane][s4] = make_float4(fb2[4 * s4], fb2[4 * s4 + 1], fb2[4 * s4 + 2], fb2[4 * s4 + 3]);
                }
                __syncwarp();
                const int nt = min(32, nk - kb);
                float hA[SG][CPL], hB[SG][CPL];
#pragma unroll
                for (int s = 0; s < SG; s++)
#pragma unroll
                    for (int cc = 0; cc < CPL; cc++) hA[s][cc] = hB[s][cc] = 0.f;
#pragma unroll 8
                for (int t = 0; t < nt; t++) {
                    const int kt = kstart + 2 * (kb + t);
                    const float *qrow = qf + (size_t)(kt - lmin) * P;
                    float qv[CPL];
#pragma unroll
                    for (int cc = 0; cc < CPL; cc++) qv[cc] = (lane + 32 * cc < P) ? qrow[lane + 32 * cc] : 0.f;
#pragma unroll
                    for (int s4 = 0; s4 < SG / 4; s4++) {
                        const float4 a4 = fsm[warp][0][t][s4], b4 = fsm[warp][1][t][s4];
                        const float av[4] = {a4.x, a4.y, a4.z, a4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
                        for (int u = 0; u < 4; u++)
#pragma unroll
                            for (int cc = 0; cc < CPL; cc++) {
                                hA[4 * s4 + u][cc] = fmaf(av[u], qv[cc], hA[4 * s4 + u][cc]);
                                hB[4 * s4 + u][cc] = fmaf(bv[u], qv[cc], hB[4 * s4 + u][cc]);
                            }
                    }
                }
#pragma unroll
                for (int s = 0; s < SG; s++)
#pragma unroll
                    for (int cc = 0; cc < CPL; cc++) {
                        kahan_add(HAh[s][cc], HAl[s][cc], hA[s][cc]);
                        kahan_add(HBh[s][cc], HBl[s][cc], hB[s][cc]);
                    }
                __syncwarp();
            }
        }
#pragma unroll
        for (int s = 0; s < SG; s++)
#pragma unroll
            for (int cc = 0; cc < CPL; cc++) {
                Hs[jo][s][lane + 32 * cc] = HAh[s][cc] + HAl[s][cc];
                Hs[jo + 2][s][lane + 32 * cc] = HBh[s][cc] + HBl[s][cc];
            }
        for (int e = threadIdx.x; e < JC * CW; e += 256) {
            const int r = e / CW, b = e - r * CW, j = j0 + r;
            Qs[r][b] = (j <= lmax && b < P) ? qf[(size_t)(j - lmin) * P + b] : 0.f;
        }
        __syncthreads();
        // F_s[b][c] += sum_r q_b(j0+r) H_s[r][c] as 4 x 4 register tiles (two
        // vector loads per 16 FMAs), then one compensated add per element
        {
            const int ntile = sgv * nb4 * nb4;
            for (int ti = threadIdx.x; ti < ntile; ti += 256) {
                const int sx = ti / (nb4 * nb4), rem = ti - sx * nb4 * nb4, bt = rem / nb4, ct = rem - bt * nb4;
                float acc[4][4];
#pragma unroll
                for (int x = 0; x < 4; x++)
#pragma unroll
                    for (int y = 0; y < 4; y++) acc[x][y] = 0.f;
#pragma unroll 16
                for (int r = 0; r < JC; r++) {
                    const float4 qv = *reinterpret_cast<const float4 *>(&Qs[r][bt * 4]);
                    const float4 hv = *reinterpret_cast<const float4 *>(&Hs[r][sx][ct * 4]);
                    const float qa[4] = {qv.x, qv.y, qv.z, qv.w}, ha[4] = {hv.x, hv.y, hv.z, hv.w};
#pragma unroll
                    for (int x = 0; x < 4; x++)
#pragma unroll
                        for (int y = 0; y < 4; y++) acc[x][y] = fmaf(qa[x], ha[y], acc[x][y]);
                }
#pragma unroll
                for (int x = 0; x < 4; x++)
#pragma unroll
                    for (int y = 0; y < 4; y++) {
                        const int b = bt * 4 + x, c = ct * 4 + y;
                        if (b < P && c < P) {
                            const int e = (4 * x + y) * NT + ti;
                            kahan_add(Fhi[e], Flo[e], acc[x][y]);
                        }
                    }
            }
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < sgv * PP; e += 256) {
        const int s = e / PP, rem = e - s * PP, b = rem / P, c = rem - b * P;
        const int f = (4 * (b & 3) + (c & 3)) * NT + (s * nb4 + (b >> 2)) * nb4 + (c >> 2);
        Fbuf[((size_t)(s0 + s) * L + slab) * PP + rem] = Fhi[f] + Flo[f];
    }
    }
}

// ---------------------------------------------------------------------------
// Tensor-core form of the FP32 slab projection (P <= 32).
//
// The two contractions of slab i,
//   H_s[j][c] = sum_k f_s(i,j,k) q_c(k)        over the points of row j,
//   F_s[b][c] += sum_j q_b(j) H_s[j][c]        over the rows,
// are split between the tensor cores and the CUDA cores.  The first (about 85%
// of the arithmetic) runs as tcgen05 MMAs with M = 128 rows (4 shapes x 32
// rows of one parity), N = 32 basis columns and K = 16 per step; the second
// stays on CUDA cores, once per block of 32 rows, as in k_project_slab_f32.
//
// Operands.  Row j of slab i holds k = j + (i & 1) + 2m, so every k of a row
// has the parity of i + j; a block of 32 rows j = jb, jb + 2, ... shares it.
// In compact coordinates m = k >> 1 row j starts one step after row j - 2: the
// block is a band, walked in chunks of 32 m (64 bytes of BF16 per row), with
// zeros outside each row's band.  Each value f = W(i,j,k) S_s(i,j,k) (FP32,
// evaluated by the thread that owns the row) is split exactly into three BF16
// pieces f1 + f2 + f3 (8 significant bits each; BF16 keeps the FP32 exponent
// range, so nothing is scaled), and q_c(k) likewise from FP64.  The six
// products fa qb with a + b <= 4 (pieces numbered from 1) carry each product to
// about 2^-24 relative, the precision of the FP32 product of the CUDA-core
// kernel; products of BF16 pieces are exact in FP32.
//
// Accumulation.  Each chunk's 12 MMAs (2 K-steps x 6 products) write a fresh
// FP32 accumulator in tensor memory (two, alternating), which the row's thread
// reads back (tcgen05.ld) and adds into its H row as a Kahan pair, as the
// CUDA-core kernel does per 32-point block.
//
// Roles: warps 0-3 own tensor-memory lanes 0-127 (thread = lane = A row): they
// evaluate the A rows, stage the B tile, drain the accumulator and run the
// fold.  Warp 4 allocates tensor memory and one of its threads issues the MMAs.
// Hand-off per buffer: `ready` (128 arrivals) and `done` (tcgen05.commit).
// Every wait is bounded; a timeout sets *err and ends the kernel.
// ---------------------------------------------------------------------------
constexpr int PT_SG = 4, PT_JR = 32;
constexpr int PT_A_PIECE = 128 * 64, PT_B_PIECE = 32 * 64;
constexpr int PT_BUF = 3 * PT_A_PIECE + 3 * PT_B_PIECE;  // 30 KB per buffer
constexpr int PT_HS_LD = 36;                             // floats per staged H row (16-byte aligned, conflict-free)
constexpr int PT_OFF_QS = 2 * PT_BUF;                    // q_b(j) of the block's rows, [32][32] floats
constexpr int PT_OFF_F = PT_OFF_QS + 32 * 32 * 4;        // F Kahan pairs, [hi|lo][32][128] floats
constexpr int PT_OFF_BAR = PT_OFF_F + 2 * 32 * 128 * 4;
constexpr int PT_SMEM = PT_OFF_BAR + 128 + 1024;         // barriers and flags, 1 KB alignment slack
constexpr uint32_t PT_TMEM_COLS = 64;
constexpr long long PT_WAIT = 2000000000LL;              // clock64 cycles, about 1 s
// kind::f16 instruction descriptor with A = B = BF16, D = F32, both K-major
constexpr uint32_t PT_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(32 >> 3) << 17) |
                              ((uint32_t)(128 >> 4) << 24);
static_assert(PT_BUF % 1024 == 0 && PT_OFF_QS % 1024 == 0, "swizzled tiles need 1 KB alignment");
static_assert(128 * PT_HS_LD * 4 <= 2 * PT_BUF, "H staging aliases the operand buffers");

// v0 -> low half, v1 -> high half: v = w1 + w2 + w3 exactly (three BF16 pieces).
__device__ __forceinline__ void bf16_split3(float v0, float v1, uint32_t &w1, uint32_t &w2, uint32_t &w3)
{
    const __nv_bfloat162 p1 = __floats2bfloat162_rn(v0, v1);
    const float r0 = v0 - __low2float(p1), r1 = v1 - __high2float(p1);
    const __nv_bfloat162 p2 = __floats2bfloat162_rn(r0, r1);
    const __nv_bfloat162 p3 = __floats2bfloat162_rn(r0 - __low2float(p2), r1 - __high2float(p2));
    w1 = *reinterpret_cast<const uint32_t *>(&p1);
    w2 = *reinterpret_cast<const uint32_t *>(&p2);
    w3 = *reinterpret_cast<const uint32_t *>(&p3);
}

// Barrier 1 over the 128 threads of warps 0-3; returns the OR of `v` over them.
__device__ __forceinline__ bool pt_bar_or(bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, 1, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v)
        : "memory");
    return r != 0;
}

// q_c(k) as three BF16 pieces, K-major per (k parity, piece):
// Bq[((par * 3 + piece) * 32 + c) * Mpad + m] = piece of q_c(2m + par), zero for
// k outside [lmin, lmax] and for c >= P.  The pieces are taken from FP64.
__global__ void k_bq_pieces(int lmin, int lmax, int P, int Mpad, const double *__restrict__ q,
                            __nv_bfloat16 *__restrict__ Bq)
{
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 64L * Mpad) return;
    const int m = (int)(e % Mpad), c = (int)((e / Mpad) % 32), par = (int)(e / (32L * Mpad));
    const int k = 2 * m + par;
    double v = (k >= lmin && k <= lmax && c < P) ? q[(size_t)(k - lmin) * P + c] : 0.0;
    const size_t plane = (size_t)32 * Mpad, at = (size_t)c * Mpad + m;
    for (int pc = 0; pc < 3; pc++) {
        const __nv_bfloat16 h = __double2bfloat16(v);
        Bq[((size_t)par * 3 + pc) * plane + at] = h;
        v -= (double)__bfloat162float(h);
    }
}

// Work item w = (slab rank w / G, group of 4 shapes w % G) from *counter; the
// shapes of group g are shapes[perm[4g .. 4g+3]] (sorted by kind and term count
// so a warp's four shapes take the same path).  Fbuf as k_project_slab_f32.
__global__ void __maxnreg__(200) k_project_slab_tc(int lmin, int lmax, int P, int S, int G, int nitems,
                                                            int *__restrict__ counter,
                                                            const int *__restrict__ slab_order,
                                                            const int *__restrict__ perm,
                                                            const float *__restrict__ qf,
                                                            const __nv_bfloat16 *__restrict__ Bq, int Mpad,
                                                            const FShape *__restrict__ shapes,
                                                            const float *__restrict__ tabf,
                                                            const float *__restrict__ Wt,
                                                            const long long *__restrict__ sbase,
                                                            float *__restrict__ Fbuf, int *__restrict__ err)
{
    using namespace tc;
    extern __shared__ uint8_t pt_raw[];
    uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(pt_raw) + 1023) & ~(uintptr_t)1023);
    float *Qs = reinterpret_cast<float *>(sm + PT_OFF_QS);
    float *Fs = reinterpret_cast<float *>(sm + PT_OFF_F);
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + PT_OFF_BAR);
    uint64_t *ready = bars, *done = bars + 2;
    volatile int *cmd = reinterpret_cast<volatile int *>(bars + 4);  // per buffer: 1 = chunk, 0 = exit
    volatile int *abort_flag = cmd + 2;
    volatile int *item_slot = cmd + 3;
    volatile uint32_t *tmem_slot = reinterpret_cast<volatile uint32_t *>(cmd + 4);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int b = 0; b < 2; b++) {
            mbar_init(smem_u32(&ready[b]), 128);
            mbar_init(smem_u32(&done[b]), 1);
        }
        cmd[0] = cmd[1] = 0;
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 4) {
        tmem_alloc(smem_u32((const void *)tmem_slot), PT_TMEM_COLS);
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 4) {
        if (lane == 0) {
            long u = 0;
            for (;; u++) {
                const int b = (int)(u & 1);
                if (!mbar_wait(smem_u32(&ready[b]), (uint32_t)((u >> 1) & 1), abort_flag, PT_WAIT)) {
                    if (!*abort_flag) { *abort_flag = 1; atomicCAS(err, 0, 21); }
                    break;
                }
                tc_fence_after();
                if (cmd[b] == 0) break;
                const uint32_t a0 = smem_u32(sm + b * PT_BUF), b0 = a0 + 3 * PT_A_PIECE;
                const uint32_t d = tmem + (uint32_t)(32 * b);
                // A piece a with B piece b, a + b <= 2 (from 0), smallest products first
                const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
                for (int ks = 0; ks < 2; ks++)
#pragma unroll
                    for (int p = 0; p < 6; p++)
                        umma_f16(d, desc_sw64(a0 + pa[p] * PT_A_PIECE + ks * 32),
                                 desc_sw64(b0 + pb[p] * PT_B_PIECE + ks * 32), PT_IDESC, (ks | p) ? 1u : 0u);
                umma_commit(smem_u32(&done[b]));
            }
            // after an abort, let the last issued chunk finish before tensor memory is freed
            if (u > 0) {
                const long l = u - 1;
                const long long t0 = clock64();
                while (!mbar_try(smem_u32(&done[l & 1]), (uint32_t)((l >> 1) & 1)) && clock64() - t0 < PT_WAIT) {
                }
            }
        }
    } else {
        const int gt = threadIdx.x;  // A row = tensor-memory lane
        const uint32_t tl = (uint32_t)(32 * warp) << 16;
        const int sl = lane & 3, jr = 8 * warp + (lane >> 2);  // row gt = (shape sl, block row jr)
        const int PP = P * P, L = lmax - lmin + 1, H = (lmax + 2) / 2, swz = (gt >> 1) & 3;
        float *Fhi = Fs, *Flo = Fs + 32 * 128;
        float *Hs = reinterpret_cast<float *>(sm);  // aliases the operand buffers between blocks
        long u = 0;
        bool stop = false;
        for (;;) {
            stop = pt_bar_or(stop);
            if (stop) break;
            if (gt == 0) *item_slot = atomicAdd(counter, 1);
            pt_bar_or(false);
            const int w = *item_slot;
            if (w >= nitems) break;
            const int slab = slab_order[w / G], g = w % G, i = lmin + slab;
            const int ps = g * PT_SG + sl;
            const bool sv = ps < S;
            FShape sh = {1, 0, 0, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, 0.f};
            if (sv) sh = shapes[perm[ps]];
            for (int e = 0; e < 32; e++) Fhi[e * 128 + gt] = Flo[e * 128 + gt] = 0.f;
            for (int par = 0; par < 2 && !stop; par++) {
                const int kp = (i + par) & 1;
                for (int jb = i + ((par - i) & 1); jb <= lmax && !stop; jb += 2 * PT_JR) {
                    // the block's band in compact k: first row's start to last row's end
                    const int mlo = (jb + (i & 1) - kp) >> 1;
                    int jl = min(jb + 2 * (PT_JR - 1), lmax);
                    if ((jl - jb) & 1) jl--;
                    int kle = min(i + jl, lmax);
                    if ((kle - kp) & 1) kle--;
                    const int mhi = (kle - kp) >> 1;
                    if (mhi < mlo) continue;
                    // this thread's row
                    const int j = jb + 2 * jr;
                    int mf = 1, ml = 0;
                    long long wb = 0;
                    if (sv && j <= lmax) {
                        const int kf = j + (i & 1);
                        int kl = min(i + j, lmax);
                        if ((kl - kp) & 1) kl--;
                        if (kl >= kf) {
                            mf = (kf - kp) >> 1;
                            ml = (kl - kp) >> 1;
                            wb = sbase[slab] + tet_row_offset(i, j, lmax) - mf;
                        }
                    }
                    const bool fast = sh.kind == MODAL_SHAPE_SEPARABLE && sh.nterms <= PJ_TCOEF;
                    float4 cf[PJ_TCOEF];
#pragma unroll
                    for (int t = 0; t < PJ_TCOEF; t++) {
                        float3 c3 = make_float3(0.f, 0.f, 0.f);
                        if (fast && ml >= mf && t < sh.nterms) c3 = sep_row_coef(sh, tabf, H, t, i, j);
                        cf[t] = make_float4(c3.x * (1.f / 6.f), c3.y * (1.f / 6.f), c3.z * (1.f / 6.f), 0.f);
                    }
                    float Hh[32], Hl[32];
#pragma unroll
                    for (int c = 0; c < 32; c++) Hh[c] = Hl[c] = 0.f;
                    const int q0 = mlo >> 5, q1 = mhi >> 5;
                    for (int q = q0; q <= q1; q++, u++) {
                        const int b = (int)(u & 1);
                        uint8_t *buf = sm + b * PT_BUF;
#pragma unroll 1
                        for (int e8 = 0; e8 < 4; e8++) {
                            const int m0 = 32 * q + 8 * e8;
                            float v[8];
#pragma unroll
                            for (int x = 0; x < 8; x++) {
                                const int m = m0 + x;
                                float val = 0.f;
                                if (m >= mf && m <= ml) {
                                    const int k = 2 * m + kp;
                                    float s;
                                    if (fast) {
                                        s = 0.f;
#pragma unroll
                                        for (int t = 0; t < PJ_TCOEF; t++) {
                                            if (t < sh.nterms) {
                                                const float4 T = tab4(sh, tabf, H, t, k);
                                                s = fmaf(cf[t].x, T.z, fmaf(cf[t].y, T.y, fmaf(cf[t].z, T.x, s)));
                                            }
                                        }
                                    } else {
                                        s = shape_f(sh, tabf, H, i, j, k);
                                    }
                                    val = __ldg(Wt + wb + m) * s;
                                }
                                v[x] = val;
                            }
                            uint32_t w1[4], w2[4], w3[4];
#pragma unroll
                            for (int y = 0; y < 4; y++) bf16_split3(v[2 * y], v[2 * y + 1], w1[y], w2[y], w3[y]);
                            const int off = gt * 64 + ((e8 ^ swz) << 4);
                            *reinterpret_cast<uint4 *>(buf + off) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
                            *reinterpret_cast<uint4 *>(buf + PT_A_PIECE + off) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
                            *reinterpret_cast<uint4 *>(buf + 2 * PT_A_PIECE + off) = make_uint4(w3[0], w3[1], w3[2], w3[3]);
                        }
                        {   // B tile: piece r, row c = gt >> 2, 16-byte chunk e = gt & 3
                            const int c = gt >> 2, e = gt & 3;
#pragma unroll
                            for (int r = 0; r < 3; r++) {
                                const uint4 bv = __ldg(reinterpret_cast<const uint4 *>(
                                    Bq + ((size_t)(kp * 3 + r) * 32 + c) * Mpad + 32 * q + 8 * e));
                                *reinterpret_cast<uint4 *>(buf + 3 * PT_A_PIECE + r * PT_B_PIECE + c * 64 +
                                                           ((e ^ ((c >> 1) & 3)) << 4)) = bv;
                            }
                        }
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        tc_fence_before();
                        if (gt == 0) cmd[b] = 1;
                        mbar_arrive(smem_u32(&ready[b]));
                        // drain the chunk before this one (the last one after the loop)
                        if (q > q0 || q == q1) {
                            const long first = (q > q0) ? u - 1 : u, last = (q == q1) ? u : u - 1;
                            for (long ud = first; ud <= last; ud++) {
                                const int bd = (int)(ud & 1);
                                bool ok = mbar_wait(smem_u32(&done[bd]), (uint32_t)((ud >> 1) & 1), abort_flag, PT_WAIT);
                                ok = __all_sync(0xffffffffu, ok);
                                if (!ok) {
                                    if (!*abort_flag) { *abort_flag = 1; atomicCAS(err, 0, 22); }
                                    stop = true;
                                    break;
                                }
                                tc_fence_after();
                                uint32_t r[32];
                                tmem_ld32(tmem + tl + (uint32_t)(32 * bd), r);
                                tmem_wait_ld();
#pragma unroll
                                for (int c = 0; c < 32; c++) kahan_add(Hh[c], Hl[c], __uint_as_float(r[c]));
                            }
                            tc_fence_before();
                        }
                        if (stop) break;
                    }
                    if (pt_bar_or(stop)) { stop = true; break; }
                    // fold: F_s[b][c] += sum_jr q_b(jb + 2 jr) H[(s, jr)][c]; the operand
                    // buffers are idle (every chunk of the block has been drained)
#pragma unroll
                    for (int c4 = 0; c4 < 8; c4++)
                        *reinterpret_cast<float4 *>(Hs + gt * PT_HS_LD + 4 * c4) =
                            make_float4(Hh[4 * c4] + Hl[4 * c4], Hh[4 * c4 + 1] + Hl[4 * c4 + 1],
                                        Hh[4 * c4 + 2] + Hl[4 * c4 + 2], Hh[4 * c4 + 3] + Hl[4 * c4 + 3]);
                    {
                        const int jq = gt >> 2, b0 = 8 * (gt & 3), jj = jb + 2 * jq;
#pragma unroll
                        for (int x = 0; x < 8; x++) {
                            const int bb = b0 + x;
                            Qs[jq * 32 + bb] = (jj <= lmax && bb < P) ? qf[(size_t)(jj - lmin) * P + bb] : 0.f;
                        }
                    }
                    pt_bar_or(false);
#pragma unroll 1
                    for (int r = 0; r < 2; r++) {
                        const int tau = gt + 128 * r, s3 = tau >> 6, bt = (tau >> 3) & 7, ct = tau & 7;
                        float acc[4][4];
#pragma unroll
                        for (int x = 0; x < 4; x++)
#pragma unroll
                            for (int y = 0; y < 4; y++) acc[x][y] = 0.f;
#pragma unroll 8
                        for (int q2 = 0; q2 < PT_JR; q2++) {
                            const float4 qv = *reinterpret_cast<const float4 *>(Qs + q2 * 32 + 4 * bt);
                            const int mrow = 32 * (q2 >> 3) + 4 * (q2 & 7) + s3;
                            const float4 hv = *reinterpret_cast<const float4 *>(Hs + mrow * PT_HS_LD + 4 * ct);
                            const float qa[4] = {qv.x, qv.y, qv.z, qv.w}, ha[4] = {hv.x, hv.y, hv.z, hv.w};
#pragma unroll
                            for (int x = 0; x < 4; x++)
#pragma unroll
                                for (int y = 0; y < 4; y++) acc[x][y] = fmaf(qa[x], ha[y], acc[x][y]);
                        }
#pragma unroll
                        for (int x = 0; x < 4; x++)
#pragma unroll
                            for (int y = 0; y < 4; y++) {
                                const int e = (r * 16 + 4 * x + y) * 128 + gt;
                                kahan_add(Fhi[e], Flo[e], acc[x][y]);
                            }
                    }
                    pt_bar_or(false);  // Hs and Qs are read before the next block writes the buffers
                }
            }
            if (stop) continue;  // the loop head agrees on stopping
#pragma unroll 1
            for (int r = 0; r < 2; r++) {
                const int tau = gt + 128 * r, s3 = tau >> 6, bt = (tau >> 3) & 7, ct = tau & 7;
                const int p3 = g * PT_SG + s3;
                if (p3 >= S) continue;
                float *dst = Fbuf + ((size_t)perm[p3] * L + slab) * PP;
#pragma unroll
                for (int x = 0; x < 4; x++)
#pragma unroll
                    for (int y = 0; y < 4; y++) {
                        const int bb = 4 * bt + x, c = 4 * ct + y;
                        const int e = (r * 16 + 4 * x + y) * 128 + gt;
                        if (bb < P && c < P) dst[bb * P + c] = Fhi[e] + Flo[e];
                    }
            }
        }
        // tell the MMA thread to stop (after every issued chunk has been drained)
        if (!stop) {
            const int b = (int)(u & 1);
            if (gt == 0) cmd[b] = 0;
            mbar_arrive(smem_u32(&ready[b]));
        }
    }
    __syncthreads();
    if (warp == 4) {
        tc_fence_after();
        tmem_dealloc(tmem, PT_TMEM_COLS);
    }
}

// B[s][a][bc] = sum_slab q[slab][a] F[s][slab][bc], FP32 with Kahan compensation.
__global__ void k_project_B_f32(int L, int P, int S, const float *__restrict__ qf, const float *__restrict__ Fbuf,
                                double *__restrict__ B)
{
    const int PP = P * P;
    size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)S * P * PP) return;
    int s = (int)(e / ((size_t)P * PP));
    int rem = (int)(e - (size_t)s * P * PP);
    int a = rem / PP, bc = rem - a * PP;
    const float *F = Fbuf + (size_t)s * L * PP + bc;
    float hi = 0.f, lo = 0.f;
    for (int l = 0; l < L; l++) kahan_add(hi, lo, qf[(size_t)l * P + a] * F[(size_t)l * PP]);
    B[e] = (double)hi + (double)lo;
}

__global__ void k_d2f(long n, const double *__restrict__ in, float *__restrict__ out)
{
    long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) out[e] = (float)in[e];
}

__global__ void k_fshapes(int S, const DShape *__restrict__ in, FShape *__restrict__ out)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    DShape d = in[s];
    FShape f;
    f.kind = d.kind;
    f.nterms = d.nterms;
    f.tab_off = d.tab_off_f;
    const double c[3] = {d.c1, d.c2, d.c3};
    for (int m = 0; m < 3; m++) {
        f.ch[m] = (float)c[m];
        f.cl[m] = (float)(c[m] - (double)f.ch[m]);
    }
    f.inv2s2 = (float)(1.0 / (2.0 * d.sigma * d.sigma));
    out[s] = f;
}



// ---------------------------------------------------------------- host side
//
// A projection is planned (shapes validated, every device buffer sized, the
// slab schedule uploaded), its inputs are staged (shape tables and
// descriptors copied to the device), and its device work is recorded on the
// context stream.  The record step allocates nothing and makes no host
// round trip, so modal_project_batch can capture it into a CUDA graph.

static long slab_points(int i, int lmax)
{
    long n = 0;
    for (int j = i; j <= lmax; j++) {
        int kf = j + (i & 1), k1 = std::min(i + j, lmax);
        if (k1 >= kf) n += (k1 - kf) / 2 + 1;
    }
    return n;
}

// Tunable launch configuration of the FP32 slab kernel (see autotune.cu).
static void proj_config(const modal_ctx *ctx, int P, int *SG, int *CPL, int *cpb)
{
    *CPL = (P <= 32) ? 1 : 2;
    *SG = (P <= 32) ? 8 : 4;
    if (ctx->proj_sg == 4 || (ctx->proj_sg == 8 && P <= 32)) *SG = ctx->proj_sg;
    *cpb = ctx->proj_cpb > 0 ? ctx->proj_cpb : 0;
}

modal_status proj_plan(modal_ctx *ctx, int S, const modal_shape *shapes, modal_prec prec, ProjPlan &pl)
{
    const int lmin = ctx->lmin, lmax = ctx->lmax, L = ctx->L, P = ctx->P, N = ctx->N, PP = P * P;
    pl = ProjPlan();
    pl.S = S;
    pl.prec = prec;
    pl.desc.resize(S);
    long tab_total = 0;
    for (int s = 0; s < S; s++) {
        const modal_shape &m = shapes[s];
        DShape &d = pl.desc[s];
        d.kind = m.kind;
        d.nterms = m.nterms;
        d.tab_off = tab_total;
        d.c1 = m.c[0]; d.c2 = m.c[1]; d.c3 = m.c[2];
        d.sigma = m.sigma;
        if (m.kind == MODAL_SHAPE_SEPARABLE) {
            if (m.nterms < 1 || !m.tab) { set_error("shape %d: separable needs nterms >= 1 and a table", s); return MODAL_ERR_ARG; }
            tab_total += (long)m.nterms * 3 * (lmax + 1);
        } else if (m.kind == MODAL_SHAPE_BUMP) {
            if (!(m.sigma > 0.0)) { set_error("shape %d: bump sigma must be > 0", s); return MODAL_ERR_ARG; }
            d.nterms = 0;
        } else {
            set_error("shape %d: unknown kind %d", s, m.kind);
            return MODAL_ERR_ARG;
        }
    }
    pl.tab_total = tab_total;
    {   // FP32 layout: 2 parities x H entries x nterms x 4 floats per separable shape
        const long H = (lmax + 2) / 2;
        long off = 0;
        for (int s = 0; s < S; s++)
            if (pl.desc[s].kind == MODAL_SHAPE_SEPARABLE) {
                pl.desc[s].tab_off_f = off;
                off += 2 * H * pl.desc[s].nterms * 4;
                pl.max_nterms = std::max(pl.max_nterms, pl.desc[s].nterms);
            }
        pl.tabf_total = off;
    }
    MODAL_TRY(ensure(ctx->shape_tab, sizeof(double) * (size_t)(tab_total > 0 ? tab_total : 1)));
    MODAL_TRY(ensure(ctx->shape_desc, sizeof(DShape) * (size_t)S));
    // slab schedule: heaviest slabs first
    std::vector<int> order(L);
    std::vector<long> cnt(L);
    for (int q = 0; q < L; q++) { order[q] = q; cnt[q] = slab_points(lmin + q, lmax); }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cnt[a] > cnt[b]; });
    MODAL_TRY(ensure(ctx->slab_order, sizeof(int) * (size_t)L));
    MODAL_CUDA(cudaMemcpyAsync(ctx->slab_order.ptr, order.data(), sizeof(int) * L, cudaMemcpyHostToDevice, ctx->stream));
    MODAL_TRY(ensure(ctx->vl, sizeof(double) * (lmax + 1)));
    MODAL_TRY(ensure(ctx->beta, sizeof(double) * (size_t)S * N));
    if (prec == MODAL_PREC_SPLIT) {
        proj_config(ctx, P, &pl.SG, &pl.CPL, &pl.cpb);
        pl.tc = (P <= 32 && ctx->proj_tc != 0);
        auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
        size_t o = 0;
        pl.o_q = o; o += al(sizeof(float) * (size_t)L * P);
        pl.o_v = o; o += al(sizeof(float) * (lmax + 1));
        pl.o_t = o; o += al(sizeof(float) * (size_t)(pl.tabf_total > 0 ? pl.tabf_total : 4));
        pl.o_s = o; o += al(sizeof(FShape) * (size_t)S);
        pl.o_F = o; o += al(sizeof(float) * (size_t)S * L * PP);
        pl.o_B = o; o += al(sizeof(double) * (size_t)S * P * PP);
        pl.o_c = o; o += al(sizeof(int));
        long long npts = 0;
        for (int i = lmin; i <= lmax; i++) npts += tet_row_offset(i, lmax + 1, lmax);
        pl.npts = npts;
        pl.o_sb = o; o += al(sizeof(long long) * (size_t)(L + 1));
        pl.o_w = o; o += al(sizeof(float) * (size_t)npts);
        if (pl.tc) {
            pl.Mpad = (lmax / 2 + 1 + 31) / 32 * 32;
            pl.o_bq = o; o += al(sizeof(__nv_bfloat16) * 2 * 3 * 32 * (size_t)pl.Mpad);
            pl.o_perm = o; o += al(sizeof(int) * (size_t)S);
        }
        MODAL_TRY(ensure(ctx->scratch, o));
        const size_t nb4 = (size_t)(P + 3) / 4;
        pl.smem = sizeof(float) * 32 * (size_t)pl.SG * nb4 * nb4;  // F Kahan pairs, element-major over 4 x 4 tiles
        int dev = ctx->device, nsm = 0;
        MODAL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        pl.nsm = nsm;
        if (pl.tc) {
            // work items of 4 shapes of one kind and term count where possible
            pl.perm.resize(S);
            for (int s = 0; s < S; s++) pl.perm[s] = s;
            std::stable_sort(pl.perm.begin(), pl.perm.end(), [&](int a, int b) {
                const DShape &x = pl.desc[a], &y = pl.desc[b];
                return x.kind != y.kind ? x.kind < y.kind : x.nterms < y.nterms;
            });
            MODAL_CUDA(cudaMemcpyAsync(ctx->scratch.as<uint8_t>() + pl.o_perm, pl.perm.data(), sizeof(int) * S,
                                       cudaMemcpyHostToDevice, ctx->stream));
            MODAL_CUDA(cudaFuncSetAttribute(k_project_slab_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, PT_SMEM));
            MODAL_TRY(oz_reset(ctx));
        }
        if (pl.SG == 8) MODAL_CUDA(cudaFuncSetAttribute(k_project_slab_f32<8, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
        else if (pl.CPL == 1) MODAL_CUDA(cudaFuncSetAttribute(k_project_slab_f32<4, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
        else MODAL_CUDA(cudaFuncSetAttribute(k_project_slab_f32<4, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
    } else {
        const int KMAX = (lmax - lmin) / 2 + 2;
        pl.smem = sizeof(double) * ((size_t)JC * KMAX + (size_t)JC * P + (size_t)JC * PJ_TCOEF64 * 3);
        if (pl.smem > 220 * 1024) { set_error("project: lmax=%d too large for the slab tile", lmax); return MODAL_ERR_ARG; }
        pl.fpt = ceil_div(PP, 256);
        if (pl.fpt > 16) { set_error("project: P=%d too large", P); return MODAL_ERR_ARG; }
        // F partials [S][L][P*P] | B [S][P][P*P] | slab bases [L+1] | weight table [points]
        long long npts = 0;
        for (int i = lmin; i <= lmax; i++) npts += tet_row_offset(i, lmax + 1, lmax);
        pl.npts = npts;
        pl.o_B = sizeof(double) * (size_t)S * L * PP;
        pl.o_sb = pl.o_B + sizeof(double) * (size_t)S * P * PP;
        pl.o_w = pl.o_sb + sizeof(long long) * (size_t)(L + 1);
        MODAL_TRY(ensure(ctx->scratch, pl.o_w + sizeof(double) * (size_t)npts));
        auto attr = [&](auto kern) -> modal_status {
            MODAL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
            return MODAL_OK;
        };
        if (pl.fpt <= 1) MODAL_TRY(attr(k_project_slab_fp64<1>));
        else if (pl.fpt <= 4) MODAL_TRY(attr(k_project_slab_fp64<4>));
        else if (pl.fpt <= 8) MODAL_TRY(attr(k_project_slab_fp64<8>));
        else MODAL_TRY(attr(k_project_slab_fp64<16>));
    }
    return MODAL_OK;
}

modal_status proj_stage(modal_ctx *ctx, const ProjPlan &pl, const modal_shape *shapes)
{
    const int lmax = ctx->lmax;
    for (int s = 0; s < pl.S; s++) {
        const modal_shape &m = shapes[s];
        if (m.kind != MODAL_SHAPE_SEPARABLE) continue;
        size_t n = (size_t)m.nterms * 3 * (lmax + 1);
        MODAL_CUDA(cudaMemcpyAsync(ctx->shape_tab.as<double>() + pl.desc[s].tab_off, m.tab, sizeof(double) * n,
                                   cudaMemcpyHostToDevice, ctx->stream));
    }
    MODAL_CUDA(cudaMemcpyAsync(ctx->shape_desc.ptr, pl.desc.data(), sizeof(DShape) * pl.S, cudaMemcpyHostToDevice,
                               ctx->stream));
    return MODAL_OK;
}

modal_status proj_record(modal_ctx *ctx, const ProjPlan &pl)
{
    const int lmin = ctx->lmin, lmax = ctx->lmax, L = ctx->L, P = ctx->P, N = ctx->N, PP = P * P, S = pl.S;
    k_vl<<<ceil_div(lmax + 1, 256), 256, 0, ctx->stream>>>(lmax, ctx->cl.as<double>(), ctx->vl.as<double>());
    MODAL_TRY(launched(ctx, "vl"));
    if (pl.prec == MODAL_PREC_SPLIT) {
        uint8_t *b = ctx->scratch.as<uint8_t>();
        float *qf = reinterpret_cast<float *>(b + pl.o_q), *vlf = reinterpret_cast<float *>(b + pl.o_v);
        float *tabf = reinterpret_cast<float *>(b + pl.o_t), *Fbuf = reinterpret_cast<float *>(b + pl.o_F);
        FShape *fs = reinterpret_cast<FShape *>(b + pl.o_s);
        double *B = reinterpret_cast<double *>(b + pl.o_B);
        int *counter = reinterpret_cast<int *>(b + pl.o_c);
        k_d2f<<<ceil_div((long)L * P, 256), 256, 0, ctx->stream>>>((long)L * P, ctx->q.as<double>(), qf);
        MODAL_TRY(launched(ctx, "d2f_q"));
        k_d2f<<<ceil_div(lmax + 1, 256), 256, 0, ctx->stream>>>(lmax + 1, ctx->vl.as<double>(), vlf);
        MODAL_TRY(launched(ctx, "d2f_vl"));
        if (pl.tabf_total > 0) {
            k_tab_f32<<<dim3(ceil_div((lmax + 1) * pl.max_nterms, 256), S), 256, 0, ctx->stream>>>(
                lmax, ctx->shape_desc.as<DShape>(), ctx->shape_tab.as<double>(), tabf);
            MODAL_TRY(launched(ctx, "tab_f32"));
        }
        k_fshapes<<<ceil_div(S, 64), 64, 0, ctx->stream>>>(S, ctx->shape_desc.as<DShape>(), fs);
        MODAL_TRY(launched(ctx, "fshapes"));
        long long *sbase = reinterpret_cast<long long *>(b + pl.o_sb);
        float *Wt = reinterpret_cast<float *>(b + pl.o_w);
        k_slab_base<<<1, 256, 0, ctx->stream>>>(lmin, lmax, sbase);
        MODAL_TRY(launched(ctx, "slab_base"));
        k_weight_table<<<dim3(L, ceil_div(L, 8)), 256, 0, ctx->stream>>>(lmin, lmax, vlf, sbase, Wt);
        MODAL_TRY(launched(ctx, "weight_table"));
        if (pl.tc) {
            __nv_bfloat16 *Bq = reinterpret_cast<__nv_bfloat16 *>(b + pl.o_bq);
            k_bq_pieces<<<ceil_div(64L * pl.Mpad, 256), 256, 0, ctx->stream>>>(lmin, lmax, P, pl.Mpad, ctx->q.as<double>(), Bq);
            MODAL_TRY(launched(ctx, "bq_pieces"));
            const int Gt = ceil_div(S, PT_SG), nit = L * Gt;
            MODAL_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), ctx->stream));
            k_project_slab_tc<<<std::min(nit, 2 * pl.nsm), 160, PT_SMEM, ctx->stream>>>(
                lmin, lmax, P, S, Gt, nit, counter, ctx->slab_order.as<int>(), reinterpret_cast<const int *>(b + pl.o_perm),
                qf, Bq, pl.Mpad, fs, tabf, Wt, sbase, Fbuf, ctx->ozerr.as<int>());
            MODAL_TRY(launched(ctx, "project_slab_tc"));
        }
        if (!pl.tc) {
            const int G = ceil_div(S, pl.SG), nitems = L * G;
            dim3 grid(L, G);
            int *cnt = nullptr;
            if (pl.cpb > 0) {
                MODAL_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), ctx->stream));
                grid = dim3(std::min(nitems, pl.nsm * pl.cpb), 1);
                cnt = counter;
            }
            auto run = [&](auto kern) -> modal_status {
                kern<<<grid, 256, pl.smem, ctx->stream>>>(lmin, lmax, P, S, G, nitems, cnt, ctx->slab_order.as<int>(), qf,
                                                         vlf, fs, tabf, Wt, sbase, Fbuf);
                return launched(ctx, "project_slab_f32");
            };
            if (pl.SG == 8) MODAL_TRY(run(k_project_slab_f32<8, 1>));
            else if (pl.CPL == 1) MODAL_TRY(run(k_project_slab_f32<4, 1>));
            else MODAL_TRY(run(k_project_slab_f32<4, 2>));
        }
        k_project_B_f32<<<ceil_div((long)S * P * PP, 256), 256, 0, ctx->stream>>>(L, P, S, qf, Fbuf, B);
        MODAL_TRY(launched(ctx, "project_B_f32"));
        k_project_beta<<<ceil_div((long)S * N, 256), 256, 0, ctx->stream>>>(N, P, S, ctx->triples.as<int>(), B,
                                                                              ctx->beta.as<double>());
        return launched(ctx, "project_beta");
    }
    uint8_t *b8 = ctx->scratch.as<uint8_t>();
    double *Fbuf = reinterpret_cast<double *>(b8);
    double *B = reinterpret_cast<double *>(b8 + pl.o_B);
    long long *sbase = reinterpret_cast<long long *>(b8 + pl.o_sb);
    double *Wd = reinterpret_cast<double *>(b8 + pl.o_w);
    k_slab_base<<<1, 256, 0, ctx->stream>>>(lmin, lmax, sbase);
    MODAL_TRY(launched(ctx, "slab_base"));
    k_weight_table_fp64<<<dim3(L, ceil_div(L, 8)), 256, 0, ctx->stream>>>(lmin, lmax, ctx->vl.as<double>(), sbase, Wd);
    MODAL_TRY(launched(ctx, "weight_table_fp64"));
    const int KMAX = (lmax - lmin) / 2 + 2;
    auto run = [&](auto kern) -> modal_status {
        kern<<<L, 256, pl.smem, ctx->stream>>>(lmin, lmax, P, S, KMAX, ctx->slab_order.as<int>(), ctx->q.as<double>(),
                                               ctx->vl.as<double>(), ctx->shape_desc.as<DShape>(),
                                               ctx->shape_tab.as<double>(), Wd, sbase, Fbuf, pl.ra);
        return launched(ctx, "project_slab_fp64");
    };
    if (pl.fpt <= 1) MODAL_TRY(run(k_project_slab_fp64<1>));
    else if (pl.fpt <= 4) MODAL_TRY(run(k_project_slab_fp64<4>));
    else if (pl.fpt <= 8) MODAL_TRY(run(k_project_slab_fp64<8>));
    else MODAL_TRY(run(k_project_slab_fp64<16>));
    k_project_B<<<ceil_div((long)S * P * PP, 256), 256, 0, ctx->stream>>>(L, P, S, ctx->q.as<double>(), Fbuf, B);
    MODAL_TRY(launched(ctx, "project_B"));
    k_project_beta<<<ceil_div((long)S * N, 256), 256, 0, ctx->stream>>>(N, P, S, ctx->triples.as<int>(), B,
                                                                          ctx->beta.as<double>());
    return launched(ctx, "project_beta");
}

modal_status project_dev(modal_ctx *ctx, int S, const modal_shape *shapes, modal_prec prec)
{
    ProjPlan pl;
    MODAL_TRY(proj_plan(ctx, S, shapes, prec, pl));
    MODAL_TRY(proj_stage(ctx, pl, shapes));
    return proj_record(ctx, pl);
}

__global__ void k_wq(int lmax, const double *__restrict__ cl, double *__restrict__ wq)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l > lmax) return;
    wq[l] = (l < 2) ? 0.0 : pow(2.0 * l + 1.0, 1.0 / 6.0) * (1.0 / sqrt(cl[l]));
}

}  // namespace modal

using namespace modal;

extern "C" modal_status modal_gamma_transfer_3d(modal_ctx *c, double deltaphi, double *gamma_t)
{
    if (!c || !gamma_t) { set_error("modal_gamma_transfer_3d: NULL argument"); return MODAL_ERR_ARG; }
    if (!c->have_modes || !c->have_spec || c->tr_xsize < 2) {
        set_error("modal_gamma_transfer_3d: set basis, modes, spectrum and transfer functions first");
        return MODAL_ERR_STATE;
    }
    if (c->lmin < 2) { set_error("modal_gamma_transfer_3d: lmin must be >= 2"); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    const int S = c->tr_Nprim, N = c->N, lmax = c->lmax;
    // each primordial mode is one radial shape of the FP64 projection
    std::vector<modal_shape> placeholder(S);
    for (int s = 0; s < S; s++) {
        placeholder[s] = modal_shape{};
        placeholder[s].kind = MODAL_SHAPE_BUMP;
        placeholder[s].sigma = 1.0;
    }
    ProjPlan pl;
    MODAL_TRY(proj_plan(c, S, placeholder.data(), MODAL_PREC_FP64, pl));
    for (int s = 0; s < S; s++) {
        pl.desc[s].kind = SHAPE_RADIAL;
        pl.desc[s].nterms = s;
    }
    MODAL_TRY(ensure(c->scratch2, sizeof(double) * (size_t)(lmax + 1)));
    k_wq<<<ceil_div(lmax + 1, 256), 256, 0, c->stream>>>(lmax, c->cl.as<double>(), c->scratch2.as<double>());
    MODAL_TRY(launched(c, "wq"));
    pl.ra.qt = c->tr_qt.as<double>();
    pl.ra.x = c->tr_x.as<double>();
    pl.ra.wq = c->scratch2.as<double>();
    pl.ra.prim = c->tr_prim.as<int>();
    pl.ra.xsize = c->tr_xsize;
    pl.ra.Pp = c->tr_Pp;
    pl.ra.L1 = lmax + 1;
    // the row factors of d_radial_rows sit after the kernel's f and H tiles
    pl.smem += sizeof(double) * ((size_t)JC * 3 * c->tr_xsize + c->tr_xsize);
    if (pl.smem > 220 * 1024) { set_error("modal_gamma_transfer_3d: lmax=%d, xsize=%d too large for the slab tile", lmax, c->tr_xsize); return MODAL_ERR_ARG; }
    {
        auto attr = [&](auto kern) -> modal_status {
            MODAL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
            return MODAL_OK;
        };
        if (pl.fpt <= 1) MODAL_TRY(attr(k_project_slab_fp64<1>));
        else if (pl.fpt <= 4) MODAL_TRY(attr(k_project_slab_fp64<4>));
        else if (pl.fpt <= 8) MODAL_TRY(attr(k_project_slab_fp64<8>));
        else MODAL_TRY(attr(k_project_slab_fp64<16>));
    }
    {
        StageTimer t(c, MODAL_T_GAMMA);
        MODAL_TRY(proj_stage(c, pl, placeholder.data()));
        MODAL_TRY(proj_record(c, pl));
    }
    std::vector<double> b((size_t)S * N);
    MODAL_CUDA(cudaMemcpyAsync(b.data(), c->beta.ptr, sizeof(double) * b.size(), cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    c->have_beta = false;  // the device beta holds these radial projections, not shapes'
    const double f = 6.0 * deltaphi * deltaphi;  // calculate_gamma_3d.c:434-439
    for (int m = 0; m < N; m++)
        for (int n = 0; n < S; n++) gamma_t[(size_t)m * S + n] = f * b[(size_t)n * N + m];
    return MODAL_OK;
}
