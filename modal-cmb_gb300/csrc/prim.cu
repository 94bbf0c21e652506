// prim.cu -- primordial k-space side: the Gram matrix of the primordial modes
// on the k-grid tetrapyd (calculate_ortho, orthogonalisation.c:14-86) and the
// projection of primordial shapes onto them (calculate_eigen,
// calculate_eigen.c:86-144; <S,S> of integrate_template2, :13-84), FP64.
//
// Grid: the walk of get_ijk_next_prim from (min,min,min) (tetrapyd_tools.c:
// 416-550) visits, in order,
//   min <= i < max,  i <= j <= max,  j <= k <= min(max, i+j+2),
// and then the end point (max, max, max), which decompose_tetrapyd_prim counts
// too.  Row j of slab i has min(max - j, i + 2) + 1 points, so a flat point
// index maps to (i, j, k) with a per-slab offset and a closed form.
// Point weight: x = calculate_weight(min,max,i,j,k) dk^3 / (dk (i+j+k)),
// dk = kmax/max (calculate_volume.c:12-133: 1 inside, boundary cells from the
// 3x3x3 neighbourhood, times 1/3/6 for the permutations).
// Mode r = (p1,p2,p3): pijk = (1/6) sum of the six products of basis[l][p]
// (orthogonalisation.c:279-295).
//
// Both sums are GEMM-shaped over points: with B[pt][r] = pijk_r(pt) and
// x = weight, Gamma = B^T diag(x) B and alpha[s] = (x S_s)^T B.  Points are
// processed in chunks: a kernel fills B, x B and the shape values for a
// chunk, then the FP64 tiled GEMM accumulates.
#include <algorithm>
#include <vector>
#include "common.cuh"

namespace modal {

namespace {

__device__ __forceinline__ double cellv(int kind, const double p[8])
{
    // p = (a,b,c,d,e,f,g,h) in the argument order of cell1..cell4 (calculate_volume.c:262-301)
    const double a = p[0], b = p[1], c = p[2], d = p[3], e = p[4], f = p[5], g = p[6], h = p[7];
    switch (kind) {
    case 1: return (11 * (a + b + c + e) + 17 * (d + g + f) + 25 * h) / 240.0;
    case 2: return (47 * a + 19 * (b + c + e) + 5 * (d + f + g) + h) / 720.0;
    case 3: return (40 * (b + c) + 35 * (a + d) + 26 * (f + g) + 19 * (e + h)) / 360.0;
    default: return (89 * a + 85 * (b + c + e) + 71 * (d + f + g) + 43 * h) / 720.0;
    }
}

// calculate_weight (calculate_volume.c:12-133).
__device__ double prim_weight(int min, int max, int i, int j, int k)
{
    int grid[3][3][3], sum = 0;
    for (int l = 0; l < 3; l++)
        for (int m = 0; m < 3; m++)
            for (int n = 0; n < 3; n++) {
                const int i0 = i + l - 1, j0 = j + m - 1, k0 = k + n - 1;
                int v;
                if (i0 < min || i0 > max || j0 < min || j0 > max || k0 < min || k0 > max) v = -8;
                else if (i0 > j0 + k0 || j0 > i0 + k0 || k0 > i0 + j0) v = 0;
                else { v = 1; sum++; }
                grid[l][m][n] = v;
            }
    double weight = 0.0;
    if (sum == 27) {
        weight = 1.0;
    } else {
        for (int s1 = 0; s1 < 2; s1++)
            for (int s2 = 0; s2 < 2; s2++)
                for (int s3 = 0; s3 < 2; s3++) {
                    int su = 0;
                    for (int l = 0; l < 2; l++)
                        for (int m = 0; m < 2; m++)
                            for (int n = 0; n < 2; n++) su += grid[l + s1][m + s2][n + s3];
                    // corner values of the hat function pt (1 at the centre only)
                    auto P = [&](int l, int m, int n) { return (l == 1 && m == 1 && n == 1) ? 1.0 : 0.0; };
                    const double a = P(s1, s2, s3), b = P(s1 + 1, s2, s3), c = P(s1, s2 + 1, s3),
                                 d = P(s1 + 1, s2 + 1, s3), e = P(s1, s2, s3 + 1), f = P(s1 + 1, s2, s3 + 1),
                                 g = P(s1, s2 + 1, s3 + 1), h = P(s1 + 1, s2 + 1, s3 + 1);
                    if (su == 4) {
                        if (grid[1 + s1][0 + s2][1 + s3] == 1) { const double q[8] = {f, e, h, g, b, a, d, c}; weight += cellv(2, q); }
                        if (grid[1 + s1][1 + s2][0 + s3] == 1) { const double q[8] = {d, c, b, a, h, g, f, e}; weight += cellv(2, q); }
                        if (grid[0 + s1][1 + s2][1 + s3] == 1) { const double q[8] = {g, h, e, f, c, d, a, b}; weight += cellv(2, q); }
                    } else if (su == 5) {
                        const double q[8] = {a, b, c, d, e, f, g, h};
                        weight += cellv(1, q);
                    } else if (su == 6) {
                        if (grid[0 + s1][0 + s2][1 + s3] == 1) { const double q[8] = {g, h, e, f, c, d, a, b}; weight += cellv(3, q); }
                        if (grid[1 + s1][0 + s2][0 + s3] == 1) { const double q[8] = {f, h, b, d, e, g, a, c}; weight += cellv(3, q); }
                        if (grid[0 + s1][1 + s2][0 + s3] == 1) { const double q[8] = {d, h, c, g, b, f, a, e}; weight += cellv(3, q); }
                    } else if (su == 7) {
                        if (grid[0 + s1][1 + s2][0 + s3] == 0) { const double q[8] = {f, e, h, g, b, a, d, c}; weight += cellv(4, q); }
                        if (grid[0 + s1][0 + s2][1 + s3] == 0) { const double q[8] = {d, c, b, a, h, g, f, e}; weight += cellv(4, q); }
                        if (grid[1 + s1][0 + s2][0 + s3] == 0) { const double q[8] = {g, h, e, f, c, d, a, b}; weight += cellv(4, q); }
                    } else if (su == 8) {
                        weight += 1.0 / 8.0;
                    }
                }
    }
    if (i != k) weight *= (i == j || j == k) ? 3.0 : 6.0;
    return weight;
}

// Flat point index -> (i, j, k).  slab_off[s] = first index of slab i = min + s,
// nslab = max - min slabs, then the end point.
__device__ __forceinline__ void prim_point(long p, int min, int max, int nslab, const long *__restrict__ slab_off,
                                           int *pi, int *pj, int *pk)
{
    if (p >= slab_off[nslab]) { *pi = *pj = *pk = max; return; }
    int lo = 0, hi = nslab - 1;
    while (lo < hi) {  // last slab with slab_off <= p
        const int mid = (lo + hi + 1) >> 1;
        if (slab_off[mid] <= p) lo = mid;
        else hi = mid - 1;
    }
    const int i = min + lo;
    long q = p - slab_off[lo];
    // rows j = i .. max - i - 2 have i + 3 points; later rows max - j + 1
    const int R = i + 3;
    const int nf0 = (max - i - 2) - i + 1, nf = nf0 > 0 ? nf0 : 0;
    int j, k;
    if (q < (long)nf * R) {
        j = i + (int)(q / R);
        k = j + (int)(q % R);
    } else {
        q -= (long)nf * R;
        j = i + nf;
        int len = max - j + 1;
        while (q >= len) { q -= len; j++; len--; }
        k = j + (int)q;
    }
    *pi = i;
    *pj = j;
    *pk = k;
}

__device__ __forceinline__ double pijk(const double *__restrict__ basis, int P, int p1, int p2, int p3, int i, int j,
                                       int k)
{
    const double *bi = basis + (size_t)i * P, *bj = basis + (size_t)j * P, *bk = basis + (size_t)k * P;
    const double b1 = bi[p1] * bj[p2] * bk[p3], b2 = bi[p2] * bj[p3] * bk[p1];
    const double b3 = bi[p3] * bj[p1] * bk[p2], b4 = bi[p3] * bj[p2] * bk[p1];
    const double b5 = bi[p2] * bj[p1] * bk[p3], b6 = bi[p1] * bj[p3] * bk[p2];
    return (b1 + b2 + b3 + b4 + b5 + b6) / 6.0;
}

// x of a chunk's points: calculate_weight dk^3 / (dk (i+j+k)) (calculate_eigen.c:110-121)
__global__ void k_prim_weights(long p0, long n, int min, int max, int nslab, const long *__restrict__ slab_off,
                               double kmax, double *__restrict__ x, int *__restrict__ ijk)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    prim_point(p0 + t, min, max, nslab, slab_off, &i, &j, &k);
    const double factor = kmax * (1e0 / (double)max), cube = factor * factor * factor;
    double v = prim_weight(min, max, i, j, k) * cube;
    double ksum = factor * i + factor * j + factor * k;
    if (ksum > 1e-10) ksum = 1e0 / ksum;
    x[t] = v * ksum;
    ijk[3 * t] = i;
    ijk[3 * t + 1] = j;
    ijk[3 * t + 2] = k;
}

// B[t][r] = pijk_r, Bw[t][r] = x_t B[t][r]
__global__ void k_prim_modes(long n, int N, int P, const int *__restrict__ ijk, const double *__restrict__ x,
                             const double *__restrict__ basis, const int *__restrict__ prim, double *__restrict__ B,
                             double *__restrict__ Bw)
{
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * N) return;
    const long t = e / N;
    const int r = (int)(e - t * N);
    const double v = pijk(basis, P, prim[3 * r], prim[3 * r + 1], prim[3 * r + 2], ijk[3 * t], ijk[3 * t + 1],
                          ijk[3 * t + 2]);
    B[e] = v;
    if (Bw) Bw[e] = x[t] * v;
}

// Shape values of a chunk: Sw[s][t] = x_t S_s(pt), n2[s] += x S^2 (per-chunk partial, atomics)
__global__ void k_prim_shapes(long n, int S, int stride, const int *__restrict__ ijk, const double *__restrict__ x,
                              const DShape *__restrict__ sh, const double *__restrict__ tab, double *__restrict__ Sw,
                              double *__restrict__ n2)
{
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * S) return;
    const long t = e / S;
    const int s = (int)(e - t * S);
    const int i = ijk[3 * t], j = ijk[3 * t + 1], k = ijk[3 * t + 2];
    const DShape d = sh[s];
    double val;
    if (d.kind == MODAL_SHAPE_SEPARABLE) {
        val = 0.0;
        for (int tt = 0; tt < d.nterms; tt++) {
            const double *f = tab + d.tab_off + (long)tt * 3 * stride, *g = f + stride, *h = g + stride;
            const double v = f[i] * g[j] * h[k] + f[i] * g[k] * h[j] + f[j] * g[i] * h[k] + f[j] * g[k] * h[i] +
                             f[k] * g[i] * h[j] + f[k] * g[j] * h[i];
            val += v / 6.0;
        }
    } else {
        const double L = (double)(i + j + k);
        const double x1 = i / L - d.c1, x2 = j / L - d.c2, x3 = k / L - d.c3;
        val = exp(-(x1 * x1 + x2 * x2 + x3 * x3) / (2.0 * d.sigma * d.sigma));
    }
    Sw[(size_t)s * n + t] = x[t] * val;
    atomicAdd(&n2[s], x[t] * (val * val));
}

// packed upper triangle (r <= s) of the lower-filled G (G[s][r], s >= r)
__global__ void k_pack_upper(int N, const double *__restrict__ G, double *__restrict__ out)
{
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long vsize = (long)N * (N + 1) / 2;
    if (e >= vsize) return;
    // invert e -> (r, s), r <= s, row-major over the upper triangle
    long r = (long)((2.0 * N + 1 - sqrt((2.0 * N + 1) * (2.0 * N + 1) - 8.0 * e)) / 2.0);
    if (r < 0) r = 0;
    while (r > 0 && r * N - r * (r - 1) / 2 > e) r--;
    while ((r + 1) * N - (r + 1) * r / 2 <= e) r++;
    const long s = r + (e - (r * N - r * (r - 1) / 2));
    out[e] = G[(size_t)s * N + r];
}

struct PrimGrid {
    int min = 0, max = 0, nslab = 0;
    long npts = 0;
    std::vector<long> off;  // [nslab + 1]
};

modal_status prim_grid(int min, int max, PrimGrid &g)
{
    if (min < 0 || max < 1 || min >= max) { set_error("primordial grid: min=%d max=%d (0 <= min < max)", min, max); return MODAL_ERR_ARG; }
    g.min = min;
    g.max = max;
    g.nslab = max - min;
    g.off.assign(g.nslab + 1, 0);
    for (int s = 0; s < g.nslab; s++) {
        const int i = min + s;
        long n = 0;
        for (int j = i; j <= max; j++) n += std::min(max - j, i + 2) + 1;
        g.off[s + 1] = g.off[s] + n;
    }
    g.npts = g.off[g.nslab] + 1;  // and the end point
    return MODAL_OK;
}

// Shared set-up of both entry points: grid, basis, triples, chunk buffers.
struct PrimRun {
    PrimGrid g;
    long C = 0;
    long *d_off = nullptr;
    double *basis = nullptr, *x = nullptr, *B = nullptr, *Bw = nullptr;
    int *prim = nullptr, *ijk = nullptr;
    uint8_t *base = nullptr;
    size_t o_end = 0;
};

modal_status prim_setup(modal_ctx *c, int min, int max, int P, const double *basis, int N, const int *prim, int extra_cols,
                        size_t extra_bytes, PrimRun &run)
{
    if (!c || P < 1 || P > 64 || N < 1 || !basis || !prim) { set_error("primordial: bad arguments (P=%d N=%d)", P, N); return MODAL_ERR_ARG; }
    for (long e = 0; e < 3L * N; e++)
        if (prim[e] < 0 || prim[e] >= P) { set_error("primordial: mode index %d outside [0,%d)", prim[e], P); return MODAL_ERR_ARG; }
    MODAL_TRY(prim_grid(min, max, run.g));
    MODAL_CUDA(cudaSetDevice(c->device));
    const int cols = N + extra_cols;
    run.C = std::max<long>(1024, std::min<long>(65536, (long)(1L << 26) / cols));
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t o = 0;
    const size_t o_off = o; o += al(sizeof(long) * (run.g.nslab + 1));
    const size_t o_bas = o; o += al(sizeof(double) * (size_t)(max + 1) * P);
    const size_t o_pr = o; o += al(sizeof(int) * 3 * (size_t)N);
    const size_t o_x = o; o += al(sizeof(double) * run.C);
    const size_t o_ijk = o; o += al(sizeof(int) * 3 * run.C);
    const size_t o_B = o; o += al(sizeof(double) * run.C * N);
    const size_t o_Bw = o; o += al(sizeof(double) * run.C * cols);
    run.o_end = o;
    MODAL_TRY(ensure(c->prim, o + extra_bytes));
    uint8_t *b = c->prim.as<uint8_t>();
    run.base = b;
    run.d_off = reinterpret_cast<long *>(b + o_off);
    run.basis = reinterpret_cast<double *>(b + o_bas);
    run.prim = reinterpret_cast<int *>(b + o_pr);
    run.x = reinterpret_cast<double *>(b + o_x);
    run.ijk = reinterpret_cast<int *>(b + o_ijk);
    run.B = reinterpret_cast<double *>(b + o_B);
    run.Bw = reinterpret_cast<double *>(b + o_Bw);
    MODAL_CUDA(cudaMemcpyAsync(run.d_off, run.g.off.data(), sizeof(long) * (run.g.nslab + 1), cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(run.basis, basis, sizeof(double) * (size_t)(max + 1) * P, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(run.prim, prim, sizeof(int) * 3 * (size_t)N, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));  // the host vectors go out of scope with the caller's run
    return MODAL_OK;
}

}  // namespace

}  // namespace modal

using namespace modal;

extern "C" {

modal_status modal_prim_points(int min, int max, long *npts, int *pts)
{
    if (!npts) { set_error("modal_prim_points: npts is NULL"); return MODAL_ERR_ARG; }
    PrimGrid g;
    MODAL_TRY(prim_grid(min, max, g));
    *npts = g.npts;
    if (!pts) return MODAL_OK;
    int dev = 0;
    MODAL_CUDA(cudaGetDevice(&dev));
    DevBuf off, x, ijk;
    modal_status st = ensure(off, sizeof(long) * (g.nslab + 1));
    if (st == MODAL_OK) st = ensure(x, sizeof(double) * g.npts);
    if (st == MODAL_OK) st = ensure(ijk, sizeof(int) * 3 * g.npts);
    cudaError_t e = cudaSuccess;
    if (st == MODAL_OK) e = cudaMemcpy(off.ptr, g.off.data(), sizeof(long) * (g.nslab + 1), cudaMemcpyHostToDevice);
    if (st == MODAL_OK && e == cudaSuccess) {
        k_prim_weights<<<ceil_div(g.npts, 256), 256>>>(0, g.npts, min, max, g.nslab, off.as<long>(), 1.0, x.as<double>(),
                                                       ijk.as<int>());
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(pts, ijk.ptr, sizeof(int) * 3 * g.npts, cudaMemcpyDeviceToHost);
    }
    release(off);
    release(x);
    release(ijk);
    if (st != MODAL_OK) return st;
    if (e != cudaSuccess) { set_error("modal_prim_points: %s", cudaGetErrorString(e)); return MODAL_ERR_CUDA; }
    return MODAL_OK;
}

modal_status modal_prim_ortho(modal_ctx *c, int min, int max, double kmax, int P, const double *basis, int N,
                              const int *prim, double *ortho)
{
    if (!ortho || !(kmax > 0.0)) { set_error("modal_prim_ortho: ortho NULL or kmax <= 0"); return MODAL_ERR_ARG; }
    PrimRun run;
    const size_t gbytes = ((sizeof(double) * (size_t)N * N + 255) & ~(size_t)255) + sizeof(double) * (size_t)N * (N + 1) / 2;
    MODAL_TRY(prim_setup(c, min, max, P, basis, N, prim, 0, gbytes, run));
    double *G = reinterpret_cast<double *>(run.base + run.o_end);
    double *packed = G + (((size_t)N * N * sizeof(double) + 255) & ~(size_t)255) / sizeof(double);
    StageTimer t(c, MODAL_T_GAMMA);
    MODAL_CUDA(cudaMemsetAsync(G, 0, sizeof(double) * (size_t)N * N, c->stream));
    for (long p0 = 0; p0 < run.g.npts; p0 += run.C) {
        const long n = std::min(run.C, run.g.npts - p0);
        k_prim_weights<<<ceil_div(n, 256), 256, 0, c->stream>>>(p0, n, min, max, run.g.nslab, run.d_off, kmax, run.x,
                                                                 run.ijk);
        MODAL_TRY(launched(c, "prim_weights"));
        k_prim_modes<<<ceil_div(n * N, 256), 256, 0, c->stream>>>(n, N, P, run.ijk, run.x, run.basis, run.prim, run.B,
                                                                   run.Bw);
        MODAL_TRY(launched(c, "prim_modes"));
        // G[s][r] += sum_t Bw[t][s] B[t][r]  (lower triangle s >= r)
        MODAL_TRY(dgemm_splitk(c, N, N, (int)n, run.Bw, N, true, run.B, N, false, G, N, 1, true));
    }
    k_pack_upper<<<ceil_div((long)N * (N + 1) / 2, 256), 256, 0, c->stream>>>(N, G, packed);
    MODAL_TRY(launched(c, "pack_upper"));
    t.stop();
    MODAL_CUDA(cudaMemcpyAsync(ortho, packed, sizeof(double) * (size_t)N * (N + 1) / 2, cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}

modal_status modal_prim_eigen(modal_ctx *c, int min, int max, double kmax, int P, const double *basis, int N,
                              const int *prim, int S, const modal_shape *shapes, double *alpha, double *norm2)
{
    if (!alpha || S < 1 || !shapes || !(kmax > 0.0)) { set_error("modal_prim_eigen: bad arguments (S=%d)", S); return MODAL_ERR_ARG; }
    // shape tables over grid indices 0..max
    std::vector<DShape> ds(S);
    long tab_total = 0;
    for (int s = 0; s < S; s++) {
        const modal_shape &m = shapes[s];
        ds[s] = DShape{m.kind, m.nterms, tab_total, m.c[0], m.c[1], m.c[2], m.sigma};
        if (m.kind == MODAL_SHAPE_SEPARABLE) {
            if (m.nterms < 1 || !m.tab) { set_error("shape %d: separable needs nterms >= 1 and a table", s); return MODAL_ERR_ARG; }
            tab_total += (long)m.nterms * 3 * (max + 1);
        } else if (m.kind != MODAL_SHAPE_BUMP || !(m.sigma > 0.0)) {
            set_error("shape %d: invalid kind or sigma", s);
            return MODAL_ERR_ARG;
        }
    }
    if (min == 0) {
        set_error("modal_prim_eigen: min >= 1 (the shapes are undefined at k = 0)");
        return MODAL_ERR_ARG;
    }
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t xb = al(sizeof(double) * (size_t)S * N) + al(sizeof(double) * S) + al(sizeof(DShape) * S) +
                      al(sizeof(double) * (size_t)(tab_total > 0 ? tab_total : 1));
    PrimRun run;
    MODAL_TRY(prim_setup(c, min, max, P, basis, N, prim, S, xb, run));
    uint8_t *b = run.base + run.o_end;
    double *A = reinterpret_cast<double *>(b);
    b += al(sizeof(double) * (size_t)S * N);
    double *n2 = reinterpret_cast<double *>(b);
    b += al(sizeof(double) * S);
    DShape *dsh = reinterpret_cast<DShape *>(b);
    b += al(sizeof(DShape) * S);
    double *tab = reinterpret_cast<double *>(b);
    for (int s = 0; s < S; s++)
        if (shapes[s].kind == MODAL_SHAPE_SEPARABLE)
            MODAL_CUDA(cudaMemcpyAsync(tab + ds[s].tab_off, shapes[s].tab,
                                       sizeof(double) * (size_t)shapes[s].nterms * 3 * (max + 1), cudaMemcpyHostToDevice,
                                       c->stream));
    MODAL_CUDA(cudaMemcpyAsync(dsh, ds.data(), sizeof(DShape) * S, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemsetAsync(A, 0, sizeof(double) * (size_t)S * N, c->stream));
    MODAL_CUDA(cudaMemsetAsync(n2, 0, sizeof(double) * S, c->stream));
    StageTimer t(c, MODAL_T_PROJECT);
    double *Sw = run.Bw;  // [S][C] shape values times x
    for (long p0 = 0; p0 < run.g.npts; p0 += run.C) {
        const long n = std::min(run.C, run.g.npts - p0);
        k_prim_weights<<<ceil_div(n, 256), 256, 0, c->stream>>>(p0, n, min, max, run.g.nslab, run.d_off, kmax, run.x,
                                                                 run.ijk);
        MODAL_TRY(launched(c, "prim_weights"));
        k_prim_modes<<<ceil_div(n * N, 256), 256, 0, c->stream>>>(n, N, P, run.ijk, run.x, run.basis, run.prim, run.B,
                                                                   nullptr);
        MODAL_TRY(launched(c, "prim_modes"));
        k_prim_shapes<<<ceil_div(n * S, 256), 256, 0, c->stream>>>(n, S, max + 1, run.ijk, run.x, dsh, tab, Sw, n2);
        MODAL_TRY(launched(c, "prim_shapes"));
        // A[s][r] += sum_t Sw[s][t] B[t][r]
        MODAL_TRY(dgemm_rows(c, S, N, (int)n, Sw, (int)n, run.B, N, false, A, N, true));
    }
    t.stop();
    MODAL_CUDA(cudaMemcpyAsync(alpha, A, sizeof(double) * (size_t)S * N, cudaMemcpyDeviceToHost, c->stream));
    if (norm2) MODAL_CUDA(cudaMemcpyAsync(norm2, n2, sizeof(double) * S, cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}

}  // extern "C"
