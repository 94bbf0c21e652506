// syev.cu -- FP64 symmetric eigen-decomposition on the GPU, the library's own.
//
// It stands in for the reference's gsl_eigen_symmv + gsl_eigen_symmv_sort
// (ortho_late_mpi.c:775-776, PCA branch :784-805) and LAPACKE_dsyevr
// (basis_optimisation_mpi.c:279).  Three stages, all FP64:
//
// 1. Householder tridiagonalisation A = Q T Q^T (lower, blocked; the algorithm
//    of LAPACK's dsytrd/dlatrd).  Each panel of TRD_NB columns is one
//    cooperative launch, one CTA per SM, each CTA owning a block of rows kept
//    in shared memory; the CTAs meet at a grid barrier twice per column: (a) finish the previous column's w vector and update the
//    next column with the panel's rank-2c correction, reduce its norm; (b)
//    form the reflector and the product y = A v over the trailing matrix (the
//    matrix-vector product that bounds this stage, summed in double-float
//    FP32 arithmetic over a (head, tail) copy of the trailing matrix).  After
//    a panel, A22 -= V W^T + W V^T on the lower triangle as an FP64-accurate
//    tensor-core product (ozgemm.cu), and the trailing block's double-float
//    copy is refreshed from it.
// 2. Divide and conquer on T (Cuppen; Dongarra-Sorensen deflation; Gu-Eisenstat
//    eigenvectors).  The tree is split down to single rows; every level's
//    merges run batched: sort and deflate (one CTA per merge), secular roots
//    (one warp per root, rational two-pole steps safeguarded by bisection),
//    zhat and the eigenvectors of the rank-one problem (one warp per row),
//    then the vector update: a grouped FP64 GEMM for small merges, the
//    tensor-core FP64-accurate product for merges of DC_OZ_MIN rows or more.
// 3. Back-transformation of the wanted eigenvectors, X <- X Q^T, by compact-WY
//    blocks of NBB reflectors in reverse order (dlarft on the blocks' Gram
//    matrices; tensor-core FP64-accurate products).
//
// Layout: row-major; eigenvectors are stored as rows (row j of V is the
// eigenvector of W[j]).  Every spin-wait is bounded; on expiry a device error
// word is set and every CTA returns (MODAL_ERR_TIMEOUT on the host).
#include <algorithm>
#include <cmath>
#include <vector>
#include "common.cuh"
#include "dfbits.cuh"

namespace modal {

namespace {

constexpr int TRD_NB = 32;                 // panel width
constexpr int DC_DEFL_SMEM = 216 * 1024;    // shared memory of the deflation's serial loop (bytes)
constexpr int TRD_THREADS = 512;           // 16 warps per CTA
constexpr int TRD_WARPS = TRD_THREADS / 32;
constexpr int VLD = TRD_NB + 1;            // shared-memory row stride of V, W (odd: no bank conflicts across rows)
constexpr int LDP = 2 * TRD_NB;            // panel row: V (TRD_NB columns) then W
constexpr int PCOMP = 2 * TRD_NB + 2;      // partial components: p[NB], q[NB], y.v, |x|^2
constexpr int NBB = 256;                   // reflectors per T block built by k_larft
constexpr int NBW = 512;                   // reflectors per compact-WY block of the back-transformation (two T blocks joined)
constexpr int OZ_SLICES = 8;               // 7-bit slices of the tensor-core FP64 products
constexpr int DC_OZ_MIN = 1024;            // merges of at least this size update their vectors on the tensor cores
constexpr long long BAR_CYCLES = 1ll << 32;  // ~2 s of clock64 per barrier wait
constexpr double EPS = 1.1102230246251565e-16;  // 2^-53

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_prod(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v *= __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Grid barrier for a cooperative launch (all CTAs co-resident), one per phase:
// bar[0] counts arrivals, bar[1] is the generation.  Measured faster here
// than per-CTA flag words that every CTA polls (152 x 152 pollers on a few L2
// lines).  Memory ordering by release/acquire atomics at GPU scope instead of
// full fences: each CTA's arrival is an acq_rel add (its writes, ordered before
// it by __syncthreads, are released; the last arrival acquires every earlier
// one), the last arrival releases the generation, the others acquire it.
// Bounded: a wait that runs out of its clock64 budget sets *err, and every CTA
// returns false once *err is set.
__device__ __forceinline__ unsigned atom_add_acq_rel_gpu(unsigned *p, unsigned v)
{
    unsigned old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ bool grid_barrier(unsigned *bar, int *err)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned g = ld_acquire_gpu(bar + 1);
        const unsigned arrived = atom_add_acq_rel_gpu(bar, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(bar, 0u);
            atom_add_acq_rel_gpu(bar + 1, 1u);
        } else {
            const long long t0 = clock64();
            while (ld_acquire_gpu(bar + 1) == g) {
                if (*(volatile int *)err) break;
                if (clock64() - t0 > BAR_CYCLES) {
                    atomicExch(err, 1);
                    break;
                }
            }
        }
    }
    __syncthreads();
    return *(volatile int *)err == 0;
}

// ------------------------------------------------------------------ stage 1

struct TrdArgs {
    double *A;          // FP64, lower triangle current (the column updates read it)
    const float2 *Ahl;  // the trailing matrix, both triangles, as double-float (head, tail) pairs
    float2 *ahl;        // [n] the updated column as double-float pairs
    int n, j0, nbp;
    double *V, *W;  // panel: rows of LDP doubles, V in columns [0, NB), W in [NB, 2 NB); zero outside the reflectors
    double *d, *e, *tau;
    double *a, *y;  // [n] work vectors
    double *part;   // [PCOMP][grid] per-CTA partial sums
    unsigned *bar;  // grid barrier: arrivals, generation
    int *err;
};

// Sum over the grid of component `comp` of the partials, by one warp (fixed order).
__device__ __forceinline__ double grid_total(const double *part, int comp, int lane)
{
    double s0 = 0.0, s1 = 0.0;
    const double *p = part + (size_t)comp * gridDim.x;
    int b = lane;
    for (; b + 32 < (int)gridDim.x; b += 64) {
        s0 += p[b];
        s1 += p[b + 32];
    }
    if (b < (int)gridDim.x) s0 += p[b];
    return warp_sum(s0 + s1);
}

// Panel of the tridiagonalisation (dlatrd, lower) as one cooperative launch.
// The CTA owns a fixed block of rows [rb0, rb1) of [j0, n) for the whole panel
// and keeps their V, W, y and updated-column entries in shared memory; only
// reductions over all rows and the head row of each reflector go through
// global memory.  Shared memory: v (n doubles) | V rows | W rows (R x NB each) | y | a.
// x = head + tail with |x - head - tail| <= 2^-48 |x|
// (head, tail) floats of x: the bits of (RN(x), RN(x - RN(x))), by integer
// arithmetic where it covers x (dfbits.cuh), else by FP64 conversions
__device__ __forceinline__ float2 df_split(double x)
{
    uint32_t hb, lb;
    if (dfb::split(x, &hb, &lb)) return make_float2(__uint_as_float(hb), __uint_as_float(lb));
    const float h = __double2float_rn(x);
    return make_float2(h, __double2float_rn(x - (double)h));
}

__global__ void __launch_bounds__(TRD_THREADS, 1) k_trd_panel(TrdArgs g)
{
    extern __shared__ double sm[];
    __shared__ double s_pq[2 * TRD_NB + 2];
    __shared__ double s_vi[TRD_NB], s_wi[TRD_NB];
    __shared__ double s_red[TRD_WARPS];
    __shared__ double s_scal[4];
    __shared__ double s_pp[8][2 * TRD_NB + 1];  // partial dot products per row group

    const int n = g.n, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int G = gridDim.x, b = blockIdx.x;
    const int R = (n - g.j0 + G - 1) / G;
    const int rb0 = min(n, g.j0 + b * R), rb1 = min(n, rb0 + R);
    float *svh = reinterpret_cast<float *>(sm), *svl = svh + n;  // the column a as head, tail (v = scale a)
    double *Vs = sm + n, *Ws = Vs + (size_t)R * VLD, *ys = Ws + (size_t)R * VLD, *as = ys + R;
    for (int e = tid; e < 2 * R * VLD; e += blockDim.x) Vs[e] = 0.0;
    __syncthreads();

    double apre = 0.0;  // this thread's row of the next column of A, loaded one phase early
    for (int c = 0; c <= g.nbp; c++) {
        const int i = g.j0 + c;  // column reduced now; head row of reflector c - 1
        const int x0 = max(rb0, i);
        double nrm = 0.0;
        // ---------------- phase X: finish w of column c - 1, update column i
        if (c > 0) {
            const int cp = c - 1;
            const int ncomp = 2 * cp + 1;
            // the head row's V, W entries and y, loaded before the reduction so that their
            // latency overlaps it (written before the last grid barrier)
            double vi = 0.0, wi = 0.0, yi = 0.0, taup = 0.0;
            if (warp == 0) {
                if (lane < c) {
                    vi = g.V[(size_t)i * LDP + lane];
                    wi = g.W[(size_t)i * LDP + lane];
                }
                yi = g.y[i];
                taup = g.tau[i - 1];
            }
            {   // grid sums of the previous phase's partials, 8 threads per component
                const int ci = tid >> 3, sub = tid & 7;
                double s = 0.0;
                if (ci < ncomp) {
                    const int comp = ci < cp ? ci : (ci < 2 * cp ? TRD_NB + (ci - cp) : 2 * TRD_NB);
                    const double *pp = g.part + (size_t)comp * G;
                    // four independent chains (GB300's FP64 additions have a long latency)
                    double s4[4] = {0.0, 0.0, 0.0, 0.0};
                    int bb = sub;
                    for (; bb + 24 < G; bb += 32)
#pragma unroll
                        for (int u = 0; u < 4; u++) s4[u] += pp[bb + 8 * u];
                    if (bb < G) s4[0] += pp[bb];
                    if (bb + 8 < G) s4[1] += pp[bb + 8];
                    if (bb + 16 < G) s4[2] += pp[bb + 16];
                    s = (s4[0] + s4[1]) + (s4[2] + s4[3]);
                }
                s += __shfl_xor_sync(0xffffffffu, s, 1);
                s += __shfl_xor_sync(0xffffffffu, s, 2);
                s += __shfl_xor_sync(0xffffffffu, s, 4);
                if (ci < ncomp && sub == 0) s_pq[ci] = s;  // p[0..cp), q[0..cp), y.v
            }
            __syncthreads();
            const double *p = s_pq, *q = s_pq + cp;
            if (warp == 0) {
                double pq = 0.0, hv = 0.0;
                if (lane < cp) {
                    pq = p[lane] * q[lane];
                    hv = vi * q[lane] + wi * p[lane];
                }
                pq = warp_sum(pq);
                hv = warp_sum(hv);
                const double yvc = s_pq[2 * cp] - 2.0 * pq;  // (corrected y).v
                // w of row i (head row: v = 1 there), computed by every CTA alike
                const double whead = taup * (yi - hv) - 0.5 * taup * taup * yvc;
                if (lane == 0) { s_scal[0] = yvc; s_scal[1] = whead; s_scal[3] = taup; }
                if (c < g.nbp && lane < c) {
                    s_vi[lane] = vi;
                    s_wi[lane] = (lane == cp) ? whead : wi;
                }
            }
            __syncthreads();
            const double taup_all = s_scal[3];
            const double yvc = s_scal[0], whead = s_scal[1];
            // four threads per row: the row's w entry and its updated column entry, each a sum
            // over the panel's columns, the threads taking every fourth term in two chains and
            // adding through two shuffles (short FP64 dependency chains on few warps: the FP64
            // pipe of an SM takes one warp instruction per 16 cycles on GB300)
            const int nrows = rb1 - x0, sub = tid & 3;
            for (int rb = 0; rb < nrows; rb += TRD_THREADS / 4) {
                const int rr = rb + (tid >> 2), r = x0 + rr;
                const bool ok = rr < nrows;
                const int lr = ok ? r - rb0 : 0;
                const double *Vr = Vs + (size_t)lr * VLD, *Wr = Ws + (size_t)lr * VLD;
                double a0 = 0.0, a1 = 0.0;
                if (ok)
                    for (int t = sub; t < cp; t += 8) {
                        a0 = fma(Vr[t], q[t], fma(Wr[t], p[t], a0));
                        if (t + 4 < cp) a1 = fma(Vr[t + 4], q[t + 4], fma(Wr[t + 4], p[t + 4], a1));
                    }
                double pa = a0 + a1;
                pa += __shfl_xor_sync(0xffffffffu, pa, 1);
                pa += __shfl_xor_sync(0xffffffffu, pa, 2);
                const double wr = ok ? ((r == i) ? whead : taup_all * (ys[lr] - pa) - 0.5 * taup_all * taup_all * yvc * Vr[cp]) : 0.0;
                if (c < g.nbp) {
                    double b0 = 0.0, b1 = 0.0;
                    if (ok)
                        for (int t = sub; t < c; t += 8) {
                            b0 = fma(Vr[t], s_wi[t], fma(t == cp ? wr : Wr[t], s_vi[t], b0));
                            if (t + 4 < c) b1 = fma(Vr[t + 4], s_wi[t + 4], fma(t + 4 == cp ? wr : Wr[t + 4], s_vi[t + 4], b1));
                        }
                    double pb = b0 + b1;
                    pb += __shfl_xor_sync(0xffffffffu, pb, 1);
                    pb += __shfl_xor_sync(0xffffffffu, pb, 2);
                    if (ok && sub == 0) {
                        const double x = ((rb == 0) ? apre : g.A[(size_t)r * n + i]) - pb;
                        as[lr] = x;
                        g.a[r] = x;
                        g.ahl[r] = df_split(x);
                        if (r >= i + 2) nrm += x * x;
                    }
                }
                __syncwarp();
                if (ok && sub == 0) {
                    Ws[(size_t)lr * VLD + cp] = wr;
                    g.W[(size_t)r * LDP + cp] = wr;
                }
            }
            if (c == g.nbp) break;
        } else {
            for (int r = x0 + tid; r < rb1; r += blockDim.x) {
                const double x = g.A[(size_t)r * n + i];
                as[r - rb0] = x;
                g.a[r] = x;
                g.ahl[r] = df_split(x);
                if (r >= i + 2) nrm += x * x;
            }
        }
        if (x0 + 8 * warp < rb1) nrm = warp_sum(nrm);  // only the warps that hold rows
        if (lane == 0) s_red[warp] = nrm;
        __syncthreads();
        if (tid == 0) {
            double s4[4];
#pragma unroll
            for (int u = 0; u < 4; u++)
                s4[u] = (s_red[u] + s_red[u + 4]) + (s_red[u + 8] + s_red[u + 12]);
            g.part[(size_t)(2 * TRD_NB + 1) * G + b] = (s4[0] + s4[1]) + (s4[2] + s4[3]);
        }
        if (!grid_barrier(g.bar, g.err)) return;

        // ---------------- phase Y: reflector of column i, y = A v on the trailing matrix
        {   // the next column's A entry of this thread's row (A does not change during the panel;
            // rows of four threads, the first keeps it)
            const int rn = max(rb0, i + 1) + (tid >> 2);
            if ((tid & 3) == 0 && c + 1 < g.nbp && rn < rb1) apre = g.A[(size_t)rn * n + i + 1];
        }
        if (warp == 0) {
            const double alpha = (lane == 0) ? g.a[i + 1] : 0.0;  // issued before the reduction
            const double sig = grid_total(g.part, 2 * TRD_NB + 1, lane);
            if (lane == 0) {
                double beta, tau, scale;
                if (sig == 0.0) {
                    beta = alpha; tau = 0.0; scale = 0.0;
                } else {
                    beta = -copysign(sqrt(alpha * alpha + sig), alpha);
                    tau = (beta - alpha) / beta;
                    scale = 1.0 / (alpha - beta);
                }
                s_scal[2] = scale;
                if (b == 0) {
                    g.d[i] = g.a[i];
                    g.e[i] = beta;
                    g.tau[i] = tau;
                }
            }
        }
        __syncthreads();
        const double scale = s_scal[2];
        const int m = n - i - 1;  // trailing size
        // v = (1, scale a[i+2..n)): the gemv uses a as double-float pairs and applies scale at the end
        for (int k = tid; k < m; k += blockDim.x) {
            const float2 h = (k == 0) ? make_float2(0.f, 0.f) : g.ahl[i + 1 + k];
            svh[k] = h.x;
            svl[k] = h.y;
        }
        __syncthreads();
        const int y0 = max(rb0, i + 1);
        // warp per row: y[r] = A[r][i+1] + scale sum_{k>=1} A[r][i+1+k] a[i+1+k], the sum in
        // double-float FP32 arithmetic (products split exactly by FMA, heads added by TwoSum):
        // about 2^-47 relative to sum |A a|, at the FP32 rate instead of GB300's FP64 rate
        const int nrw = (rb1 - y0 - warp + TRD_WARPS - 1) / TRD_WARPS;  // this warp's rows
        for (int rk = 0; rk < nrw; rk++) {
            const int r = y0 + warp + TRD_WARPS * ((c & 1) ? nrw - 1 - rk : rk);
            const float2 *Ar = g.Ahl + (size_t)r * n + i + 1;
            // elements k = kb.. as 16-byte pairs (four loads of 512 B per warp in flight);
            // an unaligned element k = 1 and an odd last element go to lane 0
            const int kb = (((size_t)r * n + i + 2) & 1) ? 2 : 1;
            const int npair = (m - kb) / 2;
            const float4 *A4 = reinterpret_cast<const float4 *>(Ar + kb);
            const float *vbh = svh + kb, *vbl = svl + kb;  // scalar shared-memory reads (kb may be odd)
            float sh[8], sl[8];
#pragma unroll
            for (int u = 0; u < 8; u++) { sh[u] = 0.f; sl[u] = 0.f; }
            auto acc = [&](float ah, float al, float vh, float vl, float &h, float &l) {
                const float p = ah * vh;
                float e = fmaf(ah, vh, -p);
                e = fmaf(ah, vl, e);
                e = fmaf(al, vh, e);
                const float t = h + p, bp = t - h;
                l += ((h - (t - bp)) + (p - bp)) + e;
                h = t;
            };
            // eight 16-byte loads in flight per lane, the last partial block predicated; odd
            // columns walk the rows backwards, so they start on the data the previous column
            // read last (still in L2)
            const int nfull = npair / (8 * 32);
            auto block = [&](int jb, bool tail) {
                const int j = jb * (8 * 32) + lane;
                float4 x[8];
#pragma unroll
                for (int u = 0; u < 8; u++)
                    x[u] = (!tail || j + 32 * u < npair) ? A4[j + 32 * u] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    if (!tail || j + 32 * u < npair) {
                        const int e = 2 * (j + 32 * u);
                        acc(x[u].x, x[u].y, vbh[e], vbl[e], sh[2 * (u & 3)], sl[2 * (u & 3)]);
                        acc(x[u].z, x[u].w, vbh[e + 1], vbl[e + 1], sh[2 * (u & 3) + 1], sl[2 * (u & 3) + 1]);
                    }
                }
            };
            const bool tail = nfull * (8 * 32) < npair;
            if (c & 1) {
                if (tail) block(nfull, true);
                for (int jb = nfull - 1; jb >= 0; jb--) block(jb, false);
            } else {
                for (int jb = 0; jb < nfull; jb++) block(jb, false);
                if (tail) block(nfull, true);
            }
            if (lane == 0) {
                if (kb == 2 && m > 1) {
                    const float2 x = Ar[1];
                    acc(x.x, x.y, svh[1], svl[1], sh[2], sl[2]);
                }
                if (kb + 2 * npair < m) {
                    const int k = kb + 2 * npair;
                    const float2 x = Ar[k];
                    acc(x.x, x.y, svh[k], svl[k], sh[3], sl[3]);
                }
            }
            // the lane's eight (head, tail) sums combined in double-FP32 (TwoSum), so that only
            // one conversion and the warp sum use the FP64 pipe (one warp instruction per 16
            // cycles of an SM on GB300)
            float hh = sh[0], hl = sl[0];
#pragma unroll
            for (int u = 1; u < 8; u++) {
                const float t = hh + sh[u], bp = t - hh;
                const float e = ((hh - (t - bp)) + (sh[u] - bp)) + (hl + sl[u]);
                hh = t + e;
                hl = e - (hh - t);
            }
            // the warp's sum in double-FP32 as well (short FP32 dependency chains instead of
            // FP64 ones), converted once
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, hh, o), ol = __shfl_xor_sync(0xffffffffu, hl, o);
                const float t = hh + oh, bp = t - hh;
                const float e = ((hh - (t - bp)) + (oh - bp)) + (hl + ol);
                hh = t + e;
                hl = e - (hh - t);
            }
            const double ssum = (double)hh + (double)hl;
            if (lane == 0) {
                const float2 a0 = Ar[0];
                const double s = fma(scale, ssum, (double)a0.x + (double)a0.y);
                const int lr = r - rb0;
                const double vr = (r == i + 1) ? 1.0 : as[lr] * scale;
                ys[lr] = s;
                g.y[r] = s;
                Vs[(size_t)lr * VLD + c] = vr;
                g.V[(size_t)r * LDP + c] = vr;
            }
        }
        __syncthreads();
        // partials over this CTA's rows: p_t = V[:,t].v, q_t = W[:,t].v (t < c), y.v;
        // all components at once: thread (group gq of 8, component t), the 8 groups'
        // sums added in order through shared memory
        const int ncomp = 2 * c + 1;
        {
            const int gq = tid >> 6;
            double sp[2] = {0.0, 0.0};
            for (int r = y0 + gq; r < rb1; r += 8) {
                const int lr = r - rb0;
                const double vr = Vs[(size_t)lr * VLD + c];  // v of the row, stored with the product
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int t = (tid & 63) + 64 * h;
                    if (t < ncomp) {
                        const double x = t < c ? Vs[(size_t)lr * VLD + t]
                                               : (t < 2 * c ? Ws[(size_t)lr * VLD + (t - c)] : ys[lr]);
                        sp[h] += x * vr;
                    }
                }
            }
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int t = (tid & 63) + 64 * h;
                if (t < ncomp) s_pp[gq][t] = sp[h];
            }
            __syncthreads();
            if (tid < ncomp) {
                double sum = 0.0;
                for (int q8 = 0; q8 < 8; q8++) sum += s_pp[q8][tid];
                const int comp = tid < c ? tid : (tid < 2 * c ? TRD_NB + (tid - c) : 2 * TRD_NB);
                g.part[(size_t)comp * G + b] = sum;
            }
        }
        if (!grid_barrier(g.bar, g.err)) return;
    }
}

// The trailing block [s, n) x [s, n) as double-float pairs, both triangles,
// from the FP64 lower triangle: one CTA per lower 32 x 32 tile writes the
// tile and its transpose (the diagonal tile reflects within itself).  The
// pairs come from the integer split (one pass of integer instructions per
// element instead of four FP64 conversions and subtractions).
__global__ void k_trail_hilo(const double *__restrict__ A, int n, int s, float2 *__restrict__ Ahl)
{
    __shared__ double tile[32][33];
    const int tr = blockIdx.y, tc = blockIdx.x;
    if (tc > tr) return;
    const int r0 = s + tr * 32, c0 = s + tc * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
    for (int k = ty; k < 32; k += 8) {
        const int rr = r0 + k, cc = c0 + tx;
        tile[k][tx] = (rr < n && cc < n && cc <= rr) ? A[(size_t)rr * n + cc] : 0.0;
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const int rr = r0 + k, cc = c0 + tx;  // (rr, cc) in this tile
        if (rr < n && cc < n) {
            const double v = (tc < tr || tx <= k) ? tile[k][tx] : tile[tx][k];
            Ahl[(size_t)rr * n + cc] = df_split(v);
        }
        if (tc < tr) {
            const int rt = c0 + k, ct = r0 + tx;  // (rt, ct) in the transposed tile
            if (rt < n && ct < n) Ahl[(size_t)rt * n + ct] = df_split(tile[tx][k]);
        }
    }
}

__global__ void k_copy_last_diag(const double *A, int n, double *d)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) d[n - 1] = A[(size_t)(n - 1) * n + (n - 1)];
}

// After a panel: Psw = [W V] (the halves of the panel rows swapped, for
// A22 -= [V W] [W V]^T) and the panel's reflectors into columns j0.. of VA.
__global__ void k_panel_post(int n, int j0, int nbp, const double *__restrict__ P, double *__restrict__ Psw,
                             double *__restrict__ VA, long ldva)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n * LDP) return;
    const int r = (int)(e / LDP), c = (int)(e % LDP);
    Psw[e] = P[(size_t)r * LDP + (c < TRD_NB ? c + TRD_NB : c - TRD_NB)];
    if (c < nbp) VA[(size_t)r * ldva + j0 + c] = P[e];
}

// Compact-WY factor of a block of reflectors (LAPACK dlarft, forward, columnwise):
// T[:, c] = -tau_c T[0:c, 0:c] G[0:c, c],  T[c][c] = tau_c, with G = V^T V the
// block's Gram matrix (T: NBB x NBB per block; one CTA per block, columns in order).
__global__ void __launch_bounds__(256) k_larft(int nv, const double *__restrict__ G, long ldg,
                                               const double *__restrict__ tau, double *__restrict__ T)
{
    const int bb = blockIdx.x, j0 = bb * NBB, w = min(NBB, nv - j0);
    const double *Gb = G + (size_t)j0 * ldg + j0;
    double *Tb = T + (size_t)bb * NBB * NBB;
    __shared__ double col[NBB];
    for (int e = threadIdx.x; e < NBB * NBB; e += blockDim.x) Tb[e] = 0.0;
    __syncthreads();
    for (int c = 0; c < w; c++) {
        const double tc = tau[j0 + c];
        for (int u = threadIdx.x; u < c; u += blockDim.x) col[u] = Gb[(size_t)u * ldg + c];
        __syncthreads();
        for (int t = threadIdx.x; t < c; t += blockDim.x) {
            double s = 0.0;
            for (int u = t; u < c; u++) s = fma(Tb[(size_t)t * NBB + u], col[u], s);
            Tb[(size_t)t * NBB + c] = -tc * s;
        }
        if (threadIdx.x == 0) Tb[(size_t)c * NBB + c] = tc;
        __syncthreads();
    }
}

// The T factors of the blocks of NBW reflectors from the two NBB blocks each
// holds: T = [[T1, T12], [0, T2]] (T12 = -T1 (V1^T V2) T2 is added by two
// products afterwards); grid (NBW * NBW / 256, blocks).
__global__ void k_tw_assemble(int nv, const double *__restrict__ TB, double *__restrict__ TW)
{
    const int k = blockIdx.y, j0 = k * NBW, w = min(NBW, nv - j0);
    const int e = blockIdx.x * blockDim.x + threadIdx.x, row = e / NBW, col = e % NBW;
    if (e >= NBW * NBW) return;
    double v = 0.0;
    if (row < NBB && col < NBB) v = TB[(size_t)(2 * k) * NBB * NBB + (size_t)row * NBB + col];
    else if (row >= NBB && col >= NBB && w > NBB)
        v = TB[(size_t)(2 * k + 1) * NBB * NBB + (size_t)(row - NBB) * NBB + (col - NBB)];
    TW[(size_t)k * NBW * NBW + e] = v;
}

// ------------------------------------------------------------------ stage 2

struct MergeInfo {
    int a, m, b;                 // segment [a, b) = [a, m) + [m, b)
    int kk, k1, k2, nd, ng;      // kept (non-deflated): k1 supported on the first half only, k2 on
                                 // both (rotated across the halves), the rest on the second half;
                                 // deflated; rotations
    double rho;
};

__global__ void k_dc_leaves(int n, const double *__restrict__ d, const double *__restrict__ e, double *__restrict__ lam)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = d[i];
    if (i > 0) v -= fabs(e[i - 1]);
    if (i < n - 1) v -= fabs(e[i]);
    lam[i] = v;
}

__global__ void k_dc_eye(int n, double *Z)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n * n) return;
    Z[e] = ((e / n) == (e % n)) ? 1.0 : 0.0;
}

struct DcWork {
    double *lam, *Z, *Zn, *U, *Zc, *e;
    int n;
    int *srt;        // [n] sorted slot -> source row
    double *Ds, *zs; // [n] sorted values and z after deflation
    int *kl;         // [n] kept j -> sorted slot (ascending)
    int *kci;        // [n] kept j -> grouped column (first-half, both-halves, second-half support)
    int *flg;        // [n] sorted slot -> support: 1 first half, 2 second half, 3 both
    int *dl;         // [n] deflated t -> sorted slot
    int2 *grot;      // [n] rotations (slot p, slot q)
    double2 *gcs;    // [n] (c, s)
    double *kd, *kw; // [n] kept values and z, compact
    int *org;        // [n] root j -> origin kept index
    double *rtau;    // [n] root j -> offset from its origin
    double *zh;      // [n] zhat of kept j
    int *rank;       // [n] root j (pos a+j) / deflated t (pos a+kk+t) -> final position in [a, b)
    MergeInfo *mi;   // per merge of the level
    int *pos2m;      // [n] position -> merge index of the level
    int *err;
};

// Sort, deflate and compact one merge (one CTA per merge).
// The serial part of the deflation (Dongarra-Sorensen: small z components,
// then Givens rotations of close pairs) on D, z and the support flags of one
// merge, from shared memory when they fit (fl: FT = unsigned char) or global
// memory (FT = int); the kept list is written to kl, its flags to kf.
template <typename FT>
__device__ void dc_deflate_serial(DcWork &w, MergeInfo &M, int a, int k, double rho, double zm, double tol, double *D,
                                  double *z, FT *fl, FT *kf)
{
    int kk = 0, nd = 0, ng = 0, k1 = 0, k2 = 0;
    if (rho * zm <= tol) {
        for (int s = 0; s < k; s++) w.dl[a + nd++] = a + s;
    } else {
        int pj = -1;
        for (int nj = 0; nj < k; nj++) {
            if (rho * fabs(z[nj]) <= tol) { w.dl[a + nd++] = a + nj; continue; }
            if (pj < 0) { pj = nj; continue; }
            // |t c s| <= tol with c = z_nj / tau, s = -z_pj / tau, tau^2 = z_pj^2 + z_nj^2,
            // tested without the square root and divisions (on GB300's slow FP64 pipe);
            // the rotation is formed only for the pairs that deflate
            const double zp = z[pj], zn = z[nj], t = D[nj] - D[pj];
            const double r2 = zp * zp + zn * zn;
            if (fabs(t) * fabs(zp * zn) <= tol * r2) {
                const double tau = sqrt(r2);
                const double c = zn / tau, s = -zp / tau;
                fl[nj] |= fl[pj];  // the rotated vector has support on both halves
                z[nj] = tau;
                z[pj] = 0.0;
                w.grot[a + ng] = make_int2(a + pj, a + nj);
                w.gcs[a + ng] = make_double2(c, s);
                ng++;
                const double t2 = D[pj] * c * c + D[nj] * s * s;
                D[nj] = D[pj] * s * s + D[nj] * c * c;
                D[pj] = t2;
                w.dl[a + nd++] = a + pj;
                pj = nj;
            } else {
                // a kept entry's flag is final (later rotations only change the newer entry)
                k1 += (fl[pj] == 1);
                k2 += (fl[pj] == 3);
                kf[kk] = fl[pj];
                w.kl[a + kk++] = a + pj;
                pj = nj;
            }
        }
        if (pj >= 0) {
            k1 += (fl[pj] == 1);
            k2 += (fl[pj] == 3);
            kf[kk] = fl[pj];
            w.kl[a + kk++] = a + pj;
        }
    }
    M.kk = kk; M.k1 = k1; M.k2 = k2; M.nd = nd; M.ng = ng; M.rho = rho;
}

// One CTA per merge.  Shared memory (when the merge fits, DC_DEFL_SMEM): D, z
// [k] doubles, support flags and kept flags [k] bytes.
__global__ void __launch_bounds__(256) k_dc_deflate(DcWork w, int use_smem)
{
    extern __shared__ double dsm[];
    MergeInfo &M = w.mi[blockIdx.x];
    const int a = M.a, m = M.m, b = M.b, k = b - a, n = w.n;
    const int tid = threadIdx.x;
    const double em = w.e[m - 1];
    const double rho = 2.0 * fabs(em);
    const double sg = em >= 0.0 ? 1.0 : -1.0;
    const double rs = 0.70710678118654752440;
    double *Dsh = dsm, *zsh = dsm + k;
    unsigned char *fsh = reinterpret_cast<unsigned char *>(dsm + 2 * k), *kfsh = fsh + k;
    // merge the two ascending halves (stable: ties take the first half first)
    for (int t = tid; t < k; t += blockDim.x) {
        const int src = a + t;
        const double v = w.lam[src];
        int lo, hi, rk;
        if (src < m) {
            lo = m; hi = b;  // count of second-half values < v
            while (lo < hi) { const int md = (lo + hi) >> 1; if (w.lam[md] < v) lo = md + 1; else hi = md; }
            rk = (src - a) + (lo - m);
        } else {
            lo = a; hi = m;  // count of first-half values <= v
            while (lo < hi) { const int md = (lo + hi) >> 1; if (w.lam[md] <= v) lo = md + 1; else hi = md; }
            rk = (src - m) + (lo - a);
        }
        const double zv = (src < m ? w.Z[(size_t)src * n + (m - 1)] : sg * w.Z[(size_t)src * n + m]) * rs;
        w.srt[a + rk] = src;
        if (use_smem) {
            Dsh[rk] = v;
            zsh[rk] = zv;
            fsh[rk] = src < m ? 1 : 2;
        } else {
            w.flg[a + rk] = src < m ? 1 : 2;
            w.Ds[a + rk] = v;
            w.zs[a + rk] = zv;
        }
    }
    __syncthreads();
    const double *Dr = use_smem ? Dsh : w.Ds + a, *zr = use_smem ? zsh : w.zs + a;
    __shared__ double s_mx[2][8];
    double dm = 0.0, zm = 0.0;
    for (int t = tid; t < k; t += blockDim.x) {
        dm = fmax(dm, fabs(Dr[t]));
        zm = fmax(zm, fabs(zr[t]));
    }
    dm = warp_max(dm);
    zm = warp_max(zm);
    if ((tid & 31) == 0) { s_mx[0][tid >> 5] = dm; s_mx[1][tid >> 5] = zm; }
    __syncthreads();
    if (tid == 0) {
        for (int t = 1; t < (int)(blockDim.x >> 5); t++) { dm = fmax(dm, s_mx[0][t]); zm = fmax(zm, s_mx[1][t]); }
        const double tol = 8.0 * EPS * fmax(dm, zm);
        if (use_smem)
            dc_deflate_serial<unsigned char>(w, M, a, k, rho, zm, tol, Dsh, zsh, fsh, kfsh);
        else
            dc_deflate_serial<int>(w, M, a, k, rho, zm, tol, w.Ds + a, w.zs + a, w.flg + a, w.kci + a);
    }
    __syncthreads();
    const int kk = M.kk, k1 = M.k1, k2 = M.k2;
    if (use_smem)  // the rotated D, z and flags back for the later kernels
        for (int t = tid; t < k; t += blockDim.x) {
            w.Ds[a + t] = Dsh[t];
            w.zs[a + t] = zsh[t];
            w.flg[a + t] = fsh[t];
        }
    if (tid != 0) return;
    // compact kept values; grouped columns: first-half support, both halves, second half
    int cg[4] = {0, 0, k1 + k2, k1};
    for (int j = 0; j < kk; j++) {
        const int sl = w.kl[a + j];
        w.kd[a + j] = use_smem ? Dsh[sl - a] : w.Ds[sl];
        w.kw[a + j] = use_smem ? zsh[sl - a] : w.zs[sl];
        w.kci[a + j] = cg[use_smem ? kfsh[j] : w.kci[a + j]]++;
    }
}

// Apply the deflation rotations of each merge to its eigenvector rows (one
// thread per component column; rotations in order).
__global__ void k_dc_rotate(DcWork w)
{
    const MergeInfo M = w.mi[blockIdx.y];
    const int col = M.a + blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= M.b || M.ng == 0) return;
    const int n = w.n;
    for (int r = 0; r < M.ng; r++) {
        const int2 pq = w.grot[M.a + r];
        const double2 cs = w.gcs[M.a + r];
        double *xp = w.Z + (size_t)w.srt[pq.x] * n + col, *xq = w.Z + (size_t)w.srt[pq.y] * n + col;
        const double x = *xp, y = *xq;
        *xp = cs.x * x + cs.y * y;
        *xq = cs.x * y - cs.y * x;
    }
}

// Secular roots: one warp per position p; root j = p - a of the merge holding p.
__global__ void __launch_bounds__(256) k_dc_secular(DcWork w)
{
    const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (p >= w.n) return;
    const int mix = w.pos2m[p];
    if (mix < 0) return;
    const MergeInfo M = w.mi[mix];
    const int j = p - M.a, kk = M.kk;
    if (j >= kk) return;
    const double *dl = w.kd + M.a, *z = w.kw + M.a;
    const double rho = M.rho;
    int o;
    double lo, hi;
    if (kk == 1) {
        if (lane == 0) { w.org[M.a] = 0; w.rtau[M.a] = rho * z[0] * z[0]; }
        return;
    }
    if (j < kk - 1) {
        const double half = 0.5 * (dl[j + 1] - dl[j]);
        double s = 0.0;
        for (int i = lane; i < kk; i += 32) s += z[i] * z[i] / ((dl[i] - dl[j]) - half);
        s = warp_sum(s);
        const double fmid = 1.0 + rho * s;
        if (fmid >= 0.0) { o = j; lo = 0.0; hi = half; }
        else { o = j + 1; lo = -half; hi = 0.0; }
    } else {
        double s = 0.0;
        for (int i = lane; i < kk; i += 32) s += z[i] * z[i];
        s = warp_sum(s);
        o = kk - 1; lo = 0.0; hi = rho * s;
    }
    const double dorg = dl[o];
    double tau = 0.5 * (lo + hi);
    for (int it = 0; it < 100; it++) {
        double psi = 0.0, phi = 0.0, dpsi = 0.0, dphi = 0.0;
        for (int i = lane; i < kk; i += 32) {
            const double dlt = (dl[i] - dorg) - tau;
            const double rd = 1.0 / dlt;  // one FP64 division per term (GB300's FP64 pipe is slow)
            const double t = z[i] * z[i] * rd;
            if (i <= j) { psi += t; dpsi += t * rd; }
            else { phi += t; dphi += t * rd; }
        }
        psi = rho * warp_sum(psi);
        phi = rho * warp_sum(phi);
        dpsi = rho * warp_sum(dpsi);
        dphi = rho * warp_sum(dphi);
        const double f = 1.0 + psi + phi;
        if (f < 0.0) lo = tau; else hi = tau;
        if (fabs(f) <= 8.0 * EPS * (1.0 + fabs(psi) + fabs(phi))) break;
        if (hi - lo <= 4.0 * EPS * fmax(fabs(lo), fabs(hi))) break;
        double tn = 0.0;
        bool ok = false;
        if (j < kk - 1) {
            const double Dj = (dl[j] - dorg) - tau, Dj1 = (dl[j + 1] - dorg) - tau;
            const double cc = f - Dj * dpsi - Dj1 * dphi;
            const double s1 = Dj * Dj * dpsi, s2 = Dj1 * Dj1 * dphi;
            const double A = cc, B = cc * (Dj + Dj1) + s1 + s2, C = cc * Dj * Dj1 + s1 * Dj1 + s2 * Dj;
            double eta = 0.0;
            bool have = false;
            if (fabs(A) <= EPS * fabs(B)) {
                if (B != 0.0) { eta = C / B; have = true; }
            } else {
                const double disc = B * B - 4.0 * A * C;
                if (disc >= 0.0) {
                    const double r1 = (B + copysign(sqrt(disc), B)) / (2.0 * A);
                    const double r2 = (r1 != 0.0) ? C / (A * r1) : 0.0;
                    const bool in1 = (r1 > Dj && r1 < Dj1), in2 = (r2 > Dj && r2 < Dj1);
                    if (in1 && in2) { eta = fabs(r1) < fabs(r2) ? r1 : r2; have = true; }
                    else if (in1) { eta = r1; have = true; }
                    else if (in2) { eta = r2; have = true; }
                }
            }
            if (have) { tn = tau + eta; ok = true; }
        } else {
            const double Dk = (dl[kk - 1] - dorg) - tau;
            const double cc = f - Dk * dpsi;
            if (cc > 0.0) { tn = tau + Dk + Dk * Dk * dpsi / cc; ok = true; }
        }
        if (!ok || !(tn > lo && tn < hi)) tn = 0.5 * (lo + hi);
        tau = tn;
    }
    if (lane == 0) { w.org[M.a + j] = o; w.rtau[M.a + j] = tau; }
}

// Gu-Eisenstat: zhat_i^2 = -Delta_ii / rho * prod_{j != i} Delta_ij / (d_i - d_j),
// Delta_ij = d_i - lambda_j = (d_i - d_org(j)) - tau_j.  One warp per kept i.
__global__ void __launch_bounds__(256) k_dc_zhat(DcWork w)
{
    const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (p >= w.n) return;
    const int mix = w.pos2m[p];
    if (mix < 0) return;
    const MergeInfo M = w.mi[mix];
    const int i = p - M.a, kk = M.kk;
    if (i >= kk) return;
    const double *dl = w.kd + M.a;
    const int *org = w.org + M.a;
    const double *rt = w.rtau + M.a;
    const double di = dl[i];
    double pr = 1.0;
    for (int j = lane; j < kk; j += 32) {
        const double dij = (di - dl[org[j]]) - rt[j];
        pr *= (j == i) ? -dij / M.rho : dij / (di - dl[j]);
    }
    pr = warp_prod(pr);
    if (lane == 0) w.zh[M.a + i] = copysign(sqrt(fabs(pr)), w.kw[M.a + i]);
}

// Row j of U (the eigenvector of root j in the kept basis, grouped columns):
// U[a+j][a+kci(i)] = zhat_i / Delta_ij, normalised.  One warp per root.
__global__ void __launch_bounds__(256) k_dc_vectors(DcWork w)
{
    const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (p >= w.n) return;
    const int mix = w.pos2m[p];
    if (mix < 0) return;
    const MergeInfo M = w.mi[mix];
    const int j = p - M.a, kk = M.kk, n = w.n;
    if (j >= kk) return;
    const double *dl = w.kd + M.a;
    const double dorg = dl[w.org[M.a + j]], tau = w.rtau[M.a + j];
    double *Ur = w.U + (size_t)(M.a + j) * n + M.a;
    double s = 0.0;
    for (int i = lane; i < kk; i += 32) {
        const double v = w.zh[M.a + i] / ((dl[i] - dorg) - tau);
        Ur[w.kci[M.a + i]] = v;
        s += v * v;
    }
    s = warp_sum(s);
    const double inv = 1.0 / sqrt(s);
    __syncwarp();
    for (int i = lane; i < kk; i += 32) Ur[w.kci[M.a + i]] *= inv;
}

// Final positions: roots (ascending) and deflated values merged by rank; new
// eigenvalues written; the gathered kept rows Zc[a + kci] = Z[srt[kept]].
__global__ void __launch_bounds__(256) k_dc_rank(DcWork w)
{
    const MergeInfo M = w.mi[blockIdx.y];
    const int k = M.b - M.a, kk = M.kk, nd = M.nd;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= k) return;
    auto val = [&](int x) -> double {
        if (x < kk) return w.kd[M.a + w.org[M.a + x]] + w.rtau[M.a + x];
        return w.Ds[w.dl[M.a + (x - kk)]];
    };
    const double v = val(t);
    int r = 0;
    for (int x = 0; x < kk + nd; x++) {
        const double u = val(x);
        r += (u < v) || (u == v && x < t);
    }
    w.rank[M.a + t] = M.a + r;
}

__global__ void k_dc_lam(DcWork w)
{
    const MergeInfo M = w.mi[blockIdx.y];
    const int k = M.b - M.a, kk = M.kk;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= k) return;
    const double v = t < kk ? w.kd[M.a + w.org[M.a + t]] + w.rtau[M.a + t] : w.Ds[w.dl[M.a + (t - kk)]];
    w.lam[w.rank[M.a + t]] = v;
}

// Gather kept rows into Zc (grouped order) and copy deflated rows to their
// final positions in Zn.  Grid: (column blocks, rows of the merge, merges).
__global__ void k_dc_gather(DcWork w)
{
    const MergeInfo M = w.mi[blockIdx.z];
    const int t = blockIdx.y, n = w.n;
    const int col = M.a + blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= M.b || t >= M.b - M.a) return;
    if (t < M.kk) {
        const int src = w.srt[w.kl[M.a + t]];
        w.Zc[(size_t)(M.a + w.kci[M.a + t]) * n + col] = w.Z[(size_t)src * n + col];
    } else {
        const int dt = t - M.kk;
        const int src = w.srt[w.dl[M.a + dt]];
        w.Zn[(size_t)w.rank[M.a + t] * n + col] = w.Z[(size_t)src * n + col];
    }
}

// Grouped FP64 GEMM for the merges of a level: for merge g and half h,
//   Zn[rank[a+j]][cols of half h] = sum_c U[a+j][a+c0+c] Zc[a+c0+c][cols of half h]
// with c over the kept vectors supported on that half (first half: groups
// first-only and both; second half: both and second-only).  64x64 tiles, 4x4
// per thread.
constexpr int DT = 64, DK = 16;
__global__ void __launch_bounds__(256) k_dc_gemm(DcWork w)
{
    const MergeInfo M = w.mi[blockIdx.z >> 1];
    const int h = blockIdx.z & 1;
    const int n = w.n;
    const int kk = M.kk;
    const int c0 = h ? M.k1 : 0, K = h ? kk - M.k1 : M.k1 + M.k2;
    const int colb = h ? M.m : M.a, ncol = h ? M.b - M.m : M.m - M.a;
    const int ntn = (ncol + DT - 1) / DT;
    const int tm = blockIdx.x / ntn, tn = blockIdx.x % ntn;
    if (tm * DT >= kk || tn >= ntn || K == 0) return;
    __shared__ double As[DK][DT + 1];
    __shared__ double Bs[DK][DT + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += DK) {
        for (int e = tid; e < DK * DT; e += 256) {
            const int kq = e % DK, mm = e / DK;
            const int r = tm * DT + mm, kx = k0 + kq;
            As[kq][mm] = (r < kk && kx < K) ? w.U[(size_t)(M.a + r) * n + M.a + c0 + kx] : 0.0;
        }
        for (int e = tid; e < DK * DT; e += 256) {
            const int nn = e % DT, kq = e / DT;
            const int cc = tn * DT + nn, kx = k0 + kq;
            Bs[kq][nn] = (cc < ncol && kx < K) ? w.Zc[(size_t)(M.a + c0 + kx) * n + colb + cc] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kq = 0; kq < DK; kq++) {
            double av[4], bv[4];
#pragma unroll
            for (int x = 0; x < 4; x++) av[x] = As[kq][ty + 16 * x];
#pragma unroll
            for (int y = 0; y < 4; y++) bv[y] = Bs[kq][tx + 16 * y];
#pragma unroll
            for (int x = 0; x < 4; x++)
#pragma unroll
                for (int y = 0; y < 4; y++) acc[x][y] = fma(av[x], bv[y], acc[x][y]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int x = 0; x < 4; x++) {
        const int r = tm * DT + ty + 16 * x;
        if (r >= kk) continue;
        double *dst = w.Zn + (size_t)w.rank[M.a + r] * n + colb;
#pragma unroll
        for (int y = 0; y < 4; y++) {
            const int cc = tn * DT + tx + 16 * y;
            if (cc < ncol) dst[cc] = acc[x][y];
        }
    }
}

// A half with no kept column leaves its part of the new rows zero.
__global__ void k_dc_zero_half(DcWork w)
{
    const MergeInfo M = w.mi[blockIdx.z >> 1];
    const int h = blockIdx.z & 1, n = w.n;
    const int K = h ? M.kk - M.k1 : M.k1 + M.k2;
    if (K != 0) return;
    const int colb = h ? M.m : M.a, ncol = h ? M.b - M.m : M.m - M.a;
    const int r = blockIdx.y, c = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= M.kk || c >= ncol) return;
    w.Zn[(size_t)w.rank[M.a + r] * n + colb + c] = 0.0;
}

// Rows of a large merge's vector update, computed densely into Zt ([kk][b - a],
// row j = root j), moved to their final positions in Zn.
__global__ void k_dc_scatter(DcWork w, int mix, const double *__restrict__ Zt)
{
    const MergeInfo M = w.mi[mix];
    const int j = blockIdx.y, k = M.b - M.a;
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= M.kk || col >= k) return;
    w.Zn[(size_t)w.rank[M.a + j] * w.n + M.a + col] = Zt[(size_t)j * k + col];
}

}  // namespace

// ------------------------------------------------------------------ host side

static void build_tree(int a, int b, int lev, std::vector<std::vector<int3>> &out)
{
    if (b - a <= 1) return;
    const int m = (a + b) / 2;
    if ((int)out.size() <= lev) out.resize(lev + 1);
    build_tree(a, m, lev + 1, out);
    build_tree(m, b, lev + 1, out);
    out[lev].push_back(make_int3(a, m, b));
}

// Carve the eigensolver's workspace out of ctx->eigw for size n.
struct SyevPtrs {
    double *P, *Psw, *VA, *GB, *TB, *TW, *TT, *d, *e, *tau, *a, *y, *part;
    float2 *Ahl, *ahl;
    long ldva;
    unsigned *bar;
    int *err;
    double *lam, *Z, *Zn, *U, *Zc, *Zt;
    int *srt, *kl, *kci, *flg, *dl, *org, *rank, *pos2m;
    double *Ds, *zs, *kd, *kw, *rtau, *zh;
    int2 *grot;
    double2 *gcs;
    MergeInfo *mi;
    int nmerge_total;
};

static size_t carve(uint8_t *base, int n, int npanel, int nlev, int nmerge, SyevPtrs &p)
{
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t r = o; o += (bytes + 255) & ~(size_t)255; return base ? (void *)(base + r) : nullptr; };
    const size_t NN = (size_t)n * n;
    const long nvpad = (long)std::max(1, ceil_div(std::max(1, n - 1), NBW)) * NBW;
    p.ldva = nvpad;
    p.P = (double *)take(sizeof(double) * (size_t)n * LDP);
    p.Ahl = (float2 *)take(sizeof(float2) * NN);
    p.ahl = (float2 *)take(sizeof(float2) * n);
    p.Psw = (double *)take(sizeof(double) * (size_t)n * LDP);
    p.VA = (double *)take(sizeof(double) * (size_t)n * nvpad);          // every reflector, column j = v_j
    p.GB = (double *)take(sizeof(double) * (size_t)nvpad * nvpad);      // diagonal NBW blocks of VA^T VA
    p.TB = (double *)take(sizeof(double) * (size_t)(nvpad / NBB) * NBB * NBB);
    p.TW = (double *)take(sizeof(double) * (size_t)(nvpad / NBW) * NBW * NBW);
    p.TT = (double *)take(sizeof(double) * (size_t)NBB * NBB);
    p.d = (double *)take(sizeof(double) * n);
    p.e = (double *)take(sizeof(double) * n);
    p.tau = (double *)take(sizeof(double) * n);
    p.a = (double *)take(sizeof(double) * n);
    p.y = (double *)take(sizeof(double) * n);
    p.part = (double *)take(sizeof(double) * PCOMP * 1024);
    p.bar = (unsigned *)take(sizeof(unsigned) * 1024);
    p.err = (int *)take(sizeof(int) * 2);
    p.lam = (double *)take(sizeof(double) * n);
    p.Z = (double *)take(sizeof(double) * NN);
    p.Zn = (double *)take(sizeof(double) * NN);
    p.U = (double *)take(sizeof(double) * NN);
    p.Zc = (double *)take(sizeof(double) * NN);
    p.Zt = (double *)take(sizeof(double) * NN);
    p.srt = (int *)take(sizeof(int) * n);
    p.kl = (int *)take(sizeof(int) * n);
    p.kci = (int *)take(sizeof(int) * n);
    p.flg = (int *)take(sizeof(int) * n);
    p.dl = (int *)take(sizeof(int) * n);
    p.org = (int *)take(sizeof(int) * n);
    p.rank = (int *)take(sizeof(int) * n);
    p.pos2m = (int *)take(sizeof(int) * (size_t)n * std::max(1, nlev));
    p.Ds = (double *)take(sizeof(double) * n);
    p.zs = (double *)take(sizeof(double) * n);
    p.kd = (double *)take(sizeof(double) * n);
    p.kw = (double *)take(sizeof(double) * n);
    p.rtau = (double *)take(sizeof(double) * n);
    p.zh = (double *)take(sizeof(double) * n);
    p.grot = (int2 *)take(sizeof(int2) * n);
    p.gcs = (double2 *)take(sizeof(double2) * n);
    p.mi = (MergeInfo *)take(sizeof(MergeInfo) * std::max(1, nmerge));
    p.nmerge_total = nmerge;
    return o;
}

struct SyevState {
    int n = -1;
    std::vector<std::vector<int3>> levels;
    std::vector<int> level_off;
    int nmerge = 0;
};

static modal_status dc_setup(modal_ctx *ctx, int n, SyevState &st, SyevPtrs &p, int npanel)
{
    st.levels.clear();
    build_tree(0, n, 0, st.levels);
    std::reverse(st.levels.begin(), st.levels.end());  // deepest first
    st.level_off.assign(st.levels.size(), 0);
    int nm = 0;
    for (size_t l = 0; l < st.levels.size(); l++) { st.level_off[l] = nm; nm += (int)st.levels[l].size(); }
    st.nmerge = nm;
    const int nlev = (int)st.levels.size();
    size_t need = carve(nullptr, n, npanel, nlev, nm, p);
    MODAL_TRY(ensure(ctx->eigw, need));
    carve(ctx->eigw.as<uint8_t>(), n, npanel, nlev, nm, p);
    // merge descriptors and position -> merge maps for every level
    std::vector<MergeInfo> mi(std::max(1, nm));
    std::vector<int> pos2m((size_t)n * std::max(1, nlev), -1);
    for (int l = 0; l < nlev; l++) {
        for (size_t x = 0; x < st.levels[l].size(); x++) {
            const int3 t = st.levels[l][x];
            MergeInfo M{};
            M.a = t.x; M.m = t.y; M.b = t.z;
            mi[st.level_off[l] + x] = M;
            for (int q = t.x; q < t.z; q++) pos2m[(size_t)l * n + q] = (int)x;
        }
    }
    if (nm > 0)
        MODAL_CUDA(cudaMemcpyAsync(p.mi, mi.data(), sizeof(MergeInfo) * nm, cudaMemcpyHostToDevice, ctx->stream));
    if (nlev > 0)
        MODAL_CUDA(cudaMemcpyAsync(p.pos2m, pos2m.data(), sizeof(int) * pos2m.size(), cudaMemcpyHostToDevice, ctx->stream));
    // the host vectors must outlive the copies
    MODAL_CUDA(cudaStreamSynchronize(ctx->stream));
    return MODAL_OK;
}

static modal_status trd_run(modal_ctx *ctx, int n, double *A, SyevPtrs &p, int npanel)
{
    int dev = ctx->device, nsm = 0, coop = 0;
    MODAL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    MODAL_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) { set_error("eigensolver: the device has no cooperative launch"); return MODAL_ERR_CUDA; }
    // CTAs per panel: one per SM for large trailing matrices, fewer (cheaper
    // barriers and reductions) once the trailing matrix is small
    auto grid_of = [&](int rows) { return std::max(1, std::min(std::min(nsm, 1024), ceil_div(rows, 16))); };
    int Rmax = 1;
    for (int j0 = 0; j0 < n - 1; j0 += TRD_NB) Rmax = std::max(Rmax, ceil_div(n - j0, grid_of(n - j0)));
    // v (n) + this CTA's V and W rows (Rmax x NB each) + y and a (Rmax each)
    const size_t smem = sizeof(double) * ((size_t)n + (size_t)Rmax * (2 * VLD + 2));
    if (smem > 200 * 1024) { set_error("eigensolver: n = %d exceeds the panel kernel's shared memory", n); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaFuncSetAttribute(k_trd_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    MODAL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trd_panel, TRD_THREADS, smem));
    if (per_sm < 1) { set_error("eigensolver: panel kernel does not fit on an SM"); return MODAL_ERR_CUDA; }
    MODAL_CUDA(cudaMemsetAsync(p.err, 0, 2 * sizeof(int), ctx->stream));
    MODAL_CUDA(cudaMemsetAsync(p.bar, 0, 2 * sizeof(unsigned), ctx->stream));
    MODAL_CUDA(cudaMemsetAsync(p.VA, 0, sizeof(double) * (size_t)n * p.ldva, ctx->stream));
    {
        const int nt = ceil_div(n, 32);
        k_trail_hilo<<<dim3(nt, nt), 256, 0, ctx->stream>>>(A, n, 0, p.Ahl);
        MODAL_TRY(launched(ctx, "trail_hilo"));
    }
    MODAL_TRY(oz_reset(ctx));
    OzOpts oz;
    oz.slices = OZ_SLICES;
    oz.lower = 1;
    oz.check = false;
    for (int pi = 0; pi < npanel; pi++) {
        const int j0 = pi * TRD_NB;
        const int nbp = std::min(TRD_NB, n - 1 - j0);  // reflectors 0 .. n-2
        MODAL_CUDA(cudaMemsetAsync(p.P, 0, sizeof(double) * (size_t)n * LDP, ctx->stream));
        TrdArgs g;
        g.A = A; g.Ahl = p.Ahl; g.ahl = p.ahl; g.n = n; g.j0 = j0; g.nbp = nbp;
        g.V = p.P;
        g.W = p.P + TRD_NB;
        g.d = p.d; g.e = p.e; g.tau = p.tau; g.a = p.a; g.y = p.y; g.part = p.part; g.bar = p.bar; g.err = p.err;
        void *args[] = {&g};
        const int G = grid_of(n - j0);
        {
            StageTimer tp(ctx, MODAL_T_EIG_PANEL);
            MODAL_CUDA(cudaLaunchCooperativeKernel((const void *)k_trd_panel, dim3(G), dim3(TRD_THREADS), args, smem,
                                                   ctx->stream));
            MODAL_TRY(launched(ctx, "trd_panel"));
        }
        k_panel_post<<<ceil_div((long)n * LDP, 256), 256, 0, ctx->stream>>>(n, j0, nbp, p.P, p.Psw, p.VA, p.ldva);
        MODAL_TRY(launched(ctx, "panel_post"));
        const int s = j0 + nbp, rest = n - s;
        if (rest > 0) {
            // A22 -= V W^T + W V^T = [V W] [W V]^T on the lower triangle (tensor cores, FP64 accuracy)
            // the same epilogue refreshes the block's (head, tail) float copy, both triangles
            double *A22 = A + (size_t)s * n + s;
            MODAL_TRY(oz_gemm_ex(ctx, rest, rest, LDP, -1.0, p.P + (size_t)s * LDP, LDP, false, p.Psw + (size_t)s * LDP,
                                 LDP, true, 1.0, A22, n, oz));
            const int nt = ceil_div(rest, 32);
            k_trail_hilo<<<dim3(nt, nt), 256, 0, ctx->stream>>>(A, n, s, p.Ahl);
            MODAL_TRY(launched(ctx, "trail_hilo"));
        }
    }
    k_copy_last_diag<<<1, 32, 0, ctx->stream>>>(A, n, p.d);
    return launched(ctx, "copy_last_diag");
}

static modal_status dc_run(modal_ctx *ctx, int n, SyevState &st, SyevPtrs &p)
{
    k_dc_leaves<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(n, p.d, p.e, p.lam);
    MODAL_TRY(launched(ctx, "dc_leaves"));
    // both buffers start as the identity: a row that is still a single-row
    // segment at some level is not written by that level's merges, and its
    // parent reads it from whichever buffer is current then
    k_dc_eye<<<ceil_div((long)n * n, 256), 256, 0, ctx->stream>>>(n, p.Z);
    MODAL_TRY(launched(ctx, "dc_eye"));
    k_dc_eye<<<ceil_div((long)n * n, 256), 256, 0, ctx->stream>>>(n, p.Zn);
    MODAL_TRY(launched(ctx, "dc_eye"));
    double *Z = p.Z, *Zn = p.Zn;
    const int nlev = (int)st.levels.size();
    MODAL_CUDA(cudaFuncSetAttribute(k_dc_deflate, cudaFuncAttributeMaxDynamicSharedMemorySize, DC_DEFL_SMEM));
    for (int l = 0; l < nlev; l++) {
        const int nm = (int)st.levels[l].size();
        int kmax = 0, hmax = 0;
        for (const int3 &t : st.levels[l]) { kmax = std::max(kmax, t.z - t.x); hmax = std::max(hmax, std::max(t.y - t.x, t.z - t.y)); }
        DcWork w;
        w.lam = p.lam; w.Z = Z; w.Zn = Zn; w.U = p.U; w.Zc = p.Zc; w.e = p.e; w.n = n;
        w.srt = p.srt; w.Ds = p.Ds; w.zs = p.zs; w.kl = p.kl; w.kci = p.kci; w.flg = p.flg; w.dl = p.dl; w.grot = p.grot; w.gcs = p.gcs;
        w.kd = p.kd; w.kw = p.kw; w.org = p.org; w.rtau = p.rtau; w.zh = p.zh; w.rank = p.rank;
        w.mi = p.mi + st.level_off[l];
        w.pos2m = p.pos2m + (size_t)l * n;
        w.err = p.err;
        // D, z and flags of the level's largest merge in shared memory when they fit
        const size_t dsmem = (size_t)kmax * (2 * sizeof(double) + 2);
        const int use_smem = dsmem <= (size_t)DC_DEFL_SMEM;
        k_dc_deflate<<<nm, 256, use_smem ? dsmem : 0, ctx->stream>>>(w, use_smem);
        MODAL_TRY(launched(ctx, "dc_deflate"));
        k_dc_rotate<<<dim3(ceil_div(kmax, 128), nm), 128, 0, ctx->stream>>>(w);
        MODAL_TRY(launched(ctx, "dc_rotate"));
        const int wblocks = ceil_div((long)n * 32, 256);
        k_dc_secular<<<wblocks, 256, 0, ctx->stream>>>(w);
        MODAL_TRY(launched(ctx, "dc_secular"));
        k_dc_zhat<<<wblocks, 256, 0, ctx->stream>>>(w);
        MODAL_TRY(launched(ctx, "dc_zhat"));
        k_dc_vectors<<<wblocks, 256, 0, ctx->stream>>>(w);
        MODAL_TRY(launched(ctx, "dc_vectors"));
        k_dc_rank<<<dim3(ceil_div(kmax, 256), nm), 256, 0, ctx->stream>>>(w);
        MODAL_TRY(launched(ctx, "dc_rank"));
        k_dc_gather<<<dim3(ceil_div(kmax, 128), kmax, nm), 128, 0, ctx->stream>>>(w);
        MODAL_TRY(launched(ctx, "dc_gather"));
        if (kmax >= DC_OZ_MIN) {
            // large merges: the two half products on the tensor cores (FP64 accuracy),
            // sized from the merge descriptors
            std::vector<MergeInfo> hm(nm);
            MODAL_CUDA(cudaMemcpyAsync(hm.data(), w.mi, sizeof(MergeInfo) * nm, cudaMemcpyDeviceToHost, ctx->stream));
            MODAL_CUDA(cudaStreamSynchronize(ctx->stream));
            OzOpts o;
            o.slices = OZ_SLICES;
            o.check = false;
            for (int x = 0; x < nm; x++) {
                const MergeInfo &M = hm[x];
                const int k = M.b - M.a, kk = M.kk;
                if (kk == 0) continue;
                const int K0 = M.k1 + M.k2, K1 = kk - M.k1;
                const double *Ub = p.U + (size_t)M.a * n + M.a, *Zb = p.Zc + (size_t)M.a * n;
                if (K0 > 0)
                    MODAL_TRY(oz_gemm_ex(ctx, kk, M.m - M.a, K0, 1.0, Ub, n, false, Zb + M.a, n, false, 0.0, p.Zt, k, o));
                if (K1 > 0)
                    MODAL_TRY(oz_gemm_ex(ctx, kk, M.b - M.m, K1, 1.0, Ub + M.k1, n, false, Zb + (size_t)M.k1 * n + M.m, n,
                                         false, 0.0, p.Zt + (M.m - M.a), k, o));
                k_dc_scatter<<<dim3(ceil_div(k, 128), kk), 128, 0, ctx->stream>>>(w, x, p.Zt);
                MODAL_TRY(launched(ctx, "dc_scatter"));
            }
        } else {
            const long tiles = (long)ceil_div(kmax, DT) * ceil_div(hmax, DT);
            k_dc_gemm<<<dim3((unsigned)tiles, 1, 2 * nm), 256, 0, ctx->stream>>>(w);
            MODAL_TRY(launched(ctx, "dc_gemm"));
        }
        k_dc_zero_half<<<dim3(ceil_div(hmax, 128), kmax, 2 * nm), 128, 0, ctx->stream>>>(w);
        MODAL_TRY(launched(ctx, "dc_zero_half"));
        k_dc_lam<<<dim3(ceil_div(kmax, 256), nm), 256, 0, ctx->stream>>>(w);
        MODAL_TRY(launched(ctx, "dc_lam"));
        std::swap(Z, Zn);
    }
    if (Z != p.Z) {
        MODAL_CUDA(cudaMemcpyAsync(p.Z, Z, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    return MODAL_OK;
}

// Compact-WY factors of the blocks of NBB reflectors: the diagonal blocks of
// the Gram matrix VA^T VA (tensor-core products), then dlarft per block.
static modal_status wy_blocks(modal_ctx *ctx, int n, SyevPtrs &p)
{
    const int nv = n - 1, nbig = ceil_div(nv, NBB), nbw = ceil_div(nv, NBW);
    OzOpts o;
    o.slices = OZ_SLICES;
    o.diag_tiles = NBW / 128;
    o.check = false;
    MODAL_TRY(oz_gemm_ex(ctx, nv, nv, n, 1.0, p.VA, p.ldva, true, p.VA, p.ldva, false, 0.0, p.GB, p.ldva, o));
    k_larft<<<nbig, 256, 0, ctx->stream>>>(nv, p.GB, p.ldva, p.tau, p.TB);
    MODAL_TRY(launched(ctx, "larft"));
    k_tw_assemble<<<dim3(NBW * NBW / 256, nbw), 256, 0, ctx->stream>>>(nv, p.TB, p.TW);
    MODAL_TRY(launched(ctx, "tw_assemble"));
    // T12 = -T1 (V1^T V2) T2 for the blocks with two halves (FP64-accurate tensor-core products,
    // 2 x 256^3 each: the FP64 tiled kernel would run them on 16 CTAs at GB300's FP64 rate)
    OzOpts oj;
    oj.slices = OZ_SLICES;
    oj.check = false;
    for (int k = 0; k < nbw; k++) {
        const int j0 = k * NBW, w = std::min(NBW, nv - j0), w2 = w - NBB;
        if (w2 <= 0) continue;
        const double *G12 = p.GB + (size_t)j0 * p.ldva + j0 + NBB;
        const double *T1 = p.TB + (size_t)(2 * k) * NBB * NBB, *T2 = p.TB + (size_t)(2 * k + 1) * NBB * NBB;
        double *T12 = p.TW + (size_t)k * NBW * NBW + NBB;
        MODAL_TRY(oz_gemm_ex(ctx, NBB, w2, w2, 1.0, G12, p.ldva, false, T2, NBB, false, 0.0, p.TT, NBB, oj));
        MODAL_TRY(oz_gemm_ex(ctx, NBB, w2, NBB, -1.0, T1, NBB, false, p.TT, NBB, false, 0.0, T12, NBW, oj));
    }
    return MODAL_OK;
}

// X[m][n] (rows = vectors in the tridiagonal basis) := X Q^T, Q = H_0 ... H_{n-2}.
// Per block of NBW reflectors, last block first (block = I - V T V^T):
//   X[:, r:] -= ((X[:, r:] V) T^T) V^T,  r = first row where the block's V is nonzero.
static modal_status backtransform(modal_ctx *ctx, int n, int m, double *X, int ldx, SyevPtrs &p)
{
    if (m <= 0 || n < 2) return MODAL_OK;
    MODAL_TRY(wy_blocks(ctx, n, p));
    MODAL_TRY(ensure(ctx->scratch2, sizeof(double) * (size_t)m * NBW * 2));
    double *XV = ctx->scratch2.as<double>(), *XT = XV + (size_t)m * NBW;
    const int nv = n - 1, nbw = ceil_div(nv, NBW);
    OzOpts o;
    o.slices = OZ_SLICES;
    o.check = false;
    for (int bb = nbw - 1; bb >= 0; bb--) {
        const int j0 = bb * NBW, w = std::min(NBW, nv - j0);
        const int r = j0 + 1, K = n - r;
        const double *V = p.VA + (size_t)r * p.ldva + j0;
        const double *T = p.TW + (size_t)bb * NBW * NBW;
        MODAL_TRY(oz_gemm_ex(ctx, m, w, K, 1.0, X + r, ldx, false, V, p.ldva, false, 0.0, XV, NBW, o));
        MODAL_TRY(oz_gemm_ex(ctx, m, w, w, 1.0, XV, NBW, false, T, NBW, true, 0.0, XT, NBW, o));
        MODAL_TRY(oz_gemm_ex(ctx, m, K, w, -1.0, XT, NBW, false, V, p.ldva, true, 1.0, X + r, ldx, o));
    }
    return oz_check(ctx);
}

// Eigen-decomposition of the symmetric n x n matrix A (device, row-major,
// overwritten).  W[n] (device) receives every eigenvalue in ascending order.
// select(W_host, n, arg, &first) returns how many eigenvectors are wanted,
// starting at ascending index `first`; those are written as rows of V (device,
// ld n): row t holds the eigenvector of W[first + t].  *nvec = that count,
// *first_out = first.
modal_status syev_dev(modal_ctx *ctx, int n, double *A, double *W, double *V, SyevSelect select, void *arg,
                      int *nvec, int *first_out)
{
    *nvec = 0;
    if (first_out) *first_out = 0;
    if (n <= 0) return MODAL_OK;
    static thread_local SyevState st;
    SyevPtrs p{};
    const int npanel = n > 1 ? ceil_div(n - 1, TRD_NB) : 0;
    MODAL_TRY(dc_setup(ctx, n, st, p, npanel));
    if (n > 1) {
        {
            StageTimer tt(ctx, MODAL_T_EIG_TRD);
            MODAL_TRY(trd_run(ctx, n, A, p, npanel));
        }
        StageTimer td(ctx, MODAL_T_EIG_DC);
        MODAL_TRY(dc_run(ctx, n, st, p));
    } else {
        MODAL_CUDA(cudaMemcpyAsync(p.lam, A, sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        MODAL_CUDA(cudaMemsetAsync(p.err, 0, 2 * sizeof(int), ctx->stream));
        k_dc_eye<<<1, 32, 0, ctx->stream>>>(1, p.Z);
        MODAL_TRY(launched(ctx, "dc_eye"));
    }
    MODAL_TRY(oz_check(ctx));
    MODAL_CUDA(cudaMemcpyAsync(W, p.lam, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    std::vector<double> hw(n);
    int herr[2] = {0, 0};
    MODAL_CUDA(cudaMemcpyAsync(hw.data(), p.lam, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    MODAL_CUDA(cudaMemcpyAsync(herr, p.err, sizeof(herr), cudaMemcpyDeviceToHost, ctx->stream));
    MODAL_CUDA(cudaStreamSynchronize(ctx->stream));
    if (herr[0]) { set_error("eigensolver: a bounded grid-barrier wait expired"); return MODAL_ERR_TIMEOUT; }
    for (int i = 0; i < n; i++)
        if (!std::isfinite(hw[i])) { set_error("eigensolver: non-finite eigenvalue"); return MODAL_ERR_NOCONV; }
    int first = 0;
    int c = select ? select(hw.data(), n, arg, &first) : n;
    if (first < 0 || first > n) first = 0;
    c = std::max(0, std::min(n - first, c));
    *nvec = c;
    if (first_out) *first_out = first;
    if (c == 0) return MODAL_OK;
    MODAL_CUDA(cudaMemcpyAsync(V, p.Z + (size_t)first * n, sizeof(double) * (size_t)c * n, cudaMemcpyDeviceToDevice,
                               ctx->stream));
    StageTimer tb(ctx, MODAL_T_EIG_BACK);
    return backtransform(ctx, n, c, V, n, p);
}

}  // namespace modal

using namespace modal;

extern "C" modal_status modal_eigh(modal_ctx *c, int n, const double *a, double *w, double *v)
{
    if (!c || n < 1 || !a || !w) { set_error("modal_eigh: bad arguments (n=%d)", n); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    const size_t NN = (size_t)n * n;
    MODAL_TRY(ensure(c->scratch, sizeof(double) * (2 * NN + (size_t)n)));
    double *A = c->scratch.as<double>(), *V = A + NN, *W = V + NN;
    MODAL_CUDA(cudaMemcpyAsync(A, a, sizeof(double) * NN, cudaMemcpyHostToDevice, c->stream));
    int nv = 0, first = 0;
    struct Want { bool vectors; } want{v != nullptr};
    auto sel = [](const double *, int nn, void *arg, int *f) -> int {
        *f = 0;
        return static_cast<Want *>(arg)->vectors ? nn : 0;
    };
    MODAL_TRY(syev_dev(c, n, A, W, V, sel, &want, &nv, &first));
    MODAL_CUDA(cudaMemcpyAsync(w, W, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    if (v) MODAL_CUDA(cudaMemcpyAsync(v, V, sizeof(double) * NN, cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}
