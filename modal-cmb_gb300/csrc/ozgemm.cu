// ozgemm.cu -- FP64-accurate matrix products on the FP16 tensor cores.
//
// GB300 runs FP64 at about 1.25 TFLOP/s but FP16 tensor products at about
// 2 PFLOP/s.  Here an FP64 product C = beta C + alpha op(A) op(B) runs on the
// tensor cores by exact integer slicing (the Ozaki scheme: Ozaki, Ogita, Oishi
// and Rump, "Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applications", Numer. Algorithms
// 59 (2012)):
//
//   every row r of op(A) (and every column of op(B)) is scaled by a power of
//   two 2^e_r so that its entries lie in (-1, 1), then written as s balanced
//   7-bit digits:  x = 2^e sum_p d_p 2^{-6-7p},  d_p integer in [-64, 64],
//   exact in FP16 (x 2^{6-e+7(s-1)} rounded once to a 55-bit integer, its
//   digits split off with integer arithmetic).  A digit product is at most 2^12 in size, so the FP32
//   tensor-memory accumulator sums up to 4096 of them without rounding; the
//   K dimension is cut into blocks of OZ_KB = 512, and the products of one
//   block with equal p + q = g (at most s of them) share one accumulator,
//   still exact (s * 512 * 2^12 <= 2^24 for s <= 8).
//
//   C = 2^{eA_m + eB_n - 12} sum_{g < s} 2^{-7g} sum_{p+q=g} sum_k dA_p dB_q,
//   products with p + q >= s dropped (below 2^{-7s} of the leading term).
//
// The exact block sums are added in double-FP32 ("double-float": an FP32
// head and tail, Knuth's TwoSum) kept in tensor memory; the tile is converted
// to FP64 once at the end.  Accuracy: about 2^-48 relative to max|row| max|col|
// per K block, the class of an FP64 GEMM over K = 5000 terms.
//
// Kernel k_oz_gemm: persistent, one CTA per SM over the output tiles
// (128 x 128); warp 0 TMA producer (8-stage ring of 16 KB: an A-slice and a
// B-slice chunk of 32 K, 64-byte swizzle), warp 1 MMA issuer (tcgen05.mma
// kind::f16, M = N = 128, K = 16) and TMEM owner, warps 2-5 epilogue.  TMEM:
// two FP32 accumulators (columns 0-255, the epilogue drains one while the next
// group fills the other) and the double-float sums (columns 256-511).  Every
// mbarrier wait is bounded; on expiry the CTA flags an error, stops, drains its
// copies, frees TMEM and returns (MODAL_ERR_TIMEOUT).
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>
#include <algorithm>
#include <mutex>
#include <vector>
#include "common.cuh"
#include "dfbits.cuh"
#include "tc_ptx.cuh"

namespace modal {

namespace {

using namespace tc;

constexpr int OZ_BM = 128, OZ_BN = 128, OZ_BK = 32, OZ_KB = 512, OZ_STAGES = 8;
constexpr int OZ_MAXS = 8;
constexpr uint32_t OZ_A_BYTES = OZ_BM * OZ_BK * 2;  // 8 KB
constexpr uint32_t OZ_B_BYTES = OZ_BN * OZ_BK * 2;  // 8 KB
constexpr uint32_t OZ_STAGE_BYTES = OZ_A_BYTES + OZ_B_BYTES;
constexpr uint32_t OZ_STAGING = 4 * 32 * 33 * 8;  // epilogue: 32 x 32 FP64 per warp (+1 column pad)
constexpr uint32_t OZ_SMEM = OZ_STAGES * OZ_STAGE_BYTES + 1024 + 256 + OZ_STAGING;
constexpr uint32_t OZ_TMEM_COLS = 512;
constexpr uint32_t OZ_SUM_COL = 256;  // first column of the double-float sums
constexpr long long OZ_WAIT = 1ll << 31;  // ~1 s of clock64 per wait
constexpr uint32_t OZ_IDESC = idesc_f16(OZ_BM, OZ_BN);

// ------------------------------------------------------------------ slicing
// Rows of op(X), R x K: element (r, k) = trans ? X[k*ld + r] : X[r*ld + k].
// Tiles of 32 rows x 32 columns through shared memory (coalesced either way).
__device__ __forceinline__ void oz_load_tile(double (*tile)[33], const double *__restrict__ X, long ld, int trans,
                                             int R, int K, int r0, int k0)
{
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (!trans) {
        for (int rr = ty; rr < 32; rr += 8) {
            const int r = r0 + rr, k = k0 + tx;
            tile[rr][tx] = (r < R && k < K) ? X[(size_t)r * ld + k] : 0.0;
        }
    } else {
        for (int kk = ty; kk < 32; kk += 8) {
            const int r = r0 + tx, k = k0 + kk;
            tile[tx][kk] = (r < R && k < K) ? X[(size_t)k * ld + r] : 0.0;
        }
    }
}

// Row exponents, over K chunks in parallel: ex[r] = max over the row of
// ilogb(|x|) + 1 (atomicMax over the chunks; ex starts at a value below every
// exponent, and an all-zero row keeps it).  grid (Rpad / 32, K chunks).
__global__ void __launch_bounds__(256) k_oz_rowexp(int R, int K, int kchunk, const double *__restrict__ X, long ld,
                                                   int trans, int *__restrict__ ex)
{
    __shared__ double tile[32][33];
    const int r0 = blockIdx.x * 32, kb = blockIdx.y * kchunk, ke = min(K, kb + kchunk);
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    // the maxima on the bit patterns (integer instructions, not the FP64 pipe)
    unsigned long long mx[4] = {0ull, 0ull, 0ull, 0ull};
    for (int k0 = kb; k0 < ke; k0 += 32) {
        oz_load_tile(tile, X, ld, trans, R, ke, r0, k0);
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 4; j++) mx[j] = dfb::absmax_bits(mx[j], tile[ty + 8 * j][tx]);
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        unsigned long long b = mx[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
        const double v = __longlong_as_double((long long)b);
        const int r = r0 + ty + 8 * j;
        if (tx == 0 && r < R && v > 0.0 && isfinite(v)) atomicMax(ex + r, ilogb(v) + 1);
    }
}

// Slices of the rows of op(X) from their exponents: out: [s][Rpad][Kpad] FP16
// digits.  Rows >= R and columns >= K are zero; a row whose exponent is still
// the starting value (all zero) gets exponent 0.  grid (Rpad / 32, K chunks).
__global__ void __launch_bounds__(256) k_oz_slice(int R, int K, int Rpad, int Kpad, int kchunk,
                                                  const double *__restrict__ X, long ld, int trans, int s,
                                                  __half *__restrict__ out, int *__restrict__ ex)
{
    __shared__ double tile[32][33];
    __shared__ int sexp[32];
    const int r0 = blockIdx.x * 32, kb = blockIdx.y * kchunk, ke = min(Kpad, kb + kchunk);
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (threadIdx.x < 32) {
        const int r = r0 + threadIdx.x;
        const int e = ex[r];
        sexp[threadIdx.x] = (e < -100000) ? 0 : e;
    }
    __syncthreads();
    if (blockIdx.y == 0 && threadIdx.x < 32) ex[r0 + threadIdx.x] = sexp[threadIdx.x];
    const size_t plane = (size_t)Rpad * Kpad;
    for (int k0 = kb; k0 < ke; k0 += 32) {
        if (k0 < K) oz_load_tile(tile, X, ld, trans, R, K, r0, k0);
        __syncthreads();
        for (int rr = ty; rr < 32; rr += 8) {
            const int r = r0 + rr, k = k0 + tx;
            // F = x 2^{6 - e + 7(s-1)} rounded to an integer, |F| < 2^55 (from the bits
            // of x; FP64 instructions only outside that route's range); its balanced
            // base-128 digits, least significant first, are exact integer operations
            const double x = (k0 < K) ? tile[rr][tx] : 0.0;
            const int sh = 6 - sexp[rr] + 7 * (s - 1);
            long long F;
            if (!dfb::scaled_rint(x, sh, &F)) {
                const double y = ldexp(x, sh);
                F = isfinite(y) ? __double2ll_rn(y) : 0ll;
            }
            __half *o = out + (size_t)r * Kpad + k;
            for (int p = s - 1; p > 0; p--) {
                const long long d = ((F + 64) & 127) - 64;
                o[p * plane] = __int2half_rn((int)d);
                F = (F - d) >> 7;
            }
            o[0] = __int2half_rn((int)F);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ GEMM
struct OzArgs {
    int M, N, Kpad, Mpad, Npad, s, nkb, ntiles, lower, kper;
    const int4 *tiles;  // work items: (tile row, tile column, K split index, -)
    double *part;       // K split > 1: partial products [split][M][N]
    const int *ea, *eb;
    double alpha, beta;
    double *C;
    long ldc;
    int *err;
};

// double-float a + b (Knuth's TwoSum, then renormalised)
__device__ __forceinline__ void df_add(float &hi, float &lo, float b)
{
    const float s = hi + b;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (b - bb);
    const float t = lo + e;
    hi = s + t;
    lo = t - (hi - s);
}

__global__ void __launch_bounds__(192, 1) k_oz_gemm(const __grid_constant__ CUtensorMap tmA,
                                                   const __grid_constant__ CUtensorMap tmB, OzArgs a)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + OZ_STAGES * OZ_STAGE_BYTES);
    uint64_t *full = bars, *empty = bars + OZ_STAGES, *afull = bars + 2 * OZ_STAGES, *aempty = afull + 2;
    volatile uint32_t *tmem_slot = reinterpret_cast<volatile uint32_t *>(bars + 2 * OZ_STAGES + 4);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(bars + 2 * OZ_STAGES + 5);
    double *stage = reinterpret_cast<double *>(smem + OZ_STAGES * OZ_STAGE_BYTES + 256);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int s = a.s;
    if (threadIdx.x == 0) {
        for (int i = 0; i < OZ_STAGES; i++) {
            mbar_init(smem_u32(&full[i]), 1);
            mbar_init(smem_u32(&empty[i]), 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(smem_u32(&afull[b]), 1);
            mbar_init(smem_u32(&aempty[b]), 4);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        tmem_alloc(smem_u32((const void *)tmem_slot), OZ_TMEM_COLS);
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            long g = 0;
            bool stop = false;
            for (int t = blockIdx.x; t < a.ntiles && !stop; t += gridDim.x) {
                const int4 tile = a.tiles[t];
                const int m0 = tile.x * OZ_BM, n0 = tile.y * OZ_BN;
                const int kb0 = tile.z * a.kper, kb1 = min(a.nkb, kb0 + a.kper);
                for (int kb = kb0; kb < kb1 && !stop; kb++) {
                    const int kbeg = kb * OZ_KB, nkc = min(OZ_KB, a.Kpad - kbeg) / OZ_BK;
                    for (int gg = 0; gg < s && !stop; gg++)
                        for (int p = 0; p <= gg && !stop; p++)
                            for (int kc = 0; kc < nkc; kc++, g++) {
                                const int st = (int)(g % OZ_STAGES);
                                const long it = g / OZ_STAGES;
                                if (it > 0 && !mbar_wait(smem_u32(&empty[st]), (uint32_t)((it - 1) & 1), abort_flag, OZ_WAIT)) {
                                    if (!*abort_flag) { *abort_flag = 1; atomicCAS(a.err, 0, 1); }
                                    stop = true;
                                    break;
                                }
                                uint8_t *sp = smem + (size_t)st * OZ_STAGE_BYTES;
                                const uint32_t fb = smem_u32(&full[st]);
                                mbar_expect_tx(fb, OZ_STAGE_BYTES);
                                const int k = kbeg + kc * OZ_BK;
                                tma_load_2d(smem_u32(sp), &tmA, k, p * a.Mpad + m0, fb);
                                tma_load_2d(smem_u32(sp + OZ_A_BYTES), &tmB, k, (gg - p) * a.Npad + n0, fb);
                            }
                }
            }
            // drain: the copies of the last stages must land before the CTA exits
            for (long h = (g > OZ_STAGES ? g - OZ_STAGES : 0); h < g; h++) {
                const int st = (int)(h % OZ_STAGES);
                const long long t0 = clock64();
                while (!mbar_try(smem_u32(&full[st]), (uint32_t)((h / OZ_STAGES) & 1)) && clock64() - t0 < OZ_WAIT) {
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            long g = 0, u = 0;
            bool stop = false;
            for (int t = blockIdx.x; t < a.ntiles && !stop; t += gridDim.x) {
                const int kb0 = a.tiles[t].z * a.kper, kb1 = min(a.nkb, kb0 + a.kper);
                for (int kb = kb0; kb < kb1 && !stop; kb++) {
                    const int kbeg = kb * OZ_KB, nkc = min(OZ_KB, a.Kpad - kbeg) / OZ_BK;
                    for (int gg = 0; gg < s && !stop; gg++, u++) {
                        const int buf = (int)(u & 1);
                        const long use = u >> 1;
                        if (use > 0 && !mbar_wait(smem_u32(&aempty[buf]), (uint32_t)((use - 1) & 1), abort_flag, OZ_WAIT)) {
                            if (!*abort_flag) { *abort_flag = 1; atomicCAS(a.err, 0, 4); }
                            stop = true;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t d = tmem + (uint32_t)(buf * OZ_BN);
                        uint32_t accf = 0;
                        for (int p = 0; p <= gg && !stop; p++)
                            for (int kc = 0; kc < nkc; kc++, g++) {
                                const int st = (int)(g % OZ_STAGES);
                                const long it = g / OZ_STAGES;
                                if (!mbar_wait(smem_u32(&full[st]), (uint32_t)(it & 1), abort_flag, OZ_WAIT)) {
                                    if (!*abort_flag) { *abort_flag = 1; atomicCAS(a.err, 0, 2); }
                                    stop = true;
                                    break;
                                }
                                tc_fence_after();
                                const uint32_t sa = smem_u32(smem + (size_t)st * OZ_STAGE_BYTES), sb = sa + OZ_A_BYTES;
#pragma unroll
                                for (int kk = 0; kk < OZ_BK / 16; kk++) {
                                    umma_f16(d, desc_sw64(sa + kk * 32), desc_sw64(sb + kk * 32), OZ_IDESC, accf);
                                    accf = 1;
                                }
                                umma_commit(smem_u32(&empty[st]));
                            }
                        if (!stop) umma_commit(smem_u32(&afull[buf]));
                    }
                }
            }
        }
    } else {
        // epilogue: warps 2..5 own TMEM lanes 32*(warp % 4) .. +31 (rows of the tile)
        const int lb = (warp & 3) * 32;
        const uint32_t trow = (uint32_t)lb << 16;
        long u = 0;
        bool stop = false;
        for (int t = blockIdx.x; t < a.ntiles && !stop; t += gridDim.x) {
            const int kb0 = a.tiles[t].z * a.kper, kb1 = min(a.nkb, kb0 + a.kper);
            for (int kb = kb0; kb < kb1 && !stop; kb++) {
                for (int gg = 0; gg < s; gg++, u++) {
                    const int buf = (int)(u & 1);
                    const long use = u >> 1;
                    if (!mbar_wait(smem_u32(&afull[buf]), (uint32_t)(use & 1), abort_flag, OZ_WAIT)) {
                        if (!*abort_flag) { *abort_flag = 1; atomicCAS(a.err, 0, 3); }
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    const float scale = ldexpf(1.0f, -7 * gg);
                    const bool first = (kb == kb0 && gg == 0);
                    for (int c0 = 0; c0 < OZ_BN; c0 += 32) {
                        uint32_t v[32], hl[32];
                        tmem_ld32(tmem + trow + (uint32_t)(buf * OZ_BN + c0), v);
                        if (!first) {
                            tmem_ld32(tmem + trow + OZ_SUM_COL + (uint32_t)(2 * c0), hl);       // heads, tails of 16 columns
                            uint32_t hl2[32];
                            tmem_ld32(tmem + trow + OZ_SUM_COL + (uint32_t)(2 * c0 + 32), hl2);  // the next 16
                            tmem_wait_ld();
#pragma unroll
                            for (int j = 0; j < 16; j++) {
                                float h = __uint_as_float(hl[2 * j]), l = __uint_as_float(hl[2 * j + 1]);
                                df_add(h, l, __uint_as_float(v[j]) * scale);
                                hl[2 * j] = __float_as_uint(h);
                                hl[2 * j + 1] = __float_as_uint(l);
                                float h2 = __uint_as_float(hl2[2 * j]), l2 = __uint_as_float(hl2[2 * j + 1]);
                                df_add(h2, l2, __uint_as_float(v[16 + j]) * scale);
                                hl2[2 * j] = __float_as_uint(h2);
                                hl2[2 * j + 1] = __float_as_uint(l2);
                            }
                            tmem_st32(tmem + trow + OZ_SUM_COL + (uint32_t)(2 * c0), hl);
                            tmem_st32(tmem + trow + OZ_SUM_COL + (uint32_t)(2 * c0 + 32), hl2);
                        } else {
                            tmem_wait_ld();
                            uint32_t h1[32], h2[32];
#pragma unroll
                            for (int j = 0; j < 16; j++) {
                                h1[2 * j] = __float_as_uint(__uint_as_float(v[j]) * scale);
                                h1[2 * j + 1] = 0u;
                                h2[2 * j] = __float_as_uint(__uint_as_float(v[16 + j]) * scale);
                                h2[2 * j + 1] = 0u;
                            }
                            tmem_st32(tmem + trow + OZ_SUM_COL + (uint32_t)(2 * c0), h1);
                            tmem_st32(tmem + trow + OZ_SUM_COL + (uint32_t)(2 * c0 + 32), h2);
                        }
                    }
                    tmem_wait_st();
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(smem_u32(&aempty[buf]));
                }
            }
            if (stop) break;
            // the tile's result: C = beta C + alpha 2^{eA + eB - 12} (head + tail), or the
            // unscaled partial of this K split.  Each warp stages its 32 rows x 32
            // columns in shared memory and writes them row by row, coalesced.
            const int4 tile = a.tiles[t];
            const int mrow = tile.x * OZ_BM + lb;
            const int n0 = tile.y * OZ_BN;
            const int m = mrow + lane;
            const double rs = ldexp(1.0, ((m < a.M) ? a.ea[m] : 0) - 12);
            const bool split = a.part != nullptr;
            double *st = stage + (size_t)(warp - 2) * 32 * 33;
            for (int c0 = 0; c0 < OZ_BN; c0 += 32) {
                uint32_t h1[32], h2[32];
                tmem_ld32(tmem + trow + OZ_SUM_COL + (uint32_t)(2 * c0), h1);
                tmem_ld32(tmem + trow + OZ_SUM_COL + (uint32_t)(2 * c0 + 32), h2);
                tmem_wait_ld();
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    st[lane * 33 + j] = ((double)__uint_as_float(h1[2 * j]) + (double)__uint_as_float(h1[2 * j + 1])) * rs;
                    st[lane * 33 + 16 + j] = ((double)__uint_as_float(h2[2 * j]) + (double)__uint_as_float(h2[2 * j + 1])) * rs;
                }
                __syncwarp();
                const int n = n0 + c0 + lane;
                const double cs = (n < a.N) ? ldexp(1.0, a.eb[n]) : 0.0;
                // the C values of 16 rows are loaded together before any store (one round
                // trip per 16 rows instead of one per row)
#pragma unroll 1
                for (int r0 = 0; r0 < 32; r0 += 16) {
                    double cv[16];
#pragma unroll
                    for (int rr = 0; rr < 16; rr++) {
                        const int mm = mrow + r0 + rr;
                        const bool ok = !split && a.beta != 0.0 && mm < a.M && n < a.N && !(a.lower && n > mm);
                        cv[rr] = ok ? a.C[(size_t)mm * a.ldc + n] : 0.0;
                    }
#pragma unroll
                    for (int rr = 0; rr < 16; rr++) {
                        const int mm = mrow + r0 + rr;
                        if (mm >= a.M || n >= a.N || (a.lower && n > mm)) continue;
                        const double v = st[(r0 + rr) * 33 + lane] * cs;
                        if (split) a.part[((size_t)tile.z * a.M + mm) * a.N + n] = v;
                        else a.C[(size_t)mm * a.ldc + n] = (a.beta == 0.0) ? a.alpha * v : fma(a.beta, cv[rr], a.alpha * v);
                    }
                }
                __syncwarp();
            }
            tc_fence_before();
            __syncwarp();
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, OZ_TMEM_COLS);
    }
}

// C = beta C + alpha sum_z part_z (K splits added in a fixed order).
__global__ void k_oz_reduce(int M, int N, int ks, const double *__restrict__ part, double alpha, double beta, double *C,
                            long ldc, int lower)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)M * N) return;
    const int m = (int)(e / N), n = (int)(e - (size_t)m * N);
    if (lower && n > m) return;
    double v = 0.0;
    for (int z = 0; z < ks; z++) v += part[(size_t)z * M * N + e];
    double *c = C + (size_t)m * ldc + n;
    *c = (beta == 0.0) ? alpha * v : fma(beta, *c, alpha * v);
}

// ------------------------------------------------------------------ host side
PFN_cuTensorMapEncodeTiled_v12000 g_oz_encode = nullptr;
std::mutex g_oz_mu;

modal_status oz_encoder()
{
    std::lock_guard<std::mutex> lock(g_oz_mu);
    if (g_oz_encode) return MODAL_OK;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
        set_error("cuTensorMapEncodeTiled unavailable: %s", cudaGetErrorString(e));
        return MODAL_ERR_CUDA;
    }
    g_oz_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return MODAL_OK;
}

// 2D FP16 map over [rows][Kpad], box [box_rows][32], 64-byte swizzle.
modal_status oz_map(CUtensorMap *m, const void *base, long rows, int Kpad, int box_rows)
{
    cuuint64_t dims[2] = {(cuuint64_t)Kpad, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)Kpad * 2};
    cuuint32_t box[2] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_oz_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return MODAL_ERR_CUDA; }
    return MODAL_OK;
}

}  // namespace

// C[M][N] (ld ldc) = beta C + alpha op(A) op(B), op(A) M x K, op(B) K x N, in
// FP64 accuracy class on the tensor cores with o.slices slices (2 <= s <= 8).
//   op(A)(m, k) = transA ? A[k*lda + m] : A[m*lda + k]
//   op(B)(k, n) = transB ? B[n*ldb + k] : B[k*ldb + n]
// o.lower: only entries with n <= m are written (square C); o.diag_tiles > 0:
// only the 128-row tiles (tm, tn) with tm / diag_tiles == tn / diag_tiles
// (the diagonal blocks of that many tiles); o.ksplit: K split over that many
// work items per tile (0: chosen to fill the GPU), partials added in order.
modal_status oz_slice(modal_ctx *ctx, int R, int K, const double *X, long ld, bool trans, int s, int Rpad, int Kpad,
                      __half *out, int *ex)
{
    if (Rpad % OZ_BM || Kpad % 64 || R > Rpad || K > Kpad || s < 2 || s > OZ_MAXS) {
        set_error("oz_slice: bad layout (R=%d Rpad=%d K=%d Kpad=%d s=%d)", R, Rpad, K, Kpad, s);
        return MODAL_ERR_ARG;
    }
    // K split into chunks (multiples of 32) so that the grid has about two CTAs per SM
    int nsm = 0;
    MODAL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
    const int rb = Rpad / 32, want = std::max(1, ceil_div(2 * nsm, rb));
    const int kchunk = std::max(32, ceil_div(ceil_div(Kpad, want), 32) * 32);
    const int nkc = ceil_div(Kpad, kchunk);
    MODAL_CUDA(cudaMemsetAsync(ex, 0x80, sizeof(int) * (size_t)Rpad, ctx->stream));  // below every exponent
    k_oz_rowexp<<<dim3(rb, ceil_div(std::max(K, 1), kchunk)), 256, 0, ctx->stream>>>(R, K, kchunk, X, ld, trans ? 1 : 0,
                                                                                     ex);
    MODAL_TRY(launched(ctx, "oz_rowexp"));
    k_oz_slice<<<dim3(rb, nkc), 256, 0, ctx->stream>>>(R, K, Rpad, Kpad, kchunk, X, ld, trans ? 1 : 0, s, out, ex);
    return launched(ctx, "oz_slice");
}

modal_status oz_run(modal_ctx *ctx, const OzOperand &A, const OzOperand &B, int Kpad, int s,
                    const std::vector<int2> *tile_list, double alpha, double beta, double *C, long ldc, const OzOpts &o)
{
    const int M = A.rows, N = B.rows, Mpad = A.rows_pad, Npad = B.rows_pad;
    if (M <= 0 || N <= 0) return MODAL_OK;
    if (s < 2 || s > OZ_MAXS || Mpad % OZ_BM || Npad % OZ_BM || Kpad % 64 || Kpad <= 0) {
        set_error("oz_run: bad layout (Mpad=%d Npad=%d Kpad=%d s=%d)", Mpad, Npad, Kpad, s);
        return MODAL_ERR_ARG;
    }
    MODAL_TRY(oz_encoder());
    const int ntm = Mpad / OZ_BM, ntn = Npad / OZ_BN;
    const int nkb = ceil_div(Kpad, OZ_KB);
    int nsm = 0;
    MODAL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
    std::vector<int2> own;
    if (!tile_list) {
        // tile order: column of tiles outer so that consecutive CTAs share B slices in L2
        for (int tn = 0; tn < ntn; tn++)
            for (int tm = 0; tm < ntm; tm++) {
                if (o.lower && tn > tm) continue;
                if (o.diag_tiles > 0 && tm / o.diag_tiles != tn / o.diag_tiles) continue;
                own.push_back(make_int2(tm, tn));
            }
    }
    const std::vector<int2> &base = tile_list ? *tile_list : own;
    if (base.empty()) return MODAL_OK;
    int ks = o.ksplit;
    if (ks <= 0) ks = (int)std::min<long>(nkb, std::max<long>(1, (long)nsm / std::max<size_t>(1, base.size())));
    ks = std::max(1, std::min(ks, nkb));
    const int kper = ceil_div(nkb, ks);
    ks = ceil_div(nkb, kper);
    std::vector<int4> tiles;
    tiles.reserve(base.size() * ks);
    for (int z = 0; z < ks; z++)
        for (const int2 &t : base) tiles.push_back(make_int4(t.x, t.y, z, 0));
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t off = 0;
    const size_t o_t = off; off += al(tiles.size() * sizeof(int4));
    const size_t o_p = off; off += (ks > 1) ? al((size_t)ks * M * N * 8) : 0;
    MODAL_TRY(ensure(ctx->ozrun, off));
    uint8_t *b = ctx->ozrun.as<uint8_t>();
    MODAL_TRY(ensure(ctx->ozerr, 256));
    int *err = ctx->ozerr.as<int>();
    MODAL_CUDA(cudaMemcpyAsync(b + o_t, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, ctx->stream));
    if (o.check) MODAL_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
    CUtensorMap ma, mb;
    MODAL_TRY(oz_map(&ma, A.slices, (long)s * Mpad, Kpad, OZ_BM));
    MODAL_TRY(oz_map(&mb, B.slices, (long)s * Npad, Kpad, OZ_BN));
    OzArgs g;
    g.M = M; g.N = N; g.Kpad = Kpad; g.Mpad = Mpad; g.Npad = Npad; g.s = s;
    g.nkb = nkb;
    g.kper = kper;
    g.ntiles = (int)tiles.size();
    g.lower = o.lower;
    g.tiles = reinterpret_cast<const int4 *>(b + o_t);
    g.part = ks > 1 ? reinterpret_cast<double *>(b + o_p) : nullptr;
    g.ea = A.ex; g.eb = B.ex; g.alpha = alpha; g.beta = beta; g.C = C; g.ldc = ldc; g.err = err;
    MODAL_CUDA(cudaFuncSetAttribute(k_oz_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OZ_SMEM));
    const int grid = std::max(1, std::min(g.ntiles, nsm));
    {
        StageTimer t(ctx, MODAL_T_TC);
        k_oz_gemm<<<grid, 192, OZ_SMEM, ctx->stream>>>(ma, mb, g);
        MODAL_TRY(launched(ctx, "oz_gemm"));
    }
    if (ks > 1) {
        k_oz_reduce<<<ceil_div((long)M * N, 256), 256, 0, ctx->stream>>>(M, N, ks, g.part, alpha, beta, C, ldc, o.lower);
        MODAL_TRY(launched(ctx, "oz_reduce"));
    }
    // unchecked calls leave the (sticky) error word for oz_check
    return o.check ? oz_check(ctx) : MODAL_OK;
}

modal_status oz_gemm_ex(modal_ctx *ctx, int M, int N, int K, double alpha, const double *A, long lda, bool transA,
                        const double *B, long ldb, bool transB, double beta, double *C, long ldc, const OzOpts &o)
{
    if (M <= 0 || N <= 0) return MODAL_OK;
    const int s = o.slices;
    if (s < 2 || s > OZ_MAXS) { set_error("oz_gemm: slices %d outside [2, %d]", s, OZ_MAXS); return MODAL_ERR_ARG; }
    if (K <= 0) {
        if (beta == 1.0) return MODAL_OK;
        set_error("oz_gemm: K = %d with beta != 1", K);
        return MODAL_ERR_ARG;
    }
    const int Mpad = ceil_div(M, OZ_BM) * OZ_BM, Npad = ceil_div(N, OZ_BN) * OZ_BN;
    const int Kpad = ceil_div(K, 64) * 64;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t off = 0;
    const size_t o_a = off; off += al((size_t)s * Mpad * Kpad * 2);
    const size_t o_b = off; off += al((size_t)s * Npad * Kpad * 2);
    const size_t o_ea = off; off += al((size_t)Mpad * 4);
    const size_t o_eb = off; off += al((size_t)Npad * 4);
    MODAL_TRY(ensure(ctx->ozw, off));
    uint8_t *b = ctx->ozw.as<uint8_t>();
    OzOperand oa{reinterpret_cast<__half *>(b + o_a), reinterpret_cast<int *>(b + o_ea), M, Mpad};
    OzOperand ob{reinterpret_cast<__half *>(b + o_b), reinterpret_cast<int *>(b + o_eb), N, Npad};
    MODAL_TRY(oz_slice(ctx, M, K, A, lda, transA, s, Mpad, Kpad, oa.slices, oa.ex));
    // columns of op(B) = rows of op(B)^T: transB ? B[n*ldb + k] (rows of B) : B[k*ldb + n] (columns of B)
    MODAL_TRY(oz_slice(ctx, N, K, B, ldb, !transB, s, Npad, Kpad, ob.slices, ob.ex));
    return oz_run(ctx, oa, ob, Kpad, s, nullptr, alpha, beta, C, ldc, o);
}

modal_status oz_reset(modal_ctx *ctx)
{
    MODAL_TRY(ensure(ctx->ozerr, 256));
    MODAL_CUDA(cudaMemsetAsync(ctx->ozerr.ptr, 0, sizeof(int), ctx->stream));
    return MODAL_OK;
}

modal_status oz_check(modal_ctx *ctx)
{
    if (!ctx->ozerr.ptr) return MODAL_OK;
    int herr = 0;
    MODAL_CUDA(cudaMemcpyAsync(&herr, ctx->ozerr.ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MODAL_CUDA(cudaStreamSynchronize(ctx->stream));
    if (herr) { set_error("a bounded wait in a tensor-core kernel expired (role %d: 1-4 Ozaki GEMM, 21-22 slab projection)", herr); return MODAL_ERR_TIMEOUT; }
    return MODAL_OK;
}

modal_status oz_gemm(modal_ctx *ctx, int M, int N, int K, double alpha, const double *A, long lda, bool transA,
                     const double *B, long ldb, bool transB, double beta, double *C, long ldc, int lower, int s)
{
    OzOpts o;
    o.lower = lower;
    o.slices = s;
    return oz_gemm_ex(ctx, M, N, K, alpha, A, lda, transA, B, ldb, transB, beta, C, ldc, o);
}

}  // namespace modal

using namespace modal;

extern "C" modal_status modal_gemm_f64(modal_ctx *c, int M, int N, int K, double alpha, const double *A, int transA,
                                       const double *B, int transB, double beta, double *C, int slices)
{
    if (!c || M < 1 || N < 1 || K < 1 || !A || !B || !C || slices < 2 || slices > OZ_MAXS) {
        set_error("modal_gemm_f64: bad arguments (M=%d N=%d K=%d slices=%d)", M, N, K, slices);
        return MODAL_ERR_ARG;
    }
    MODAL_CUDA(cudaSetDevice(c->device));
    const size_t na = (size_t)M * K, nb = (size_t)K * N, nc = (size_t)M * N;
    MODAL_TRY(ensure(c->scratch, sizeof(double) * (na + nb + nc)));
    double *dA = c->scratch.as<double>(), *dB = dA + na, *dC = dB + nb;
    MODAL_CUDA(cudaMemcpyAsync(dA, A, sizeof(double) * na, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(dB, B, sizeof(double) * nb, cudaMemcpyHostToDevice, c->stream));
    MODAL_CUDA(cudaMemcpyAsync(dC, C, sizeof(double) * nc, cudaMemcpyHostToDevice, c->stream));
    MODAL_TRY(oz_gemm(c, M, N, K, alpha, dA, transA ? M : K, transA != 0, dB, transB ? K : N, transB != 0, beta, dC, N, 0,
                      slices));
    MODAL_CUDA(cudaMemcpyAsync(C, dC, sizeof(double) * nc, cudaMemcpyDeviceToHost, c->stream));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}
