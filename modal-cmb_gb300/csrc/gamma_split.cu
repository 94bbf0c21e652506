// gamma_split.cu -- split-precision tensor-core form of the mu-contraction.
//
// Gamma_mn = sum_k w_k/(48 pi) perm3(M(k)[m_a][n_b])   (orthogonalisation_late.c:239-336)
// is lifted to a GEMM over pairs.  With u = (a,b), a <= b, a pair of basis
// indices (U = P(P+1)/2 of them) and X_u(k) = M_ab(mu_k):
//     T[u][v][t] = sum_k X_u(k) * (w_k/(48 pi) X_v(k) X_t(k))      (fully symmetric)
//     Gamma_mn   = sum over the six orderings s of T[(m1,n_s1)][(m2,n_s2)][(m3,n_s3)]
// T is only needed for u <= v <= t: C(U+2,3) values (16.9M at P = 30).
//
// GEMM: rows u (A = X, 128-row tiles), columns (v,t) with v <= t (B = Y,
// Y_vt(k) = w_k X_v(k) X_t(k), 256-column tiles), K = n_mu.  Column tiles whose
// smallest u is above their largest v are skipped (44% of the full work at
// P = 30).  Precision: every row of X and of Y is scaled by a power of two and
// split into two FP16 pieces (x = x1 + x2, 22 significant bits); three tensor
// products x1 y1 + x1 y2 + x2 y1 accumulate in FP32 in tensor memory over the
// whole of K; T is stored in FP32 and Gamma summed in FP64.  Measured error vs
// the FP64 form: ~5e-8 relative (Frobenius) in emulation at l <= 1000.
//
// Kernel k_gamma_lift: persistent, one CTA per SM walking the (u tile, vt tile)
// list, 6 warps:
//   warp 0   TMA producer (4-stage ring of 48 KB: X1, X2 [128 x 32], Y1, Y2 [256 x 32],
//            64-byte swizzle), warp 1 MMA issuer (tcgen05.mma kind::f16, M=128 N=256 K=16)
//            and TMEM owner (2 accumulators x 256 columns), warps 2-5 epilogue
//            (tcgen05.ld -> T) draining one accumulator while the next tile fills the other.
// Every mbarrier wait is bounded (~1 s of clock64); on expiry the CTA records an
// error code, stops issuing, drains, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>
#include <mutex>
#include <vector>
#include "common.cuh"
#include "tc_ptx.cuh"

namespace modal {

constexpr int SP_BK = 32;    // K elements per stage: 64-byte FP16 rows, 64-byte swizzle
constexpr int SP_BM = 128;   // u rows per tile = TMEM lanes
constexpr int SP_BN = 256;   // vt columns per tile = TMEM columns of one accumulator
constexpr int SP_STAGES = 4;
constexpr int SP_KPAD = 64;  // K padding of the operand rows
constexpr uint32_t SP_A_BYTES = SP_BM * SP_BK * 2;                          // 8 KB
constexpr uint32_t SP_B_BYTES = SP_BN * SP_BK * 2;                          // 16 KB
constexpr uint32_t SP_STAGE_BYTES = 2 * SP_A_BYTES + 2 * SP_B_BYTES;        // 48 KB
constexpr uint32_t SP_SMEM = SP_STAGES * SP_STAGE_BYTES + 1024 + 256;       // + alignment + barriers
constexpr uint32_t SP_TMEM_COLS = 2 * SP_BN;                                 // two accumulators
constexpr long long SP_WAIT_CYCLES = 1ll << 31;                              // ~1 s

// Instruction descriptor, kind::f16: D = F32, A = B = F16, both K-major, M = 128, N = 256.
constexpr uint32_t SP_IDESC = tc::idesc_f16(SP_BM, SP_BN);

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag)
{
    return tc::mbar_wait(bar, parity, abort_flag, SP_WAIT_CYCLES);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int c0, int c1, uint32_t bar)
{
    tc::tma_load_2d(dst, map, c0, c1, bar);
}

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc)
{
    tc::umma_f16(tmem_d, a, b, SP_IDESC, acc);
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v)
{
    uint32_t r[32];
    tc::tmem_ld32(taddr, r);
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

using tc::smem_u32;
using tc::mbar_init;
using tc::mbar_expect_tx;
using tc::mbar_try;
using tc::mbar_arrive;
using tc::umma_commit;
inline __device__ uint64_t umma_desc(uint32_t saddr) { return tc::desc_sw64(saddr); }

// -------------------------------------------------------- operand preparation

// weights w_k/(48 pi) in FP32, zero beyond n_mu
__global__ void k_wgt48_f(int nmu, int Kpad, const double *__restrict__ w, float *__restrict__ wf)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < Kpad) wf[k] = (k < nmu) ? (float)(w[k] / (48e0 * 3.14159265358979323846)) : 0.f;
}

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Power of two bringing the row maximum m into [2^14, 2^15); 1 for an all-zero row.
__device__ __forceinline__ double pow2_scale(double m)
{
    if (!(m > 0.0) || !isfinite(m)) return 1.0;
    return ldexp(1.0, 14 - ilogb(m));
}

// One warp per pair row u: X1/X2 FP16 pieces of X_u(k) * s_u, FP32 copy of X_u(k).
__global__ void k_split_x(int U, int Upad, int P, int nmu, int Kpad, const int2 *__restrict__ pairs,
                          const double *__restrict__ mt, __half *__restrict__ X1, __half *__restrict__ X2,
                          float *__restrict__ xf, double *__restrict__ sx_inv)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int u = warp;
    if (u >= Upad) return;
    __half *x1 = X1 + (size_t)u * Kpad, *x2 = X2 + (size_t)u * Kpad;
    if (u >= U) {
        for (int k = lane; k < Kpad; k += 32) { x1[k] = __float2half(0.f); x2[k] = __float2half(0.f); }
        if (lane == 0) sx_inv[u] = 0.0;
        return;
    }
    const int2 ab = pairs[u];
    const size_t off = (size_t)ab.x * P + ab.y, PP = (size_t)P * P;
    double m = 0.0;
    for (int k = lane; k < nmu; k += 32) m = fmax(m, fabs(mt[(size_t)k * PP + off]));
    m = warp_max(m);
    const double s = pow2_scale(m);
    float *xr = xf + (size_t)u * Kpad;
    for (int k = lane; k < Kpad; k += 32) {
        double x = (k < nmu) ? mt[(size_t)k * PP + off] : 0.0;
        double xs = x * s;
        __half h = __double2half(xs);
        __half l = __double2half(xs - (double)__half2float(h));
        x1[k] = h;
        x2[k] = l;
        xr[k] = (float)x;
    }
    if (lane == 0) sx_inv[u] = 1.0 / s;
}

// One warp per (v,t) row: Y_vt(k) = w_k X_v(k) X_t(k) in FP32, scaled and split.
__global__ void k_split_y(int UV, int UVpad, int Kpad, const int2 *__restrict__ vt_pairs,
                          const float *__restrict__ xf, const float *__restrict__ wf, __half *__restrict__ Y1,
                          __half *__restrict__ Y2, double *__restrict__ sy_inv)
{
    const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= UVpad) return;
    const long r = warp;
    __half2 *y1 = reinterpret_cast<__half2 *>(Y1 + (size_t)r * Kpad);
    __half2 *y2 = reinterpret_cast<__half2 *>(Y2 + (size_t)r * Kpad);
    const int K2 = Kpad / 2;
    if (r >= UV) {
        for (int k = lane; k < K2; k += 32) { y1[k] = __float2half2_rn(0.f); y2[k] = __float2half2_rn(0.f); }
        if (lane == 0) sy_inv[r] = 0.0;
        return;
    }
    const int2 vt = vt_pairs[r];
    const float2 *xv = reinterpret_cast<const float2 *>(xf + (size_t)vt.x * Kpad);
    const float2 *xt = reinterpret_cast<const float2 *>(xf + (size_t)vt.y * Kpad);
    const float2 *w2 = reinterpret_cast<const float2 *>(wf);
    float m = 0.f;
    for (int k = lane; k < K2; k += 32) {
        float2 a = xv[k], b = xt[k], w = w2[k];
        m = fmaxf(m, fmaxf(fabsf(w.x * a.x * b.x), fabsf(w.y * a.y * b.y)));
    }
    double md = warp_max((double)m);
    const double s = pow2_scale(md);
    const float sf = (float)s;
    for (int k = lane; k < K2; k += 32) {
        float2 a = xv[k], b = xt[k], w = w2[k];
        float ya = w.x * a.x * b.x * sf, yb = w.y * a.y * b.y * sf;
        __half2 h = __floats2half2_rn(ya, yb);
        float2 hf = __half22float2(h);
        __half2 l = __floats2half2_rn(ya - hf.x, yb - hf.y);
        y1[k] = h;
        y2[k] = l;
    }
    if (lane == 0) sy_inv[r] = 1.0 / s;
}

// ------------------------------------------------------------------ the GEMM
struct LiftArgs {
    const int2 *tiles;        // (u tile, vt tile), vt-major
    int ntiles, nK, U, UV;
    const int2 *vt_pairs;     // [UV]
    const long long *vt_off;  // [UV] offset of row (v,t) in Tsym
    const double *sx_inv, *sy_inv;
    float *Tsym;
    int *err;
};

// Persistent: CTA b takes tiles b, b + grid, ...; the MMA warp fills one TMEM
// accumulator while the epilogue warps drain the other.
__global__ void __launch_bounds__(192, 1) k_gamma_lift(const __grid_constant__ CUtensorMap tmX1,
                                                      const __grid_constant__ CUtensorMap tmX2,
                                                      const __grid_constant__ CUtensorMap tmY1,
                                                      const __grid_constant__ CUtensorMap tmY2, LiftArgs a)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + SP_STAGES * SP_STAGE_BYTES);
    // bars[0..S) full, [S..2S) empty, [2S..2S+2) accumulator full, [2S+2..2S+4) accumulator empty
    uint64_t *full = bars, *empty = bars + SP_STAGES, *afull = bars + 2 * SP_STAGES, *aempty = afull + 2;
    volatile uint32_t *tmem_slot = reinterpret_cast<volatile uint32_t *>(bars + 2 * SP_STAGES + 4);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(bars + 2 * SP_STAGES + 5);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nK = a.nK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < SP_STAGES; s++) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(smem_u32(&afull[b]), 1);
            mbar_init(smem_u32(&aempty[b]), 4);  // one arrival per epilogue warp
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32((const void *)tmem_slot)),
                     "r"(SP_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            long g = 0;
            for (int t = blockIdx.x; t < a.ntiles && !*abort_flag; t += gridDim.x) {
                const int2 tile = a.tiles[t];
                const int u0 = tile.x * SP_BM, vt0 = tile.y * SP_BN;
                for (int kc = 0; kc < nK; kc++, g++) {
                    const int s = (int)(g % SP_STAGES);
                    const long it = g / SP_STAGES;
                    if (it > 0 && !mbar_wait(smem_u32(&empty[s]), (uint32_t)((it - 1) & 1), abort_flag)) {
                        if (!*abort_flag) { *abort_flag = 1; atomicCAS(a.err, 0, 1); }
                        break;
                    }
                    uint8_t *st = smem + (size_t)s * SP_STAGE_BYTES;
                    const uint32_t fb = smem_u32(&full[s]);
                    mbar_expect_tx(fb, SP_STAGE_BYTES);
                    tma_load_2d(smem_u32(st), &tmX1, kc * SP_BK, u0, fb);
                    tma_load_2d(smem_u32(st + SP_A_BYTES), &tmX2, kc * SP_BK, u0, fb);
                    tma_load_2d(smem_u32(st + 2 * SP_A_BYTES), &tmY1, kc * SP_BK, vt0, fb);
                    tma_load_2d(smem_u32(st + 2 * SP_A_BYTES + SP_B_BYTES), &tmY2, kc * SP_BK, vt0, fb);
                }
            }
            // drain: wait for the copies of the last stages to land before the CTA can exit
            for (long h = (g > SP_STAGES ? g - SP_STAGES : 0); h < g; h++) {
                const int s = (int)(h % SP_STAGES);
                long long t0 = clock64();
                while (!mbar_try(smem_u32(&full[s]), (uint32_t)((h / SP_STAGES) & 1)) && clock64() - t0 < SP_WAIT_CYCLES) {
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            long g = 0;
            int tl = 0;
            for (int t = blockIdx.x; t < a.ntiles && !*abort_flag; t += gridDim.x, tl++) {
                const int acc = tl & 1, use = tl >> 1;
                if (use > 0 && !mbar_wait(smem_u32(&aempty[acc]), (uint32_t)((use - 1) & 1), abort_flag)) {
                    if (!*abort_flag) { *abort_flag = 1; atomicCAS(a.err, 0, 4); }
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t d = tmem + (uint32_t)(acc * SP_BN);
                for (int kc = 0; kc < nK; kc++, g++) {
                    const int s = (int)(g % SP_STAGES);
                    const long it = g / SP_STAGES;
                    if (!mbar_wait(smem_u32(&full[s]), (uint32_t)(it & 1), abort_flag)) {
                        if (!*abort_flag) { *abort_flag = 1; atomicCAS(a.err, 0, 2); }
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t st = smem_u32(smem + (size_t)s * SP_STAGE_BYTES);
                    const uint32_t x1 = st, x2 = st + SP_A_BYTES, y1 = st + 2 * SP_A_BYTES, y2 = y1 + SP_B_BYTES;
#pragma unroll
                    for (int kk = 0; kk < SP_BK / 16; kk++) {
                        const uint32_t o = kk * 32;  // 16 FP16 = 32 bytes along the swizzled row
                        umma_f16(d, umma_desc(x1 + o), umma_desc(y1 + o), (kc | kk) != 0);
                        umma_f16(d, umma_desc(x1 + o), umma_desc(y2 + o), 1);
                        umma_f16(d, umma_desc(x2 + o), umma_desc(y1 + o), 1);
                    }
                    umma_commit(smem_u32(&empty[s]));  // frees the stage when these MMAs finish
                }
                umma_commit(smem_u32(&afull[acc]));  // this tile's accumulator is complete
            }
        }
    } else {
        // epilogue: warps 2..5 own TMEM lanes 32*(warp % 4) .. +31
        const int lb = (warp & 3) * 32;
        int tl = 0;
        for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x, tl++) {
            const int acc = tl & 1, use = tl >> 1;
            const bool ok = mbar_wait(smem_u32(&afull[acc]), (uint32_t)(use & 1), abort_flag);
            if (!ok) {
                if (!*abort_flag) { *abort_flag = 1; atomicCAS(a.err, 0, 3); }
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int2 tile = a.tiles[t];
            const int u0 = tile.x * SP_BM, vt0 = tile.y * SP_BN;
            const int u = u0 + lb + lane;
            const double su = (u < a.U) ? a.sx_inv[u] : 0.0;
            for (int c0 = 0; c0 < SP_BN; c0 += 32) {
                float v[32];
                tmem_ld32(tmem + ((uint32_t)lb << 16) + (uint32_t)(acc * SP_BN + c0), v);
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    const int vt = vt0 + c0 + j;
                    if (vt < a.UV) {
                        const int2 p = a.vt_pairs[vt];
                        if (u <= p.x) a.Tsym[a.vt_off[vt] + u] = (float)((double)v[j] * su * a.sy_inv[vt]);
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&aempty[acc]));
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(SP_TMEM_COLS) : "memory");
    }
}

// ------------------------------------------------------------------ gather
// Gamma_mn = sum over the six orderings of T[sorted pair indices]; one thread
// per (m,n) of a 32x32 tile with tile(m) <= tile(n).
__global__ void __launch_bounds__(256) k_gamma_gather(int N, int P, int U, const int *__restrict__ triples,
                                                      const int *__restrict__ pidx, const long long *__restrict__ vbase,
                                                      const float *__restrict__ Tsym, double *__restrict__ gamma)
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
            int x = sp[mm[0] * P + nn[perm[s][0]]];
            int y = sp[mm[1] * P + nn[perm[s][1]]];
            int z = sp[mm[2] * P + nn[perm[s][2]]];
            int lo = min(x, min(y, z)), hi = max(x, max(y, z)), mid = x + y + z - lo - hi;
            g += (double)Tsym[sbase[mid] + (long long)(hi - mid) * (mid + 1) + lo];
        }
        gamma[(size_t)m * N + n] = g;
        gamma[(size_t)n * N + m] = g;
    }
}

// ------------------------------------------------------------------ host side
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::mutex g_encode_mu;

static modal_status get_encode()
{
    std::lock_guard<std::mutex> lock(g_encode_mu);
    if (g_encode) return MODAL_OK;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
        set_error("cuTensorMapEncodeTiled unavailable: %s", cudaGetErrorString(e));
        return MODAL_ERR_CUDA;
    }
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return MODAL_OK;
}

// 2D FP16 map over [rows][Kpad], box [box_rows][32], 64-byte swizzle.
static modal_status make_map(CUtensorMap *m, const void *base, long rows, int Kpad, int box_rows)
{
    cuuint64_t dims[2] = {(cuuint64_t)Kpad, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)Kpad * 2};
    cuuint32_t box[2] = {(cuuint32_t)SP_BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return MODAL_ERR_CUDA; }
    return MODAL_OK;
}

// Per-P tables, kept in the context's split buffers.
struct SplitPlan {
    int P = -1, U = 0, Upad = 0, UV = 0, UVpad = 0, ntiles = 0;
    long long ntsym = 0;
};

modal_status gamma_split_dev(modal_ctx *ctx, int mu0, int nmu)
{
    MODAL_TRY(get_encode());
    const int P = ctx->P, N = ctx->N;
    const double *mt = ctx->mt.as<double>() + (size_t)mu0 * P * P, *w = ctx->w.as<double>() + mu0;
    const int U = P * (P + 1) / 2;
    const int Upad = ceil_div(U, SP_BM) * SP_BM;
    const long UV = (long)U * (U + 1) / 2;
    const long UVpad = (long)ceil_div(UV, SP_BN) * SP_BN;
    const int Kpad = ceil_div(nmu, SP_KPAD) * SP_KPAD;
    const long long ntsym = (long long)U * (U + 1) * (U + 2) / 6;

    // host tables: pairs, pair index, vt pairs and offsets, tile list
    std::vector<int2> pairs(U);
    std::vector<int> pidx((size_t)P * P);
    {
        int u = 0;
        for (int p = 0; p < P; p++)
            for (int q = p; q < P; q++) { pairs[u] = make_int2(p, q); pidx[p * P + q] = pidx[q * P + p] = u; u++; }
    }
    std::vector<long long> vbase(U);
    {
        long long acc = 0;
        for (int v = 0; v < U; v++) { vbase[v] = acc; acc += (long long)(U - v) * (v + 1); }
    }
    std::vector<int2> vtp(UV);
    std::vector<long long> vto(UV);
    {
        long r = 0;
        for (int v = 0; v < U; v++)
            for (int t = v; t < U; t++) { vtp[r] = make_int2(v, t); vto[r] = vbase[v] + (long long)(t - v) * (v + 1); r++; }
    }
    std::vector<int2> tiles;
    for (long j = 0; j < UVpad / SP_BN; j++) {
        long last = std::min(UV - 1, (j + 1) * SP_BN - 1);
        int vmax = vtp[last].x;
        for (int i = 0; i * SP_BM <= vmax; i++) tiles.push_back(make_int2(i, (int)j));
    }

    // device buffers, laid out in ctx->split (one allocation)
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t o = 0;
    const size_t o_x1 = o; o += al((size_t)Upad * Kpad * 2);
    const size_t o_x2 = o; o += al((size_t)Upad * Kpad * 2);
    const size_t o_xf = o; o += al((size_t)U * Kpad * 4);
    const size_t o_sx = o; o += al((size_t)Upad * 8);
    const size_t o_y1 = o; o += al((size_t)UVpad * Kpad * 2);
    const size_t o_y2 = o; o += al((size_t)UVpad * Kpad * 2);
    const size_t o_sy = o; o += al((size_t)UVpad * 8);
    const size_t o_wf = o; o += al((size_t)Kpad * 4);
    const size_t o_pairs = o; o += al((size_t)U * sizeof(int2));
    const size_t o_pidx = o; o += al((size_t)P * P * 4);
    const size_t o_vbase = o; o += al((size_t)U * 8);
    const size_t o_vtp = o; o += al((size_t)UV * sizeof(int2));
    const size_t o_vto = o; o += al((size_t)UV * 8);
    const size_t o_tiles = o; o += al(tiles.size() * sizeof(int2));
    const size_t o_err = o; o += 256;
    const size_t o_T = o; o += al((size_t)ntsym * 4);
    MODAL_TRY(ensure(ctx->split, o));
    uint8_t *b = ctx->split.as<uint8_t>();
    __half *X1 = reinterpret_cast<__half *>(b + o_x1), *X2 = reinterpret_cast<__half *>(b + o_x2);
    __half *Y1 = reinterpret_cast<__half *>(b + o_y1), *Y2 = reinterpret_cast<__half *>(b + o_y2);
    float *xf = reinterpret_cast<float *>(b + o_xf), *wf = reinterpret_cast<float *>(b + o_wf);
    double *sx = reinterpret_cast<double *>(b + o_sx), *sy = reinterpret_cast<double *>(b + o_sy);
    int *err = reinterpret_cast<int *>(b + o_err);
    float *Tsym = reinterpret_cast<float *>(b + o_T);
    // the host tables depend on P and, through the offsets, on the K padding; a
    // reallocated buffer has lost them
    if (ctx->split_P != P || ctx->split_key != (long)Kpad || ctx->split_ptr != ctx->split.ptr ||
        ctx->split_bytes != ctx->split.bytes) {
        MODAL_CUDA(cudaMemcpyAsync(b + o_pairs, pairs.data(), U * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream));
        MODAL_CUDA(cudaMemcpyAsync(b + o_pidx, pidx.data(), pidx.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
        MODAL_CUDA(cudaMemcpyAsync(b + o_vbase, vbase.data(), U * 8, cudaMemcpyHostToDevice, ctx->stream));
        MODAL_CUDA(cudaMemcpyAsync(b + o_vtp, vtp.data(), UV * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream));
        MODAL_CUDA(cudaMemcpyAsync(b + o_vto, vto.data(), UV * 8, cudaMemcpyHostToDevice, ctx->stream));
        MODAL_CUDA(cudaMemcpyAsync(b + o_tiles, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                   ctx->stream));
        MODAL_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->split_P = P;
        ctx->split_key = Kpad;
        ctx->split_ptr = ctx->split.ptr;
        ctx->split_bytes = ctx->split.bytes;
    }
    MODAL_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));

    k_wgt48_f<<<ceil_div(Kpad, 256), 256, 0, ctx->stream>>>(nmu, Kpad, w, wf);
    MODAL_TRY(launched(ctx, "wgt48_f"));
    k_split_x<<<ceil_div((long)Upad * 32, 256), 256, 0, ctx->stream>>>(
        U, Upad, P, nmu, Kpad, reinterpret_cast<const int2 *>(b + o_pairs), mt, X1, X2, xf, sx);
    MODAL_TRY(launched(ctx, "split_x"));
    k_split_y<<<ceil_div(UVpad * 32, 256), 256, 0, ctx->stream>>>(
        (int)UV, (int)UVpad, Kpad, reinterpret_cast<const int2 *>(b + o_vtp), xf, wf, Y1, Y2, sy);
    MODAL_TRY(launched(ctx, "split_y"));

    CUtensorMap mx1, mx2, my1, my2;
    MODAL_TRY(make_map(&mx1, X1, Upad, Kpad, SP_BM));
    MODAL_TRY(make_map(&mx2, X2, Upad, Kpad, SP_BM));
    MODAL_TRY(make_map(&my1, Y1, UVpad, Kpad, SP_BN));
    MODAL_TRY(make_map(&my2, Y2, UVpad, Kpad, SP_BN));
    LiftArgs la;
    la.tiles = reinterpret_cast<const int2 *>(b + o_tiles);
    la.ntiles = (int)tiles.size();
    la.nK = Kpad / SP_BK;
    la.U = U;
    la.UV = (int)UV;
    la.vt_pairs = reinterpret_cast<const int2 *>(b + o_vtp);
    la.vt_off = reinterpret_cast<const long long *>(b + o_vto);
    la.sx_inv = sx;
    la.sy_inv = sy;
    la.Tsym = Tsym;
    la.err = err;
    MODAL_CUDA(cudaFuncSetAttribute(k_gamma_lift, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SP_SMEM));
    int nsm = 0;
    MODAL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
    const int grid = (int)std::min<long>((long)tiles.size(), (long)(nsm > 0 ? nsm : 1));
    {
        StageTimer tl(ctx, MODAL_T_LIFT);
        k_gamma_lift<<<grid, 192, SP_SMEM, ctx->stream>>>(mx1, mx2, my1, my2, la);
        MODAL_TRY(launched(ctx, "gamma_lift"));
    }

    MODAL_TRY(ensure(ctx->gamma, sizeof(double) * (size_t)N * N));
    size_t gsm = (size_t)U * 8 + (size_t)P * P * 4;
    MODAL_CUDA(cudaFuncSetAttribute(k_gamma_gather, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsm));
    const int nt = ceil_div(N, 32);
    k_gamma_gather<<<dim3(nt, nt), 256, gsm, ctx->stream>>>(N, P, U, ctx->triples.as<int>(),
                                                              reinterpret_cast<const int *>(b + o_pidx),
                                                              reinterpret_cast<const long long *>(b + o_vbase), Tsym,
                                                              ctx->gamma.as<double>());
    MODAL_TRY(launched(ctx, "gamma_gather"));
    int herr = 0;
    MODAL_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MODAL_CUDA(cudaStreamSynchronize(ctx->stream));
    if (herr) {
        set_error("gamma (split): a bounded wait in the tensor-core kernel expired (stage %d)", herr);
        return MODAL_ERR_TIMEOUT;
    }
    return MODAL_OK;
}

}  // namespace modal
