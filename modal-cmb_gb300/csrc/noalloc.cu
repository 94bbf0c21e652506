// noalloc.cu -- FP64 Gamma that allocates no device memory.
//
// Who needs this: code that runs where device allocation is not allowed or
// not possible -- inside an arena-managed engine that owns all device memory
// and forbids cudaMalloc/cudaFree (they synchronise the device and fragment
// the arena), plugins loaded into a host process that hands them
// pre-allocated buffers, and tight loops where an allocation per call would
// stall.  Such callers pass device buffers for the inputs and
// the output; every intermediate (quadrature, P_l table, l-contraction)
// lives in one fixed array compiled into this library.
//
// The intermediates live in `g_noalloc_scratch`, a file-scope __device__ array
// of MODAL_NOALLOC_SCRATCH_BYTES (8 MiB).  Every GPU that loads the library
// holds those 8 MiB until the process exits.  In host code the array's name
// is only a host-side stand-in, not a device address, so on the first call
// on each device (with that device current) the entry point asks the runtime
// for the real address with cudaGetSymbolAddress and remembers it; later
// calls on that device reuse it.  The address is kept for the life of the
// process, so the device must not be reset (cudaDeviceReset) while the
// library is loaded.  Every call reads a status word back into a host
// variable and waits for its stream before returning, so no call (first or
// later) can be made while a stream is being captured into a CUDA graph.
//
// Every call shares the one array and overwrites it; the kernels fully
// rewrite every region they read, so nothing needs clearing between calls.
// Calls that overlap on the GPU (on different streams, or from several host
// threads) race on the array: serialise them, e.g. by issuing them all on
// one stream.
//
// The kernels are the ones the regular FP64 path launches (gl.cu,
// gamma_fp64.cu); only the buffers differ.
#include <mutex>
#include "common.cuh"

#define MODAL_NOALLOC_MAX_DEVICES 64

namespace modal {

// Kernels defined in gl.cu and gamma_fp64.cu.
__global__ void k_gl_nodes(int n, double *mu, double *w);
__global__ void k_pl_factors(int lmax, double *pw);
__global__ void k_legendre_table(int nmu, int lmax, const double *mu, const double *pw, double *pl);
__global__ void k_mij_fp64(int nmu, int lmin, int lmax, int P, int npair, const double *pl, const double *q,
                           const int2 *pairs, double *mt);
__global__ void k_wgt48(int nmu, const double *w, double *wg);
__global__ void k_gamma_fp64(int N, int P, int nmu, int KC, const int *triples, const double *mt,
                             const double *wg, double *gamma);

// Launch geometry of k_mij_fp64 (its tile: 64 mu x 32 pairs, 256 threads) and
// of k_gamma_fp64 (32 x 32 mode tile, 256 threads), as in gamma_fp64.cu.
constexpr int NA_MIJ_BK = 64, NA_MIJ_BU = 32;

static __device__ __align__(256) unsigned char g_noalloc_scratch[MODAL_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void *g_noalloc_addr[MODAL_NOALLOC_MAX_DEVICES];

// (p,q) with p <= q for every pair index u, as the regular path uploads
// them; also clears the status word before the triples are checked.
__global__ void k_noalloc_pairs(int P, int2 *pairs, int *status)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    *status = 0;
    int u = 0;
    for (int p = 0; p < P; p++)
        for (int q = p; q < P; q++) pairs[u++] = make_int2(p, q);
}

// Copy the caller's mode triples into scratch; an index outside [0,P) is
// replaced by 0 and flagged, so the Gamma kernel never reads outside its tile.
__global__ void k_noalloc_triples(int N, int P, const int *__restrict__ in, int *__restrict__ out, int *status)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3 * N) return;
    int v = in[e];
    if (v < 0 || v >= P) {
        atomicExch(status, 1);
        v = 0;
    }
    out[e] = v;
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace modal

using namespace modal;

extern "C" modal_status modal_gamma_fp64_noalloc(int lmin, int lmax, int P, const double *d_q, int N,
                                                 const int *d_triples, int nmu, const double *d_nodes,
                                                 const double *d_weights, double *d_gamma, void *stream)
{
    if (lmin < 0 || lmax < lmin || P < 1 || P > 64 || N < 1 || !d_q || !d_triples || !d_gamma) {
        set_error("modal_gamma_fp64_noalloc: lmin=%d lmax=%d P=%d N=%d (1 <= P <= 64, N >= 1, non-NULL buffers)",
                  lmin, lmax, P, N);
        return MODAL_ERR_ARG;
    }
    const bool own_nodes = (d_nodes == nullptr);
    if (own_nodes != (d_weights == nullptr)) {
        set_error("modal_gamma_fp64_noalloc: pass both d_nodes and d_weights, or neither");
        return MODAL_ERR_ARG;
    }
    if (own_nodes) nmu = 3 * lmax / 2 + 1;  // orthogonalisation_late.c:37
    if (nmu < 1) { set_error("modal_gamma_fp64_noalloc: nmu=%d", nmu); return MODAL_ERR_ARG; }
    // the P_l table kernel keeps 3 (lmax + 1) doubles in shared memory (<= 48 KB)
    if (lmax > 2000) { set_error("modal_gamma_fp64_noalloc: lmax=%d above 2000", lmax); return MODAL_ERR_ARG; }
    const int npair = P * (P + 1) / 2;
    // scratch layout: status, triples[3N], wg[nmu], pw[lmax+1], pairs[npair], mu[nmu], w[nmu],
    //                 pl[(lmax+1) nmu], mt[nmu P P]
    size_t off_status = 0;
    size_t off_tr = off_status + 256;
    size_t off_wg = off_tr + align256(sizeof(int) * 3 * (size_t)N);
    size_t off_pw = off_wg + align256(sizeof(double) * nmu);
    size_t off_pairs = off_pw + align256(sizeof(double) * (lmax + 1));
    size_t off_mu = off_pairs + align256(sizeof(int2) * npair);
    size_t off_w = off_mu + align256(own_nodes ? sizeof(double) * nmu : 0);
    size_t off_pl = off_w + align256(own_nodes ? sizeof(double) * nmu : 0);
    size_t off_mt = off_pl + align256(sizeof(double) * (size_t)(lmax + 1) * nmu);
    size_t need = off_mt + align256(sizeof(double) * (size_t)nmu * P * P);
    if (need > MODAL_NOALLOC_SCRATCH_BYTES) {
        set_error("modal_gamma_fp64_noalloc: lmax=%d, n_mu=%d, P=%d need %zu bytes of scratch; the built-in "
                  "scratch holds %u bytes (use modal_gamma for larger problems)",
                  lmax, nmu, P, need, (unsigned)MODAL_NOALLOC_SCRATCH_BYTES);
        return MODAL_ERR_ARG;
    }
    int dev = 0;
    MODAL_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MODAL_NOALLOC_MAX_DEVICES) { set_error("modal_gamma_fp64_noalloc: device %d", dev); return MODAL_ERR_ARG; }
    unsigned char *base;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                set_error("modal_gamma_fp64_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
                return MODAL_ERR_CUDA;
            }
            g_noalloc_addr[dev] = p;
        }
        base = static_cast<unsigned char *>(g_noalloc_addr[dev]);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int *status = reinterpret_cast<int *>(base + off_status);
    int *triples = reinterpret_cast<int *>(base + off_tr);
    double *wg = reinterpret_cast<double *>(base + off_wg);
    double *pw = reinterpret_cast<double *>(base + off_pw);
    int2 *pairs = reinterpret_cast<int2 *>(base + off_pairs);
    double *pl = reinterpret_cast<double *>(base + off_pl);
    double *mt = reinterpret_cast<double *>(base + off_mt);
    const double *mu = d_nodes, *w = d_weights;
    if (own_nodes) {
        double *mu_s = reinterpret_cast<double *>(base + off_mu), *w_s = reinterpret_cast<double *>(base + off_w);
        k_gl_nodes<<<ceil_div(nmu / 2 + 1, 64), 64, 0, s>>>(nmu, mu_s, w_s);
        mu = mu_s;
        w = w_s;
    }
    k_pl_factors<<<ceil_div(lmax + 1, 256), 256, 0, s>>>(lmax, pw);
    // the table kernel keeps its integer factors in 3 (lmax + 1) doubles of shared
    // memory (at most 24 KB for the problems the scratch array admits)
    k_legendre_table<<<ceil_div(nmu, 32), 32, sizeof(double) * 3 * (size_t)(lmax + 1), s>>>(nmu, lmax, mu, pw, pl);
    k_noalloc_pairs<<<1, 1, 0, s>>>(P, pairs, status);
    k_noalloc_triples<<<ceil_div(3L * N, 256), 256, 0, s>>>(N, P, d_triples, triples, status);
    dim3 gm(ceil_div(nmu, NA_MIJ_BK), ceil_div(npair, NA_MIJ_BU));
    k_mij_fp64<<<gm, 256, 0, s>>>(nmu, lmin, lmax, P, npair, pl, d_q, pairs, mt);
    k_wgt48<<<ceil_div(nmu, 256), 256, 0, s>>>(nmu, w, wg);
    int KC = (96 * 1024) / (P * P * 8);
    if (KC < 1) KC = 1;
    if (KC > 32) KC = 32;
    size_t smem = sizeof(double) * ((size_t)KC + (size_t)KC * P * P);
    MODAL_CUDA(cudaFuncSetAttribute(k_gamma_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int nt = ceil_div(N, 32);
    k_gamma_fp64<<<dim3(nt, nt), 256, smem, s>>>(N, P, nmu, KC, triples, mt, wg, d_gamma);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { set_error("modal_gamma_fp64_noalloc: launch: %s", cudaGetErrorString(e)); return MODAL_ERR_CUDA; }
    // read the triples check back into a stack word (no allocation); this also
    // makes the call return with Gamma complete
    int h_status = 0;
    MODAL_CUDA(cudaMemcpyAsync(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost, s));
    MODAL_CUDA(cudaStreamSynchronize(s));
    if (h_status) {
        set_error("modal_gamma_fp64_noalloc: a mode triple has a basis index outside [0,%d); Gamma is not valid", P);
        return MODAL_ERR_ARG;
    }
    return MODAL_OK;
}
