// common.cuh -- context state and helpers shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#include "../../include/modal_gb300.h"

namespace modal {

// Last error text (thread-local), returned by modal_last_error().
void set_error(const char *fmt, ...);

// Device buffer that grows on demand; contents are not preserved on growth.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    template <typename T> T *as() const { return static_cast<T *>(ptr); }
};

}  // namespace modal

namespace modal { struct BatchGraph; }

struct modal_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    long launches = 0;

    // problem description
    int lmin = 0, lmax = 0, L = 0, P = 0, N = 0, nmu = 0;
    bool have_basis = false, have_modes = false, have_user_gl = false;
    bool have_glint = false, have_gamma = false, have_spec = false, have_ortho = false;
    bool have_beta = false;
    bool have_mt = false;   // M table of the current quadrature computed (made on first use by the FP64 paths)
    int ortho_branch = 0, ortho_rank = 0;
    double pca_floor = 0.0;  // PCA keeps eigenvalues > pca_floor * e_max (0: the reference's > 0)
    modal::BatchGraph *batch = nullptr;  // captured batched-projection graph (batch.cu)
    long captures = 0;                   // graphs captured so far
    // tuned launch configurations (0: built-in defaults; set by modal_autotune)
    int proj_sg = 0, proj_cpb = 0, gamma_kc = 0;
    int proj_tc = 0;  // 1: FP32 projection on the tensor cores where P <= 32 (0: CUDA-core kernel)
    int beta_S = 0;

    // device state
    modal::DevBuf q;        // [L][P] basis
    modal::DevBuf triples;  // [N][3]
    modal::DevBuf mu, w;    // [nmu] quadrature
    modal::DevBuf pl;       // [lmax+1][nmu] (2l+1)^{2/3} P_l(mu_k), l-major
    modal::DevBuf mt;       // [nmu][P][P] l-contraction, mu-major
    modal::DevBuf gamma;    // [N][N]
    modal::DevBuf chol;     // [N][N] work: normalised Gamma -> L
    modal::DevBuf linv;     // [N][N] work: L^{-1}
    modal::DevBuf orthol;   // [N][N]
    modal::DevBuf lambdal;  // [N][N]
    modal::DevBuf norm;     // [N]
    modal::DevBuf info;     // [4] int status words
    modal::DevBuf cl;       // [lmax+1] C_l + N_l/b_l^2
    modal::DevBuf vl;       // [lmax+1] (2l+1)^{-1/3} w_l
    modal::DevBuf beta;     // [S][N]
    modal::DevBuf alpha;    // [S][N]
    modal::DevBuf modesr;   // [S][N]
    modal::DevBuf scratch;  // general work area
    modal::DevBuf scratch2;
    modal::DevBuf shape_tab;   // separable tables
    modal::DevBuf shape_desc;  // device shape descriptors
    modal::DevBuf slab_order;  // projection slab schedule
    modal::DevBuf split;       // split-precision Gamma: operand pieces, T table, per-P tables
    int split_P = -1;          // layout the tables in `split` were uploaded for: P, K padding, buffer
    long split_key = -1;
    void *split_ptr = nullptr;
    size_t split_bytes = 0;
    int gl_n = -1;             // n of the GPU quadrature held in mu/w (-1: none or caller-supplied)

    // late x primordial transfer Gamma
    int tr_Pp = 0, tr_xsize = 0, tr_Nprim = 0;
    modal::DevBuf tr_x;        // [xsize] grid, then [xsize] spline weights
    modal::DevBuf tr_qt;       // [xsize][Pp][lmax+1] transfer functions
    modal::DevBuf tr_prim;     // [Nprim][3]
    modal::DevBuf tr_mt;       // [xsize][nmu][Pp][P]
    modal::DevBuf tr_v;        // [lmax+1] weights
    modal::DevBuf tr_out;      // [XG][N][Nprim] partial sums per radial-sample group (polarised: group g of
                               // form f at (3g + f) N Nprim); only the first slice holds the result after the reduction
    bool tr_pol = false;       // E side of the transfer functions installed
    modal::DevBuf tr_qte;      // [xsize][Pp][lmax+1] E transfer functions
    modal::DevBuf tr_we;       // [2][lmax+1] E weights (q~_E factor, q~_T leakage factor)
    modal::DevBuf tr_mte;      // [xsize][nmu][Pp][P_E]

    // adjoint: shape legs and forward products, per-mu adjoints, upstreams
    modal::DevBuf adj, adj2, adj3;
    modal::DevBuf prune;  // basis pruning: normalised Gamma, minors, eigenvalues, work
    modal::DevBuf gemm_part;  // split-K partial sums of the skinny FP64 products (alpha solve)

    // polarisation: E basis, E-mode M table, TTE/TEE/EEE triples, their Gammas
    bool have_basis_e = false, have_pol = false, have_gamma_pol = false;
    int lmin_e = 0, lmax_e = 0, L_e = 0, P_e = 0;
    modal::DevBuf qe;         // [L_e][P_e]
    modal::DevBuf me;         // [nmu][P_e][P_e]
    modal::DevBuf tri_pol;    // [3][N][3]: TTE (T,T,E), TEE (T,E,E), EEE (E,E,E)
    modal::DevBuf gamma_pol;  // [3][N][N]

    // primordial k-space side (prim.cu): grid offsets, basis, chunk buffers
    modal::DevBuf prim;
    double *h_info = nullptr;  // pinned readback
    modal::DevBuf eigw;        // eigensolver workspace (syev.cu)
    modal::DevBuf ozw;         // tensor-core FP64 products: operand slices, exponents, tiles (ozgemm.cu)
    modal::DevBuf ozerr;       // their sticky error word
    modal::DevBuf ozrun;       // their work-item lists and K-split partial sums

    // profiling: event pairs per stage, summed on read
    bool profile = false;
    struct TimerRec { cudaEvent_t a, b; };
    std::vector<TimerRec> timers[MODAL_T_COUNT];
    std::vector<cudaEvent_t> event_pool;
};

namespace modal {

modal_status ensure(DevBuf &b, size_t bytes);
void release(DevBuf &b);
// FP64 symmetric eigen-decomposition (syev.cu).  A [n][n] (device, row-major,
// overwritten); W [n] ascending; select(W_host, n, arg, &first) -> number of
// eigenvectors wanted from ascending index first on; V rows hold them.
typedef int (*SyevSelect)(const double *w, int n, void *arg, int *first);
modal_status syev_dev(modal_ctx *ctx, int n, double *A, double *W, double *V, SyevSelect select, void *arg,
                      int *nvec, int *first);

#define MODAL_CUDA(call)                                                                  \
    do {                                                                                  \
        cudaError_t err__ = (call);                                                       \
        if (err__ != cudaSuccess) {                                                       \
            ::modal::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,                 \
                               cudaGetErrorString(err__));                                \
            return MODAL_ERR_CUDA;                                                        \
        }                                                                                 \
    } while (0)

#define MODAL_TRY(expr)                                                                   \
    do {                                                                                  \
        modal_status st__ = (expr);                                                       \
        if (st__ != MODAL_OK) return st__;                                                \
    } while (0)

// Check the last launch; counts it on the context.
inline modal_status launched(modal_ctx *ctx, const char *what)
{
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("launch %s: %s", what, cudaGetErrorString(e));
        return MODAL_ERR_CUDA;
    }
    return MODAL_OK;
}

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

// Stage timer: records an event at construction and at stop() when profiling.
struct StageTimer {
    modal_ctx *ctx;
    int id;
    cudaEvent_t a = nullptr;
    StageTimer(modal_ctx *c, int i);
    void stop();
    ~StageTimer() { stop(); }
};

// ---- entry points implemented per translation unit (internal) ----
modal_status gl_nodes_dev(modal_ctx *ctx, int n, double *d_mu, double *d_w);
modal_status legendre_table_dev(modal_ctx *ctx, int nmu, int lmax, const double *d_mu, double *d_pl);
modal_status mij_dev(modal_ctx *ctx);
// The FP64 M table of the current basis and quadrature, computed on first use.
modal_status mt_ready(modal_ctx *ctx);
modal_status mij_table_dev(modal_ctx *ctx, const double *q, int lmin, int lmax, int P, DevBuf &out);
// Gamma over the quadrature nodes mu0 .. mu0 + nmu - 1 (all of them: mu0 = 0, nmu = ctx->nmu).
modal_status gamma_fp64_dev(modal_ctx *ctx, int mu0, int nmu);
modal_status gamma_split_dev(modal_ctx *ctx, int mu0, int nmu);
modal_status ortho_dev(modal_ctx *ctx, int pca_flag);
modal_status project_dev(modal_ctx *ctx, int S, const modal_shape *shapes, modal_prec prec);
modal_status alpha_dev(modal_ctx *ctx, int S);
modal_status lambdainv_dev(modal_ctx *ctx);  // linv = lower triangle of orthol
modal_status transpose_dev(modal_ctx *ctx, const double *in, double *out, int R, int C);
modal_status basis_legendre_dev(modal_ctx *ctx, int size, int pmax, double min, double max, const double *d_values,
                                double *d_out);
modal_status geometric_dev(modal_ctx *ctx, long npts, const int *d_pts, double *d_out);

// dq[L][P] (device, accumulated) += the Gamma adjoint for an upstream dL/dGamma G[N][N] (device).
modal_status gamma_vjp_accum_dev(modal_ctx *ctx, const double *G, double *dq);

// Device descriptor of one shape (projection kernels).
struct DShape {
    int kind, nterms;
    long tab_off;  // FP64 tables: [term][f, g, h][l] from this double offset
    double c1, c2, c3, sigma;
    long tab_off_f = 0;  // FP32 form: [parity of l][l / 2][term][f, g, h, 0] from this float offset
};

// Internal shape kind of the 3D transfer Gamma: the radial integral s_n(l1,l2,l3)
// of primordial mode n = DShape::nterms (calculate_sijk_TTT), arguments below.
constexpr int SHAPE_RADIAL = 2;
struct RadialArgs {
    const double *qt = nullptr;  // [xsize][Pp][L1] transfer functions q~_p(l, x)
    const double *x = nullptr;   // [xsize] radial grid
    const double *wq = nullptr;  // [L1] (2l+1)^{1/6}/sqrt(C_l + N_l/b_l^2), 0 for l < 2
    const int *prim = nullptr;   // [Nprim][3] primordial triples
    int xsize = 0, Pp = 0, L1 = 0;
};

// A planned projection: validated descriptors, buffer offsets, launch shape.
struct ProjPlan {
    int S = 0;
    modal_prec prec = MODAL_PREC_FP64;
    long tab_total = 0;
    std::vector<DShape> desc;
    int SG = 8, CPL = 1, cpb = 0, nsm = 0, fpt = 0;
    size_t smem = 0, o_q = 0, o_v = 0, o_t = 0, o_s = 0, o_F = 0, o_B = 0, o_c = 0, o_w = 0, o_sb = 0;
    long long npts = 0;  // tetrapyd points (FP32 weight table entries)
    long tabf_total = 0;  // floats of the FP32 separable tables
    RadialArgs ra;        // radial shapes (3D transfer Gamma only)
    int max_nterms = 0;
    bool tc = false;        // tensor-core slab kernel (FP32 form, P <= 32)
    int Mpad = 0;           // compact k entries per row of its BF16 q pieces
    size_t o_bq = 0, o_perm = 0;
    std::vector<int> perm;  // shape order of its work items (by kind and term count)
};
// plan: validate, size every buffer, upload the slab schedule (may allocate);
// stage: copy shape tables/descriptors to the device; record: enqueue the
// device work only (no allocation, no host round trip: capturable).
modal_status proj_plan(modal_ctx *ctx, int S, const modal_shape *shapes, modal_prec prec, ProjPlan &pl);
modal_status proj_stage(modal_ctx *ctx, const ProjPlan &pl, const modal_shape *shapes);
modal_status proj_record(modal_ctx *ctx, const ProjPlan &pl);

// Frees the captured batched-projection graph and its pinned staging buffers.
void batch_release(modal_ctx *ctx);

// FP64 tiled GEMM on the context stream:
//   C[m][n] = beta*C[m][n] + alpha * sum_k opA(m,k) opB(k,n)
//   opA(m,k) = transA ? A[k*lda+m] : A[m*lda+k];  opB(k,n) = transB ? B[n*ldb+k] : B[k*ldb+n]
//   lower != 0: only entries with n <= m (tiles above the diagonal skipped).
modal_status dgemm(modal_ctx *ctx, int M, int N, int K, double alpha, const double *A, int lda, bool transA,
                   const double *B, int ldb, bool transB, double beta, double *C, int ldc, int lower);
// FP64-accuracy product on the FP16 tensor cores by exact integer slices
// (ozgemm.cu): C = beta C + alpha op(A) op(B), s slices of 7 bits (2..8).
//   op(A)(m,k) = transA ? A[k*lda+m] : A[m*lda+k];  op(B)(k,n) = transB ? B[n*ldb+k] : B[k*ldb+n]
modal_status oz_gemm(modal_ctx *ctx, int M, int N, int K, double alpha, const double *A, long lda, bool transA,
                     const double *B, long ldb, bool transB, double beta, double *C, long ldc, int lower, int s);
struct OzOpts {
    int slices = 8;      // 7-bit digits per operand (8: the FP64 accuracy class)
    int lower = 0;       // square C: only n <= m
    int diag_tiles = 0;  // > 0: only the diagonal blocks of that many 128-tiles
    int ksplit = 0;      // K split over work items (0: fill the GPU)
    bool check = true;   // synchronise and report an expired wait now (else: oz_check later)
};
// Sliced operand of the tensor-core product: [s][rows_pad][Kpad] FP16 digits and
// the per-row exponents (rows_pad a multiple of 128, Kpad of 64).
struct OzOperand {
    __half *slices;
    int *ex;
    int rows, rows_pad;
};
// Digits of the rows of op(X) (R x K; trans: element (r, k) = X[k*ld + r]).
modal_status oz_slice(modal_ctx *ctx, int R, int K, const double *X, long ld, bool trans, int s, int Rpad, int Kpad,
                      __half *out, int *ex);
// C (M x N = A.rows x B.rows) = beta C + alpha A B^T over pre-sliced operands;
// tile_list: the 128 x 128 output tiles to compute (NULL: all, or per o.lower / o.diag_tiles).
modal_status oz_run(modal_ctx *ctx, const OzOperand &A, const OzOperand &B, int Kpad, int s,
                    const std::vector<int2> *tile_list, double alpha, double beta, double *C, long ldc, const OzOpts &o);
modal_status oz_reset(modal_ctx *ctx);  // clear the sticky error word of unchecked calls
modal_status oz_check(modal_ctx *ctx);  // synchronise; MODAL_ERR_TIMEOUT if any call's wait expired
modal_status oz_gemm_ex(modal_ctx *ctx, int M, int N, int K, double alpha, const double *A, long lda, bool transA,
                        const double *B, long ldb, bool transB, double beta, double *C, long ldc, const OzOpts &o);
// C (+)= A op(B) for A [S][K] with few rows S: skinny kernels for S <= 32 (alpha 1; accumulate: C +=)
modal_status dgemm_rows(modal_ctx *ctx, int S, int N, int K, const double *A, int lda, const double *B, int ldb,
                        bool transB, double *C, int ldc, bool accumulate);
// dgemm with K split over CTAs for small output grids and long K (alpha 1; accumulate: C +=)
modal_status dgemm_splitk(modal_ctx *ctx, int M, int N, int K, const double *A, int lda, bool transA, const double *B,
                          int ldb, bool transB, double *C, int ldc, int lower, bool accumulate);

}  // namespace modal
