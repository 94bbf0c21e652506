/* modal_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the
 * Modal-CMB mode-space hot path: Gauss-Legendre quadrature, the P_l(mu)
 * table, the l-contraction M/A(mu), the Gamma matrix of inner products of
 * symmetrised separable modes, its orthogonalisation, the projection of
 * bispectrum shapes onto the modes and the alpha solve.
 *
 * Plain C: pointers, sizes and status codes; no CUDA or torch types.  Host
 * pointers are caller-owned; device buffers are owned by the context.  Each
 * context owns one CUDA stream; calls on one context are stream-ordered and
 * blocking unless stated; a context is not thread-safe (like the reference's
 * module-static state).  Layouts are the reference's: row-major FP64 arrays
 * exactly as its fwrite'd files (arrays.c:6-21).
 *
 * Each entry point names the reference function it replaces (file:line in
 * the Modal-CMB sources).
 */
#ifndef MODAL_GB300_H
#define MODAL_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MODAL_OK = 0,
    MODAL_ERR_ARG = 1,      /* bad size, NULL pointer, mode index out of range */
    MODAL_ERR_CUDA = 2,     /* CUDA runtime failure; text in modal_last_error() */
    MODAL_ERR_NOT_PD = 3,   /* Cholesky met a non-positive pivot; *info = pivot row */
    MODAL_ERR_TIMEOUT = 4,  /* a bounded device wait gave up */
    MODAL_ERR_NOMEM = 5,    /* device allocation failed */
    MODAL_ERR_STATE = 6,    /* a prerequisite call is missing (basis, modes, ...) */
    MODAL_ERR_NOCONV = 7    /* iterative eigensolver did not converge */
} modal_status;

typedef enum {
    MODAL_PREC_FP64 = 0,    /* plain form: FP64 throughout */
    MODAL_PREC_SPLIT = 1    /* split-precision tensor-core form, FP64 accumulation */
} modal_prec;

typedef enum {
    MODAL_SHAPE_SEPARABLE = 0, /* S = sum_t (1/6) sum_perm f_t(l1) g_t(l2) h_t(l3) */
    MODAL_SHAPE_BUMP = 1       /* S = exp(-|(l1,l2,l3)/(l1+l2+l3) - c|^2 / (2 sigma^2)) */
} modal_shape_kind;

/* One bispectrum shape, evaluated on the device at each tetrapyd point
 * (replaces the per-point callback calculate_3D_bispectrum,
 * calculate_mode_3D.c:266-281). */
typedef struct {
    int kind;            /* modal_shape_kind */
    int nterms;          /* SEPARABLE: number of terms T */
    const double *tab;   /* SEPARABLE: host [T][3][lmax+1]: f_t, g_t, h_t over l = 0..lmax */
    double c[3];         /* BUMP: centre */
    double sigma;        /* BUMP: width */
} modal_shape;

typedef struct modal_ctx modal_ctx;

/* ---------------------------------------------------------------- context */

/* Create a context on CUDA device `device` with its own stream. */
modal_status modal_ctx_create(int device, modal_ctx **out);
void modal_ctx_destroy(modal_ctx *ctx);
/* Text of the last failure on the calling thread ("" if none). */
const char *modal_last_error(void);
/* The context's cudaStream_t, as an opaque pointer (for event timing). */
void *modal_ctx_stream(modal_ctx *ctx);
/* Number of CUDA kernels this context has launched so far. */
long modal_ctx_launches(const modal_ctx *ctx);
/* Block until all work on the context's stream is done. */
modal_status modal_ctx_sync(modal_ctx *ctx);

/* Per-stage device timers (CUDA events on the context's stream).  With
 * profiling enabled every stage below records an event pair around its
 * kernels; modal_ctx_timer synchronises and returns the summed milliseconds
 * and the number of timed runs since the last reset.  No reference
 * counterpart (the reference prints CPU times, mtime.c:17-25). */
typedef enum {
    MODAL_T_GL = 0,       /* Gauss-Legendre nodes */
    MODAL_T_PL = 1,       /* P_l(mu) table */
    MODAL_T_MIJ = 2,      /* l-contraction */
    MODAL_T_GAMMA = 3,    /* mu-contraction (Gamma) */
    MODAL_T_ORTHO = 4,    /* orthogonalisation */
    MODAL_T_PROJECT = 5,  /* projection of the shapes */
    MODAL_T_ALPHA = 6,    /* alpha solve */
    MODAL_T_LIFT = 7,     /* split form: the tensor-core GEMM of the mu-contraction alone */
    MODAL_T_ADJOINT = 8,  /* gradients with respect to the basis values */
    MODAL_T_PRUNE = 9,    /* greedy basis pruning */
    MODAL_T_EIG_TRD = 10, /* eigensolver: Householder tridiagonalisation */
    MODAL_T_EIG_DC = 11,  /* eigensolver: divide and conquer on the tridiagonal matrix */
    MODAL_T_EIG_BACK = 12, /* eigensolver: back-transformation of the kept eigenvectors */
    MODAL_T_TC = 13,      /* every FP64-accuracy tensor-core product kernel (k_oz_gemm) */
    MODAL_T_EIG_PANEL = 14, /* eigensolver: the tridiagonalisation's panel kernels alone */
    MODAL_T_COUNT = 15
} modal_timer;
modal_status modal_ctx_profile(modal_ctx *ctx, int enable);
modal_status modal_ctx_timer(modal_ctx *ctx, int timer, double *ms, long *count);
modal_status modal_ctx_timer_reset(modal_ctx *ctx);

/* ------------------------------------------------- stand-alone primitives */

/* Gauss-Legendre nodes and weights on [-1,1], ascending, computed on the GPU.
 * Replaces asy() (gl_integration.c:46-168; global.h:421).  Same layout:
 * symmetric pairs, exact 0 middle node for odd n. */
modal_status modal_gl_nodes(int n, double *nodes, double *weights);

/* out[k][l] = (2l+1)^{2/3} P_l(mu[k]), l = 0..lmax, FP64 three-term
 * recurrence on the GPU.  Replaces the gl_Pl loop with gsl_sf_legendre_Pl
 * (orthogonalisation_late.c:47-54). */
modal_status modal_legendre_table(int nmu, int lmax, const double *mu, double *out);

/* Shifted Legendre basis out[i][j] = P_j(2(values[i]-min)/(max-min) - 1),
 * j = 0..pmax.  Replaces basis_functions_legendre (basis_functions.c:88-107;
 * global.h:361). */
modal_status modal_basis_legendre(int size, int pmax, double min, double max,
                                  const double *values, double *out);

/* Asymptotic geometric factor h~^2(l1,l2,l3) at npts points pts[n][3].
 * Replaces calculate_geometric (calculate_geometric.c:59-92; global.h:370). */
modal_status modal_geometric(long npts, const int *pts, double *out);

/* Number of tetrapyd points lmin <= i <= j <= k <= lmax, k <= i+j, i+j+k even,
 * as counted by decompose_tetrapyd_XXX (tetrapyd_tools.c:31-51). */
modal_status modal_tetrapyd_count(int lmin, int lmax, long *count);

/* ------------------------------------------------------------- pipeline */

/* Install the 1D basis q[L][P] (L = lmax-lmin+1; layout of basis_late_T,
 * fixed_data.c:1764) for l = lmin..lmax.  Resets everything derived from it.
 * Replaces the basis reads of init_orthol_glint (orthogonalisation_late.c:56-64). */
modal_status modal_set_basis(modal_ctx *ctx, int lmin, int lmax, int P, const double *q);

/* Install the mode list triples[N][3] (order_late_TTT layout,
 * set_terms_late fixed_data.c:272-467 / find_perm_late_TTT :983-990). */
modal_status modal_set_modes(modal_ctx *ctx, int N, const int *triples);

/* Optional: use caller-supplied quadrature (e.g. the output of the
 * reference's asy()) instead of the GPU nodes.  nodes/weights[nmu]. */
modal_status modal_set_gl(modal_ctx *ctx, int nmu, const double *nodes, const double *weights);

/* GL nodes (n_mu = 3 lmax/2 + 1 unless set), P_l table and the l-contraction
 * M[i][j][k] for all P^2 (i,j) in FP64.  Replaces init_orthol_glint
 * (orthogonalisation_late.c:23-97) + calculate_orthoMij_T for all pairs
 * (:99-129, ortho_late_mpi.c:170-225) + sync_orthoMij (:159-237). */
modal_status modal_init_glint(modal_ctx *ctx);

/* Download M as Mij_T[P][P][n_mu] (orthogonalisation_late.c:76). */
modal_status modal_get_mij(modal_ctx *ctx, double *out);
/* Download the quadrature in use (n_mu values each). */
modal_status modal_get_gl(modal_ctx *ctx, int *nmu, double *nodes, double *weights);

/* Gamma[N][N] = <Q_m, Q_n> with the 1/(48 pi) GL weight, full symmetric
 * matrix, same scale as calculate_orthol (orthogonalisation_late.c:239-336)
 * filled over all pairs and symmetrised (ortho_late_mpi.c:231-363).
 * gamma may be NULL: the result stays on the device for the next steps. */
modal_status modal_gamma(modal_ctx *ctx, modal_prec prec, double *gamma);

/* Gamma restricted to the quadrature nodes mu_begin .. mu_end - 1 (0 <= mu_begin <
 * mu_end <= n_mu): the sum over the nodes in calculate_orthol
 * (orthogonalisation_late.c:272-296) taken over that node range only.  Partials over disjoint ranges that
 * cover all nodes add up to Gamma, so Gamma shards over the mu axis with one sum
 * reduction of N x N doubles; the reference splits the (m, n) pairs over ranks
 * instead (ortho_late_mpi.c:242-255).  gamma [N][N] on the host is required; the
 * context's device Gamma is left invalid (a partial), so modal_orthogonalise
 * needs the summed Gamma passed in. */
modal_status modal_gamma_partial(modal_ctx *ctx, modal_prec prec, int mu_begin, int mu_end, double *gamma);

/* result[0] = Gamma_mn (and result[1..3] = TTE, TEE, EEE after
 * modal_set_modes_pol), the per-pair interface of calculate_orthol
 * (orthogonalisation_late.c:239; global.h:211).  Computes the whole matrix
 * on first use and answers later pairs from it. */
modal_status modal_orthol_pair(modal_ctx *ctx, int m, int n, double *result);

/* Orthogonalise Gamma (ortho_late_mpi.c:724-876): normalise by sqrt(diag),
 * then either Cholesky (orthol = D^{1/2} L, lambdal = L^{-1} D^{-1/2}) or,
 * when pca_flag == 0 or the normalised Gamma is not positive definite, the
 * PCA branch on its eigen-decomposition.  gamma: host [N][N] or NULL for
 * the device result of modal_gamma.  orthol/lambdal: host [N][N] or NULL
 * (kept on the device).  *branch = 0 Cholesky, 1 PCA; *rank = number of
 * retained eigenvalues (N for Cholesky).  FP64 on the GPU. */
modal_status modal_orthogonalise(modal_ctx *ctx, const double *gamma, int pca_flag,
                                 double *orthol, double *lambdal, int *branch, int *rank);

/* Install C_l + N_l/b_l^2 for l = 0..lmax (get_cl_TT etc., used for the
 * per-leg weight w_l = (2l+1)^{1/6}/sqrt(.) of calculate_mode_3D.c:53-62). */
modal_status modal_set_spectrum(modal_ctx *ctx, const double *cl);

/* beta[s][r] = sum over the tetrapyd of permsix h~^2 prod(2l+1)^{-1/3}
 * S_s(l1,l2,l3) w_l1 w_l2 w_l3 Q_r(l1,l2,l3) for S shapes in one call.
 * Replaces calculate_mode_3D (calculate_mode_3D.c:217-264) driven over
 * decompose_tetrapyd_XXX blocks (eigenmodetoday_mpi.c:235-273).  beta may be
 * NULL (kept on the device for modal_alpha). */
modal_status modal_project(modal_ctx *ctx, int S, const modal_shape *shapes, modal_prec prec,
                           double *beta);

/* modify_bispectrum (calculate_modes.c:6-45) on the GPU, in place on the host
 * array b[size][size][size]: b <- c_i c_j c_k h~^2(l_i,l_j,l_k) (1.55e-8)^2 b on
 * even-parity triangle triples (l = vec[index]), 0 elsewhere;
 * c_i = beam_i / ((2 l_i + 1)^{1/6} sqrt(beam_i^2 cl_i + noise_i)) when cl_i != 0
 * and l_i != 0.  cl, beam, noise, vec: [size], indexed like b. */
modal_status modal_modify_bispectrum(int size, const int *vec, const double *cl, const double *beam,
                                     const double *noise, double *b);

/* calculate_modes (calculate_modes.c:47-79) for every mode at once:
 * beta[r] = sum over i <= j <= k < size of m(i,j,k) plijk_TTT(r,i,j,k) b[i][j][k]
 * (m = 1, 3, 6 orderings; the array index is the multipole l, as in the
 * reference).  b: host [size][size][size], typically after
 * modal_modify_bispectrum.  beta: host [N] or NULL (kept for modal_alpha). */
modal_status modal_calculate_modes(modal_ctx *ctx, int size, const double *b, double *beta);

/* Late x primordial transfer Gamma (calculate_gamma.c, default path of
 * gamma_mpi.c: init_gamma_glint :48-250, precompute_gammaMij_T :254-303,
 * gamma_2d_pt_TTT :512-555, calculate_gamma_2d :773-842 with
 * integrate_cubic_spline :845-934).  Install the radial grid xvec[xsize]
 * (increasing, xsize >= 4), the raw transfer functions
 * qtilde[xsize][Pp][lmax+1] = q~_p(l, x) (get_qtilde_T(p, l, x)) and the
 * primordial mode triples prim[Nprim][3] (find_perm_prim). */
modal_status modal_set_transfer(modal_ctx *ctx, int Pp, int xsize, const double *xvec, const double *qtilde,
                                int Nprim, const int *prim);

/* gamma_t[m][n] = calculate_gamma_2d(m, n)[0] for every late mode m < N and
 * primordial mode n < Nprim, with weight (2l+1)^{5/6}/sqrt(C_l + N_l/b_l^2)
 * from modal_set_spectrum and scale deltaphi^2/(8 pi).  FP64 on the GPU. */
modal_status modal_gamma_transfer(modal_ctx *ctx, double deltaphi, double *gamma_t);

/* The 3D transfer Gamma, gamma_mpi.c's rflag_do3D == 0 path: gamma_t[m][n] =
 * 6 deltaphi^2 sum over the tetrapyd (l = 2..lmax) of permsix h~^2 prod
 * (2l+1)^{-1/3} plijk_TTT(m, l1, l2, l3) s_n(l1, l2, l3), where s_n is the
 * trapezium x-integral of calculate_sijk_TTT (calculate_gamma_TTT_3D_nested,
 * calculate_gamma_3d.c:274-440, 783-860; init_gamma_3Dint :23-60), for every
 * late mode m < N and primordial mode n < Nprim (the reference sizes the
 * matrix by the primordial count and fills m < Nprim).  Inputs as for
 * modal_gamma_transfer (modal_set_transfer, modal_set_spectrum).  FP64 on the
 * GPU: each primordial mode is projected as one radial shape. */
modal_status modal_gamma_transfer_3d(modal_ctx *ctx, double deltaphi, double *gamma_t);

/* Load an orthogonalisation computed elsewhere, as eigenmodetoday_mpi.c reads
 * it from the orthol_TTT / lambdal_TTT files (read_orthol / read_lambdal,
 * fixed_data.c:3453-3469, 3749-3788): orthol and lambdal host [N][N]
 * row-major.  modal_alpha then forms alpha = lambdal^T lambdal beta and
 * modesR from the lower triangle of orthol (eigenmodetoday_mpi.c:148-162,
 * 303-316), as after modal_orthogonalise.  Needs the modes (N). */
modal_status modal_set_ortho(modal_ctx *ctx, const double *orthol, const double *lambdal);

/* Eigenvalue floor of the PCA branch: keep the leading eigenvalues of the
 * normalised Gamma above floor * (largest eigenvalue).  0 (the default) is the
 * reference's rule, every positive eigenvalue (ortho_late_mpi.c:786-792).  At
 * cond ~1e16 the smallest kept eigenvalues are rounding noise and alpha
 * amplifies any perturbation of Gamma or beta by 1/e; a floor above the
 * relative error of Gamma (about 1e-7 for the split form) makes alpha
 * reproducible.  Takes effect at the next modal_orthogonalise. */
modal_status modal_set_pca_floor(modal_ctx *ctx, double floor);

/* Kernel of the FP32 (MODAL_PREC_SPLIT) projection: 1 runs the point-by-basis
 * contraction of each slab on the tcgen05 tensor cores (three exact BF16
 * pieces per operand, six products, FP32 tensor-memory sums per 32-point
 * chunk, Kahan across chunks) where P <= 32; 0 (default), or P > 32, runs the
 * CUDA-core FP32 slab kernel.  Both evaluate every shape at every point on the
 * CUDA cores, which is most of the work, so the tensor-core form is not the
 * faster one on GB300; modal_autotune times both.  modal_get_proj_kernel
 * reports which one the current basis uses.  No reference counterpart. */
modal_status modal_set_proj_kernel(modal_ctx *ctx, int tensor_cores);
modal_status modal_get_proj_kernel(const modal_ctx *ctx, int *tensor_cores);

/* Eigen-decomposition of the symmetric n x n matrix a (host, row-major; only
 * read): every eigenvalue in ascending order in w[n], and, when v is not NULL,
 * the eigenvectors as rows of v[n][n] (row j belongs to w[j]).  FP64 on the
 * GPU (Householder tridiagonalisation, divide and conquer, back-
 * transformation).  Replaces gsl_eigen_symmv + gsl_eigen_symmv_sort
 * (ortho_late_mpi.c:775-776, which sorts descending) and LAPACKE_dsyevr
 * (basis_optimisation_mpi.c:279); the PCA branch of modal_orthogonalise and
 * modal_basis_prune use the same solver. */
modal_status modal_eigh(modal_ctx *ctx, int n, const double *a, double *w, double *v);

/* C = beta C + alpha op(A) op(B) for row-major host arrays (op(A) M x K,
 * op(B) K x N, C M x N; trans* != 0 takes the transpose), with FP64
 * accuracy on the FP16 tensor cores: each row of op(A) and column of op(B) is
 * scaled by a power of two and cut into `slices` (2..8) exact 7-bit integer
 * digits, the digit products are summed exactly in the tensor memory over
 * blocks of 512 terms and the blocks in double-FP32.  slices = 8 gives the
 * accuracy class of an FP64 product.  No reference counterpart: the library's
 * eigensolver and Gamma use the same products internally. */
modal_status modal_gemm_f64(modal_ctx *ctx, int M, int N, int K, double alpha, const double *A, int transA,
                            const double *B, int transB, double beta, double *C, int slices);

/* Batched projection replayed from a captured CUDA graph.  Same inputs,
 * result and FP64/FP32 forms as modal_project (beta: host [S][N], required;
 * it also stays on the device for modal_alpha).  The first call for a batch
 * layout -- S, and each shape's kind and term count -- captures the device
 * work (staging copies from pinned buffers, the slab kernel over all shapes,
 * the reductions, the copy of beta back) into a graph; later calls with the
 * same layout copy the new values into the pinned staging buffers and launch
 * the graph once.  A change of layout, basis size or of any buffer the graph
 * uses is detected and re-captured.  No reference counterpart (the reference
 * re-walks the tetrapyd per shape, calculate_mode_3D.c:217-264). */
modal_status modal_project_batch(modal_ctx *ctx, int S, const modal_shape *shapes, modal_prec prec, double *beta);
/* Number of CUDA graphs this context has captured. */
long modal_ctx_captures(const modal_ctx *ctx);

/* Launch-configuration tuner.  Times the candidate configurations of the
 * FP32 projection (the tensor-core kernel where P <= 32; the CUDA-core kernel
 * with shapes per CTA and grid or persistent 1-2 CTAs per SM) and of the FP64
 * Gamma kernel (mu steps per shared-memory stage) on this
 * context's problem, keeps the fastest, and appends them to the text file
 * cache_path (NULL: no file) keyed by GPU architecture and problem size; a
 * later call that finds its keys there applies them without timing.  Needs
 * basis, modes and spectrum.  No reference counterpart. */
modal_status modal_autotune(modal_ctx *ctx, const char *cache_path);
/* The configuration in effect (0 = built-in default). */
modal_status modal_get_tuning(const modal_ctx *ctx, int *proj_sg, int *proj_cpb, int *gamma_kc);

/* alpha = lambdal^T lambdal beta and modesR = orthol^T alpha
 * (eigenmodetoday_mpi.c:148-162, 286-316) for S shapes, FP64 on the GPU.
 * beta: host [S][N] or NULL for the device result of modal_project.
 * alpha/modesR: host [S][N] or NULL. */
modal_status modal_alpha(modal_ctx *ctx, int S, const double *beta, double *alpha, double *modesR);

/* ----------------------------------------------------------- polarisation */

/* E-mode basis qe[L_E][P_E] (basis_late_E layout, fixed_data.c) on
 * l = lmin_e..lmax_e: the do_polarisation side of init_orthol_glint
 * (orthogonalisation_late.c:33-37, 68-95).  With it the quadrature and the
 * P_l table cover max(lmax_T, lmax_E), and modal_init_glint also builds the E
 * table (calculate_orthoMij_E, :131-157).  Resets everything derived. */
modal_status modal_set_basis_e(modal_ctx *ctx, int lmin_e, int lmax_e, int P_e, const double *qe);

/* Mode triples of the polarised lists, N each (N of modal_set_modes), in the
 * conventions of find_perm_late_TTE/TEE/EEE (fixed_data.c): tte[n] = (T,T,E),
 * tee[n] = (T,E,E), eee[n] = (E,E,E) basis indices.  With them
 * modal_orthol_pair also fills result[1..3]. */
modal_status modal_set_modes_pol(modal_ctx *ctx, const int *tte, const int *tee, const int *eee);

/* Gamma_TTE, Gamma_TEE, Gamma_EEE [N][N] (host, each may be NULL): results
 * [1], [2], [3] of calculate_orthol with do_polarisation
 * (orthogonalisation_late.c:293-320) over every pair, FP64 on the GPU. */
modal_status modal_gamma_pol(modal_ctx *ctx, double *gamma_tte, double *gamma_tee, double *gamma_eee);

/* Spectra for the E side of the transfer Gamma, arrays over l = 0..lmax_T:
 * signal C_l, beams b_l and noise N_l of TT, TE and EE, and the sky
 * fractions (get_cl_XX, get_beam_XX, get_noise_XX, fskyT/fskyE of the
 * reference's fixed_data.c / parameter.c). */
typedef struct {
    const double *cl_tt, *cl_te, *cl_ee;
    const double *beam_tt, *beam_te, *beam_ee;
    const double *noise_tt, *noise_te, *noise_ee;
    double fsky_t, fsky_e;
} modal_pol_spectra;

/* E transfer functions qtilde_e[xsize][Pp][lmax_T+1] (get_qtilde_E, same grid
 * and primordial basis as modal_set_transfer) and the spectra of the E weights
 * (calculate_gamma.c:142-183):
 *   EEweight_l = (2l+1)^{5/6} b_E / sqrt(s_TT (s_TT s_EE - s_TE^2)),
 *   q~_E' = EEweight (s_TT q~_E - (sqrt(fsky_E/fsky_T) b_TE^2 C_TE + N_TE) q~_T),
 *   s_XY = b_X b_Y C_XY + N_XY.
 * Needs modal_set_transfer, modal_set_basis_e (lmax_E <= lmax_T) and
 * modal_set_modes_pol.  The TT weight keeps using modal_set_spectrum's
 * C_l + N_l/b_l^2, which must equal (b_TT^2 C_TT + N_TT)/b_TT^2 here. */
modal_status modal_set_transfer_pol(modal_ctx *ctx, const double *qtilde_e, const modal_pol_spectra *spectra);

/* Gamma_t TTE, TEE, EEE [N][Nprim] (host, each may be NULL): results [1..3]
 * of calculate_gamma_2d with do_polarisation (calculate_gamma.c:558-687,
 * 773-842), scale deltaphi^2/(8 pi), FP64 on the GPU. */
modal_status modal_gamma_transfer_pol(modal_ctx *ctx, double deltaphi, double *gamma_tte, double *gamma_tee,
                                      double *gamma_eee);

/* ------------------------------------------------- primordial k-space side */

/* Points of the primordial k-grid tetrapyd in the order of get_ijk_next_prim
 * from (min,min,min) (tetrapyd_tools.c:416-550): min <= i < max, i <= j <= max,
 * j <= k <= min(max, i+j+2), then the end point (max,max,max) that
 * decompose_tetrapyd_prim also counts.  *npts = their number; pts[npts][3]
 * (host, or NULL for the count only) enumerated on the current GPU. */
modal_status modal_prim_points(int min, int max, long *npts, int *pts);

/* Gram matrix of the primordial modes on that grid, calculate_ortho
 * (orthogonalisation.c:14-86): sum over points of
 *   calculate_weight(min,max,i,j,k) dk^3 / (dk (i+j+k)) pijk_r pijk_s,
 * dk = kmax/max, pijk the symmetrised product of basis[l][p] (get_basis_prim,
 * basis [max+1][P] on grid indices), modes prim[N][3] (find_perm_prim).
 * ortho: host [N(N+1)/2], the reference's packed upper triangle (r <= s,
 * row by row).  FP64 on the GPU. */
modal_status modal_prim_ortho(modal_ctx *ctx, int min, int max, double kmax, int P, const double *basis, int N,
                              const int *prim, double *ortho);

/* Projection of S primordial shapes onto the modes, calculate_eigen
 * (calculate_eigen.c:86-144): alpha[s][r] = sum over points of the same weight
 * times S_s pijk_r, and norm2[s] = sum weight S_s^2 (integrate_template2,
 * :13-84; NULL to skip).  Shapes as modal_shape with separable tables over
 * grid indices 0..max; min >= 1.  FP64 on the GPU. */
modal_status modal_prim_eigen(modal_ctx *ctx, int min, int max, double kmax, int P, const double *basis, int N,
                              const int *prim, int S, const modal_shape *shapes, double *alpha, double *norm2);

/* ---------------------------------------------------------------- adjoint */

/* Gradients with respect to the basis values q[L][P] of modal_set_basis, FP64
 * on the GPU.  No counterpart in the reference: its basis optimisation
 * (basis_optimisation_mpi.c:199-337) prunes modes greedily by the smallest
 * eigenvalue of leave-one-out Gamma submatrices and has no derivatives; these
 * entries give the gradient such a search (or a continuous optimiser over
 * basis coefficients) follows.
 *
 * The shape side works in Gamma's own inner product: separable shapes
 * (MODAL_SHAPE_SEPARABLE only) are weighted per l like the basis,
 * w_l = (2l+1)^{1/6}/sqrt(C_l + N_l/b_l^2) from modal_set_spectrum
 * (calculate_mode_3D.c:53-62), and projected through the Gauss-Legendre form
 * of h^2 (the exact one Gamma uses), so that <S,S> - beta^T Gamma^{-1} beta
 * is the squared residual of the shape's projection onto the modes. */

/* beta[S][N] = <S_s, Q_n> and norm2[S] = <S_s, S_s> (host, either NULL). */
modal_status modal_project_gl(modal_ctx *ctx, int S, const modal_shape *shapes, double *beta, double *norm2);

/* dL_dq[L][P] (host) for an upstream dL_dgamma[N][N] (host) through the FP64
 * Gamma of the current basis/modes/quadrature (modal_gamma, both forms). */
modal_status modal_gamma_vjp(modal_ctx *ctx, const double *dL_dgamma, double *dL_dq);

/* dL_dq[L][P] for an upstream dL_dbeta[S][N] through modal_project_gl. */
modal_status modal_project_gl_vjp(modal_ctx *ctx, int S, const modal_shape *shapes, const double *dL_dbeta,
                                  double *dL_dq);

/* alpha[S][N] = Gamma^{-1} beta = lambdal^T lambdal beta with beta from
 * modal_project_gl and lambdal from modal_orthogonalise (the alpha solve of
 * eigenmodetoday_mpi.c:148-162); with dL_dalpha[S][N] also dL_dq[L][P]
 * (both or neither).  Exact when the orthogonalisation took the Cholesky
 * branch (lambdal^T lambdal = Gamma^{-1}); on the PCA branch the gradient is
 * that of the truncated pseudo-inverse with the eigenvectors held fixed. */
modal_status modal_alpha_gl(modal_ctx *ctx, int S, const modal_shape *shapes, double *alpha, const double *dL_dalpha,
                            double *dL_dq);

/* Basis-quality objective: the mean relative squared projection residual
 *   J = (1/S) sum_s (<S_s,S_s> - beta_s^T Gamma^{-1} beta_s) / <S_s,S_s>
 * (0 when every shape lies in the span of the modes), and dJ_dq[L][P] (host,
 * NULL to skip).  Needs modal_gamma (FP64) and modal_orthogonalise first. */
modal_status modal_adjoint_residual(modal_ctx *ctx, int S, const modal_shape *shapes, double *J, double *dJ_dq);

/* ----------------------------------------------------------- basis pruning */

/* Greedy basis pruning of basis_optimisation_mpi.c:184-337.  Over the modes
 * not in faillist[nfail] (the reference's faillist file, :134-147), Gamma is
 * normalised to unit diagonal (:184-190); then, while two or more modes are
 * active, the mode whose removal leaves the normalised Gamma with the largest
 * smallest eigenvalue is removed (first maximum, :256-312).  order[t] is the
 * mode removed at step t and lambda_min[t] that largest smallest eigenvalue;
 * the last entry is the surviving mode with lambda_min = 1, as the reference
 * prints it (:326-343).  Both arrays are host [N - nfail].  gamma: host
 * [N][N] (the master Gamma the reference reads, :90-109) or NULL for the
 * device Gamma of modal_gamma (N must match).  Every leave-one-out smallest
 * eigenvalue comes from one eigendecomposition per step (FP64, the library's
 * own eigensolver) and
 * the secular equation of the minor (see prune.cu), not one eigensolve per
 * candidate.  Repeated or out-of-range fail-list entries give MODAL_ERR_ARG
 * (the reference would mis-size its active list). */
modal_status modal_basis_prune(modal_ctx *ctx, int N, const double *gamma, int nfail, const int *faillist, int *order,
                               double *lambda_min);

/* The reference's basis-quality figure as an objective: the smallest
 * eigenvalue of the normalised device Gamma (of modal_gamma), its eigenvector
 * eigvec[N] (host, or NULL) and the gradient dlam_dq[L][P] (host, or NULL)
 * with respect to the basis values, through the Gamma adjoint. */
modal_status modal_lambda_min(modal_ctx *ctx, double *lambda_min, double *eigvec, double *dlam_dq);

/* ------------------------------------------------- allocation-free Gamma */

/* FP64 Gamma for callers that cannot allocate device memory: code running
 * inside an engine that owns every device byte and forbids cudaMalloc/cudaFree
 * (which synchronise the device and fragment its arena), or a plugin that is
 * handed pre-allocated buffers.  No
 * counterpart in the reference (it allocates with malloc on the host).
 *
 * All buffers are DEVICE pointers owned by the caller: d_q[L][P] basis
 * (L = lmax-lmin+1), d_triples[N][3], optional d_nodes/d_weights[nmu] (both
 * NULL: n_mu = 3 lmax/2 + 1 GPU nodes; nmu is then ignored), d_gamma[N][N]
 * output.  Same result as modal_gamma(..., MODAL_PREC_FP64, ...) with the
 * same quadrature.  Work runs on `stream` (a cudaStream_t, NULL = default
 * stream); the call waits for it to finish before returning.
 *
 * The intermediates live in one 8 MiB array built into the library
 * (MODAL_NOALLOC_SCRATCH_BYTES); every GPU that loads the library holds it
 * until exit.  Problems needing more (about lmax <= 500 with P <= 10, or
 * lmax <= 600 with P <= 6, fit) are rejected with MODAL_ERR_ARG and a
 * message giving the size needed; no device memory is ever allocated.
 * Every call reads a status word back into host memory and waits for
 * `stream` before returning, so NO call may be made while a stream is being
 * captured into a CUDA graph (the copy and the synchronisation are illegal
 * during capture and would invalidate the caller's capture).  The first call
 * on a device looks up the array's device address; that address is kept for
 * the life of the process, so do not reset the device while the library is
 * loaded.  All calls share the array: calls that overlap on the GPU
 * (different streams or threads) race, so serialise them.
 * Out-of-range triples give MODAL_ERR_ARG. */
#define MODAL_NOALLOC_SCRATCH_BYTES (8u << 20)
modal_status modal_gamma_fp64_noalloc(int lmin, int lmax, int P, const double *d_q, int N,
                                      const int *d_triples, int nmu, const double *d_nodes,
                                      const double *d_weights, double *d_gamma, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MODAL_GB300_H */
