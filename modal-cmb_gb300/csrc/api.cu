// api.cu -- C ABI: context management, argument checks, host<->device copies,
// and dispatch to the kernels in the other translation units.
#include <cstdarg>
#include <cstdlib>
#include <vector>
#include <algorithm>
#include "common.cuh"

namespace modal {

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

modal_status ensure(DevBuf &b, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return MODAL_OK;
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    cudaError_t e = cudaMalloc(&b.ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b.ptr = nullptr;
        set_error("cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
        return MODAL_ERR_NOMEM;
    }
    b.bytes = bytes;
    return MODAL_OK;
}

void release(DevBuf &b)
{
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
}

// A throw-away context on the current device for the stand-alone primitives.
struct TempCtx {
    modal_ctx ctx;
    bool ok = false;
    TempCtx()
    {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) { cudaGetLastError(); return; }
        if (cudaGetDevice(&ctx.device) != cudaSuccess) return;
        if (cudaStreamCreateWithFlags(&ctx.stream, cudaStreamNonBlocking) != cudaSuccess) return;
        ok = true;
    }
    ~TempCtx()
    {
        DevBuf *bufs[] = {&ctx.scratch, &ctx.scratch2};
        for (DevBuf *b : bufs) release(*b);
        if (ctx.stream) cudaStreamDestroy(ctx.stream);
        ctx.stream = nullptr;
    }
};

static modal_status h2d(modal_ctx *c, DevBuf &b, const void *src, size_t bytes)
{
    MODAL_TRY(ensure(b, bytes));
    MODAL_CUDA(cudaMemcpyAsync(b.ptr, src, bytes, cudaMemcpyHostToDevice, c->stream));
    return MODAL_OK;
}

static modal_status d2h(modal_ctx *c, void *dst, const void *src, size_t bytes)
{
    MODAL_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
    return MODAL_OK;
}

static modal_status sync(modal_ctx *c)
{
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    return MODAL_OK;
}

static modal_status need(modal_ctx *c, bool ok, const char *what)
{
    if (!c) { set_error("context is NULL"); return MODAL_ERR_ARG; }
    if (!ok) { set_error("%s", what); return MODAL_ERR_STATE; }
    return MODAL_OK;
}

static cudaEvent_t take_event(modal_ctx *c)
{
    if (!c->event_pool.empty()) {
        cudaEvent_t e = c->event_pool.back();
        c->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    return e;
}

StageTimer::StageTimer(modal_ctx *c, int i) : ctx(c), id(i)
{
    if (ctx && ctx->profile) {
        a = take_event(ctx);
        if (a) cudaEventRecord(a, ctx->stream);
    }
}

void StageTimer::stop()
{
    if (!a) return;
    cudaEvent_t b = take_event(ctx);
    if (b) {
        cudaEventRecord(b, ctx->stream);
        ctx->timers[id].push_back({a, b});
    } else {
        ctx->event_pool.push_back(a);
    }
    a = nullptr;
}

static void timers_clear(modal_ctx *c)
{
    for (auto &v : c->timers) {
        for (auto &r : v) { c->event_pool.push_back(r.a); c->event_pool.push_back(r.b); }
        v.clear();
    }
}

}  // namespace modal

using namespace modal;

extern "C" {

const char *modal_last_error(void) { return g_err; }

modal_status modal_ctx_create(int device, modal_ctx **out)
{
    if (!out) { set_error("modal_ctx_create: out is NULL"); return MODAL_ERR_ARG; }
    *out = nullptr;
    int ndev = 0;
    MODAL_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) { set_error("modal_ctx_create: device %d of %d", device, ndev); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(device));
    modal_ctx *c = new modal_ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; set_error("stream: %s", cudaGetErrorString(e)); return MODAL_ERR_CUDA; }
    *out = c;
    return MODAL_OK;
}

void modal_ctx_destroy(modal_ctx *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    DevBuf *bufs[] = {&c->q, &c->triples, &c->mu, &c->w, &c->pl, &c->mt, &c->gamma, &c->chol, &c->linv,
                      &c->orthol, &c->lambdal, &c->norm, &c->info, &c->cl, &c->vl, &c->beta, &c->alpha,
                      &c->modesr, &c->scratch, &c->scratch2, &c->shape_tab, &c->shape_desc, &c->slab_order,
                      &c->split, &c->tr_x, &c->tr_qt, &c->tr_prim, &c->tr_mt, &c->tr_v, &c->tr_out,
                      &c->adj, &c->adj2, &c->adj3, &c->prune, &c->gemm_part, &c->qe, &c->me, &c->tri_pol, &c->gamma_pol,
                      &c->tr_qte, &c->tr_we, &c->tr_mte, &c->prim, &c->eigw, &c->ozw, &c->ozerr, &c->ozrun};
    batch_release(c);
    for (DevBuf *b : bufs) release(*b);
    timers_clear(c);
    for (cudaEvent_t e : c->event_pool) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

modal_status modal_ctx_profile(modal_ctx *c, int enable)
{
    if (!c) { set_error("ctx is NULL"); return MODAL_ERR_ARG; }
    c->profile = enable != 0;
    return MODAL_OK;
}

modal_status modal_ctx_timer(modal_ctx *c, int id, double *ms, long *count)
{
    if (!c || id < 0 || id >= MODAL_T_COUNT) { set_error("modal_ctx_timer: bad args"); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    MODAL_TRY(sync(c));
    double tot = 0.0;
    for (auto &r : c->timers[id]) {
        float t = 0.f;
        MODAL_CUDA(cudaEventElapsedTime(&t, r.a, r.b));
        tot += t;
    }
    if (ms) *ms = tot;
    if (count) *count = (long)c->timers[id].size();
    return MODAL_OK;
}

modal_status modal_ctx_timer_reset(modal_ctx *c)
{
    if (!c) { set_error("ctx is NULL"); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    MODAL_TRY(sync(c));
    timers_clear(c);
    return MODAL_OK;
}

void *modal_ctx_stream(modal_ctx *c) { return c ? (void *)c->stream : nullptr; }
long modal_ctx_launches(const modal_ctx *c) { return c ? c->launches : 0; }

modal_status modal_ctx_sync(modal_ctx *c)
{
    if (!c) { set_error("ctx is NULL"); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    return sync(c);
}

// ------------------------------------------------------------- primitives

modal_status modal_gl_nodes(int n, double *nodes, double *weights)
{
    if (n < 1 || !nodes || !weights) { set_error("modal_gl_nodes: n=%d", n); return MODAL_ERR_ARG; }
    TempCtx t;
    if (!t.ok) { set_error("modal_gl_nodes: no CUDA device"); return MODAL_ERR_CUDA; }
    DevBuf dm, dw;
    modal_status st = ensure(dm, sizeof(double) * n);
    if (st == MODAL_OK) st = ensure(dw, sizeof(double) * n);
    if (st == MODAL_OK) st = gl_nodes_dev(&t.ctx, n, dm.as<double>(), dw.as<double>());
    if (st == MODAL_OK) st = d2h(&t.ctx, nodes, dm.ptr, sizeof(double) * n);
    if (st == MODAL_OK) st = d2h(&t.ctx, weights, dw.ptr, sizeof(double) * n);
    if (st == MODAL_OK) st = sync(&t.ctx);
    release(dm);
    release(dw);
    return st;
}

modal_status modal_legendre_table(int nmu, int lmax, const double *mu, double *out)
{
    if (nmu < 1 || lmax < 0 || !mu || !out) { set_error("modal_legendre_table: bad args"); return MODAL_ERR_ARG; }
    TempCtx t;
    if (!t.ok) { set_error("modal_legendre_table: no CUDA device"); return MODAL_ERR_CUDA; }
    DevBuf dm, dp, dt;
    size_t tb = sizeof(double) * (size_t)nmu * (lmax + 1);
    modal_status st = h2d(&t.ctx, dm, mu, sizeof(double) * nmu);
    if (st == MODAL_OK) st = ensure(dp, tb);
    if (st == MODAL_OK) st = ensure(dt, tb);
    if (st == MODAL_OK) st = legendre_table_dev(&t.ctx, nmu, lmax, dm.as<double>(), dp.as<double>());
    // device layout is l-major [lmax+1][nmu]; gl_Pl is [nmu][lmax+1]
    if (st == MODAL_OK) st = transpose_dev(&t.ctx, dp.as<double>(), dt.as<double>(), lmax + 1, nmu);
    if (st == MODAL_OK) st = d2h(&t.ctx, out, dt.ptr, tb);
    if (st == MODAL_OK) st = sync(&t.ctx);
    release(dm);
    release(dp);
    release(dt);
    return st;
}

modal_status modal_basis_legendre(int size, int pmax, double min, double max, const double *values, double *out)
{
    if (size < 1 || pmax < 0 || !values || !out || !(max != min)) { set_error("modal_basis_legendre: bad args"); return MODAL_ERR_ARG; }
    TempCtx t;
    if (!t.ok) { set_error("modal_basis_legendre: no CUDA device"); return MODAL_ERR_CUDA; }
    DevBuf dv, dout;
    size_t ob = sizeof(double) * (size_t)size * (pmax + 1);
    modal_status st = h2d(&t.ctx, dv, values, sizeof(double) * size);
    if (st == MODAL_OK) st = ensure(dout, ob);
    if (st == MODAL_OK) st = basis_legendre_dev(&t.ctx, size, pmax, min, max, dv.as<double>(), dout.as<double>());
    if (st == MODAL_OK) st = d2h(&t.ctx, out, dout.ptr, ob);
    if (st == MODAL_OK) st = sync(&t.ctx);
    release(dv);
    release(dout);
    return st;
}

modal_status modal_geometric(long npts, const int *pts, double *out)
{
    if (npts < 0 || (npts > 0 && (!pts || !out))) { set_error("modal_geometric: bad args"); return MODAL_ERR_ARG; }
    if (npts == 0) return MODAL_OK;
    TempCtx t;
    if (!t.ok) { set_error("modal_geometric: no CUDA device"); return MODAL_ERR_CUDA; }
    DevBuf dp, dout;
    modal_status st = h2d(&t.ctx, dp, pts, sizeof(int) * 3 * (size_t)npts);
    if (st == MODAL_OK) st = ensure(dout, sizeof(double) * (size_t)npts);
    if (st == MODAL_OK) st = geometric_dev(&t.ctx, npts, dp.as<int>(), dout.as<double>());
    if (st == MODAL_OK) st = d2h(&t.ctx, out, dout.ptr, sizeof(double) * (size_t)npts);
    if (st == MODAL_OK) st = sync(&t.ctx);
    release(dp);
    release(dout);
    return st;
}

modal_status modal_tetrapyd_count(int lmin, int lmax, long *count)
{
    if (!count || lmin < 0 || lmax < lmin) { set_error("modal_tetrapyd_count: bad args"); return MODAL_ERR_ARG; }
    long n = 0;
    for (int i = lmin; i <= lmax; i++)
        for (int j = i; j <= lmax; j++) {
            int kf = j + (i & 1), k1 = (i + j < lmax) ? i + j : lmax;
            if (k1 >= kf) n += (k1 - kf) / 2 + 1;
        }
    *count = n;
    return MODAL_OK;
}

// ------------------------------------------------------------- pipeline

modal_status modal_set_basis(modal_ctx *c, int lmin, int lmax, int P, const double *q)
{
    MODAL_TRY(need(c, true, ""));
    if (lmin < 0 || lmax < lmin || P < 1 || P > 64 || !q) {
        set_error("modal_set_basis: lmin=%d lmax=%d P=%d (1 <= P <= 64)", lmin, lmax, P);
        return MODAL_ERR_ARG;
    }
    MODAL_CUDA(cudaSetDevice(c->device));
    c->lmin = lmin;
    c->lmax = lmax;
    c->L = lmax - lmin + 1;
    c->P = P;
    MODAL_TRY(h2d(c, c->q, q, sizeof(double) * (size_t)c->L * P));
    MODAL_TRY(sync(c));
    c->have_basis = true;
    c->have_glint = c->have_gamma = c->have_ortho = c->have_beta = false;
    c->have_pol = c->have_gamma_pol = false;  // polarised modes are re-set after the bases
    if (c->have_modes) {
        // re-validate the mode list against the new basis size
        std::vector<int> tr(3 * (size_t)c->N);
        MODAL_TRY(d2h(c, tr.data(), c->triples.ptr, sizeof(int) * tr.size()));
        MODAL_TRY(sync(c));
        for (int v : tr)
            if (v < 0 || v >= P) { c->have_modes = false; break; }
    }
    return MODAL_OK;
}

modal_status modal_set_modes(modal_ctx *c, int N, const int *triples)
{
    MODAL_TRY(need(c, c && c->have_basis, "modal_set_modes: set the basis first"));
    if (N < 1 || !triples) { set_error("modal_set_modes: N=%d", N); return MODAL_ERR_ARG; }
    for (long e = 0; e < 3L * N; e++)
        if (triples[e] < 0 || triples[e] >= c->P) {
            set_error("modal_set_modes: mode %ld has basis index %d outside [0,%d)", e / 3, triples[e], c->P);
            return MODAL_ERR_ARG;
        }
    MODAL_CUDA(cudaSetDevice(c->device));
    c->N = N;
    MODAL_TRY(h2d(c, c->triples, triples, sizeof(int) * 3 * (size_t)N));
    MODAL_TRY(sync(c));
    c->have_modes = true;
    c->have_gamma = c->have_ortho = c->have_beta = false;
    c->have_pol = c->have_gamma_pol = false;
    return MODAL_OK;
}

modal_status modal_set_gl(modal_ctx *c, int nmu, const double *nodes, const double *weights)
{
    MODAL_TRY(need(c, true, ""));
    if (nmu < 1 || !nodes || !weights) { set_error("modal_set_gl: nmu=%d", nmu); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    c->nmu = nmu;
    MODAL_TRY(h2d(c, c->mu, nodes, sizeof(double) * nmu));
    MODAL_TRY(h2d(c, c->w, weights, sizeof(double) * nmu));
    c->gl_n = -1;
    MODAL_TRY(sync(c));
    c->have_user_gl = true;
    c->have_glint = c->have_gamma = c->have_ortho = false;
    return MODAL_OK;
}

modal_status modal_init_glint(modal_ctx *c)
{
    MODAL_TRY(need(c, c && c->have_basis, "modal_init_glint: set the basis first"));
    MODAL_CUDA(cudaSetDevice(c->device));
    // with an E basis the quadrature and the P_l table cover max(lmax_T, lmax_E)
    // (orthogonalisation_late.c:33-37)
    const int lmax_all = c->have_basis_e ? std::max(c->lmax, c->lmax_e) : c->lmax;
    if (!c->have_user_gl) {
        c->nmu = 3 * lmax_all / 2 + 1;  // orthogonalisation_late.c:37
        if (c->gl_n != c->nmu) {      // the nodes depend on n only: computed once per n
            MODAL_TRY(ensure(c->mu, sizeof(double) * c->nmu));
            MODAL_TRY(ensure(c->w, sizeof(double) * c->nmu));
            StageTimer t(c, MODAL_T_GL);
            MODAL_TRY(gl_nodes_dev(c, c->nmu, c->mu.as<double>(), c->w.as<double>()));
            c->gl_n = c->nmu;
        }
    }
    MODAL_TRY(ensure(c->pl, sizeof(double) * (size_t)(lmax_all + 1) * c->nmu));
    {
        StageTimer t(c, MODAL_T_PL);
        MODAL_TRY(legendre_table_dev(c, c->nmu, lmax_all, c->mu.as<double>(), c->pl.as<double>()));
    }
    // the FP64 M table (calculate_orthoMij_T) is made on first use by the FP64
    // paths (mt_ready); the split form contracts the P_l table on the tensor cores
    c->have_mt = false;
    if (c->have_basis_e) {  // calculate_orthoMij_E (orthogonalisation_late.c:131-157)
        StageTimer t(c, MODAL_T_MIJ);
        MODAL_TRY(mij_table_dev(c, c->qe.as<double>(), c->lmin_e, c->lmax_e, c->P_e, c->me));
    }
    MODAL_TRY(sync(c));
    c->have_glint = true;
    c->have_gamma = c->have_ortho = c->have_gamma_pol = false;
    return MODAL_OK;
}

modal_status modal_get_mij(modal_ctx *c, double *out)
{
    MODAL_TRY(need(c, c && c->have_glint, "modal_get_mij: call modal_init_glint first"));
    if (!out) { set_error("modal_get_mij: out is NULL"); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    const int P = c->P, nmu = c->nmu;
    // device [nmu][P*P] -> reference Mij_T[P][P][nmu]
    MODAL_TRY(mt_ready(c));
    MODAL_TRY(ensure(c->scratch2, sizeof(double) * (size_t)nmu * P * P));
    MODAL_TRY(transpose_dev(c, c->mt.as<double>(), c->scratch2.as<double>(), nmu, P * P));
    MODAL_TRY(d2h(c, out, c->scratch2.ptr, sizeof(double) * (size_t)nmu * P * P));
    return sync(c);
}

modal_status modal_get_gl(modal_ctx *c, int *nmu, double *nodes, double *weights)
{
    MODAL_TRY(need(c, c && c->have_glint, "modal_get_gl: call modal_init_glint first"));
    MODAL_CUDA(cudaSetDevice(c->device));
    if (nmu) *nmu = c->nmu;
    if (nodes) MODAL_TRY(d2h(c, nodes, c->mu.ptr, sizeof(double) * c->nmu));
    if (weights) MODAL_TRY(d2h(c, weights, c->w.ptr, sizeof(double) * c->nmu));
    return sync(c);
}

modal_status modal_gamma(modal_ctx *c, modal_prec prec, double *gamma)
{
    MODAL_TRY(need(c, c && c->have_modes, "modal_gamma: set basis and modes first"));
    if (prec != MODAL_PREC_FP64 && prec != MODAL_PREC_SPLIT) { set_error("modal_gamma: prec=%d", (int)prec); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    if (!c->have_glint) MODAL_TRY(modal_init_glint(c));
    {
        StageTimer t(c, MODAL_T_GAMMA);
        if (prec == MODAL_PREC_FP64) MODAL_TRY(gamma_fp64_dev(c, 0, c->nmu));
        else MODAL_TRY(gamma_split_dev(c, 0, c->nmu));
    }
    c->have_gamma = true;
    c->have_ortho = false;
    if (gamma) MODAL_TRY(d2h(c, gamma, c->gamma.ptr, sizeof(double) * (size_t)c->N * c->N));
    return sync(c);
}

modal_status modal_gamma_partial(modal_ctx *c, modal_prec prec, int mu_begin, int mu_end, double *gamma)
{
    MODAL_TRY(need(c, c && c->have_modes, "modal_gamma_partial: set basis and modes first"));
    if (prec != MODAL_PREC_FP64 && prec != MODAL_PREC_SPLIT) { set_error("modal_gamma_partial: prec=%d", (int)prec); return MODAL_ERR_ARG; }
    if (!gamma) { set_error("modal_gamma_partial: gamma is NULL"); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    if (!c->have_glint) MODAL_TRY(modal_init_glint(c));
    if (mu_begin < 0 || mu_end > c->nmu || mu_begin >= mu_end) {
        set_error("modal_gamma_partial: node range [%d, %d) outside [0, %d) or empty", mu_begin, mu_end, c->nmu);
        return MODAL_ERR_ARG;
    }
    {
        StageTimer t(c, MODAL_T_GAMMA);
        if (prec == MODAL_PREC_FP64) MODAL_TRY(gamma_fp64_dev(c, mu_begin, mu_end - mu_begin));
        else MODAL_TRY(gamma_split_dev(c, mu_begin, mu_end - mu_begin));
    }
    // the device buffer now holds a partial sum, not Gamma
    c->have_gamma = false;
    c->have_ortho = false;
    MODAL_TRY(d2h(c, gamma, c->gamma.ptr, sizeof(double) * (size_t)c->N * c->N));
    return sync(c);
}

modal_status modal_orthol_pair(modal_ctx *c, int m, int n, double *result)
{
    MODAL_TRY(need(c, c && c->have_modes, "modal_orthol_pair: set basis and modes first"));
    if (!result || m < 0 || n < 0 || m >= c->N || n >= c->N) { set_error("modal_orthol_pair: m=%d n=%d", m, n); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    if (!c->have_gamma) MODAL_TRY(modal_gamma(c, MODAL_PREC_FP64, nullptr));
    MODAL_TRY(d2h(c, result, c->gamma.as<double>() + (size_t)m * c->N + n, sizeof(double)));
    if (c->have_pol) {  // result[1..3] = TTE, TEE, EEE as with do_polarisation
        if (!c->have_gamma_pol) MODAL_TRY(modal_gamma_pol(c, nullptr, nullptr, nullptr));
        const size_t NN = (size_t)c->N * c->N;
        for (int f = 0; f < 3; f++)
            MODAL_TRY(d2h(c, result + 1 + f, c->gamma_pol.as<double>() + f * NN + (size_t)m * c->N + n, sizeof(double)));
    }
    return sync(c);
}

modal_status modal_orthogonalise(modal_ctx *c, const double *gamma, int pca_flag, double *orthol, double *lambdal,
                                 int *branch, int *rank)
{
    MODAL_TRY(need(c, true, ""));
    MODAL_CUDA(cudaSetDevice(c->device));
    if (gamma) {
        if (!c->have_modes) { set_error("modal_orthogonalise: set the modes (N) first"); return MODAL_ERR_STATE; }
        MODAL_TRY(h2d(c, c->gamma, gamma, sizeof(double) * (size_t)c->N * c->N));
        c->have_gamma = true;
    }
    if (!c->have_gamma) { set_error("modal_orthogonalise: no Gamma (pass one or call modal_gamma)"); return MODAL_ERR_STATE; }
    {
        StageTimer t(c, MODAL_T_ORTHO);
        MODAL_TRY(ortho_dev(c, pca_flag));
    }
    size_t NN = (size_t)c->N * c->N;
    if (orthol) MODAL_TRY(d2h(c, orthol, c->orthol.ptr, sizeof(double) * NN));
    if (lambdal) MODAL_TRY(d2h(c, lambdal, c->lambdal.ptr, sizeof(double) * NN));
    MODAL_TRY(sync(c));
    if (branch) *branch = c->ortho_branch;
    if (rank) *rank = c->ortho_rank;
    return MODAL_OK;
}

modal_status modal_set_ortho(modal_ctx *c, const double *orthol, const double *lambdal)
{
    MODAL_TRY(need(c, c && c->have_modes, "modal_set_ortho: set the modes (N) first"));
    if (!orthol || !lambdal) { set_error("modal_set_ortho: orthol and lambdal are required"); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    const size_t NN = (size_t)c->N * c->N;
    c->have_ortho = false;
    MODAL_TRY(h2d(c, c->orthol, orthol, sizeof(double) * NN));
    MODAL_TRY(h2d(c, c->lambdal, lambdal, sizeof(double) * NN));
    MODAL_TRY(lambdainv_dev(c));
    c->ortho_branch = 2;  // caller-supplied: modesR takes the lower triangle
    c->ortho_rank = c->N;
    c->have_ortho = true;
    return sync(c);
}

modal_status modal_set_pca_floor(modal_ctx *c, double floor)
{
    if (!c || !(floor >= 0.0 && floor < 1.0)) { set_error("modal_set_pca_floor: floor must be in [0, 1)"); return MODAL_ERR_ARG; }
    c->pca_floor = floor;
    c->have_ortho = false;
    return MODAL_OK;
}

modal_status modal_set_proj_kernel(modal_ctx *c, int tensor_cores)
{
    if (!c || (tensor_cores != 0 && tensor_cores != 1)) {
        set_error("modal_set_proj_kernel: 0 (CUDA cores) or 1 (tensor cores)");
        return MODAL_ERR_ARG;
    }
    c->proj_tc = tensor_cores;
    return MODAL_OK;
}

modal_status modal_get_proj_kernel(const modal_ctx *c, int *tensor_cores)
{
    if (!c || !tensor_cores) { set_error("modal_get_proj_kernel: NULL argument"); return MODAL_ERR_ARG; }
    *tensor_cores = (c->proj_tc != 0 && c->P <= 32) ? 1 : 0;
    return MODAL_OK;
}

modal_status modal_set_spectrum(modal_ctx *c, const double *cl)
{
    MODAL_TRY(need(c, c && c->have_basis, "modal_set_spectrum: set the basis first"));
    if (!cl) { set_error("modal_set_spectrum: cl is NULL"); return MODAL_ERR_ARG; }
    for (int l = (c->lmin > 2 ? c->lmin : 2); l <= c->lmax; l++)
        if (!(cl[l] > 0.0)) { set_error("modal_set_spectrum: C_l + N_l/b_l^2 must be > 0 (l=%d)", l); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    MODAL_TRY(h2d(c, c->cl, cl, sizeof(double) * (c->lmax + 1)));
    MODAL_TRY(sync(c));
    c->have_spec = true;
    return MODAL_OK;
}

modal_status modal_project(modal_ctx *c, int S, const modal_shape *shapes, modal_prec prec, double *beta)
{
    MODAL_TRY(need(c, c && c->have_modes && c->have_spec, "modal_project: set basis, modes and spectrum first"));
    if (S < 1 || !shapes) { set_error("modal_project: S=%d", S); return MODAL_ERR_ARG; }
    if (c->lmin < 2) { set_error("modal_project: lmin must be >= 2 (w_0 = w_1 = 0)"); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    {
        StageTimer t(c, MODAL_T_PROJECT);
        MODAL_TRY(project_dev(c, S, shapes, prec));
    }
    c->have_beta = true;
    c->beta_S = S;
    if (beta) MODAL_TRY(d2h(c, beta, c->beta.ptr, sizeof(double) * (size_t)S * c->N));
    MODAL_TRY(sync(c));
    return oz_check(c);  // a bounded wait of the tensor-core slab kernel that expired
}

modal_status modal_alpha(modal_ctx *c, int S, const double *beta, double *alpha, double *modesR)
{
    MODAL_TRY(need(c, c && c->have_ortho, "modal_alpha: orthogonalise first"));
    if (S < 1) { set_error("modal_alpha: S=%d", S); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    if (beta) {
        MODAL_TRY(h2d(c, c->beta, beta, sizeof(double) * (size_t)S * c->N));
    } else if (!c->have_beta || c->beta_S != S) {
        set_error("modal_alpha: no device beta for S=%d (pass beta or call modal_project)", S);
        return MODAL_ERR_STATE;
    }
    {
        StageTimer t(c, MODAL_T_ALPHA);
        MODAL_TRY(alpha_dev(c, S));
    }
    if (alpha) MODAL_TRY(d2h(c, alpha, c->alpha.ptr, sizeof(double) * (size_t)S * c->N));
    if (modesR) MODAL_TRY(d2h(c, modesR, c->modesr.ptr, sizeof(double) * (size_t)S * c->N));
    return sync(c);
}

}  // extern "C"
