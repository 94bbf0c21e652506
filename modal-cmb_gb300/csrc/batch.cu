// batch.cu -- batched shape projection replayed from a captured CUDA graph.
//
// modal_project (calculate_mode_3D's replacement) plans, stages and records a
// projection on every call.  For repeated batches of the same layout (same
// number of shapes, kinds and term counts; new parameter values each time, as
// in a template scan), modal_project_batch captures the recorded device work
// once -- the host-to-device copies of the shape tables and descriptors from
// pinned staging buffers, the slab kernel over all shapes, the reductions and
// the copy of beta back to pinned memory -- and afterwards only refreshes the
// staging buffers and launches the graph: one graph launch per batch.
//
// A captured graph holds device addresses.  Before each replay the addresses
// of every buffer it uses are compared with the context's current ones; any
// change (a buffer grown by another call, a new basis size) re-plans and
// re-captures.
#include <cstring>
#include <vector>
#include "common.cuh"

namespace modal {

struct BatchGraph {
    // layout key
    int S = 0, prec = -1, lmin = -1, lmax = -1, P = -1, N = -1, sg = -1, cpb = -1, tc = -1;
    std::vector<int> kinds, nterms;
    std::vector<const void *> ptrs;
    // graph and pinned staging
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    double *h_tab = nullptr;
    DShape *h_desc = nullptr;
    double *h_beta = nullptr;
    ProjPlan plan;
    long kernels = 0;  // kernel nodes per replay
    void clear()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (h_tab) cudaFreeHost(h_tab);
        if (h_desc) cudaFreeHost(h_desc);
        if (h_beta) cudaFreeHost(h_beta);
        *this = BatchGraph();
    }
};

void batch_release(modal_ctx *c)
{
    if (c && c->batch) {
        c->batch->clear();
        delete c->batch;
        c->batch = nullptr;
    }
}

static std::vector<const void *> batch_ptrs(const modal_ctx *c)
{
    return {c->q.ptr, c->cl.ptr, c->vl.ptr, c->triples.ptr, c->slab_order.ptr, c->shape_tab.ptr, c->shape_desc.ptr,
            c->scratch.ptr, c->beta.ptr};
}

static bool batch_matches(const BatchGraph &g, const modal_ctx *c, int S, const modal_shape *shapes, modal_prec prec)
{
    if (!g.exec || g.S != S || g.prec != (int)prec || g.lmin != c->lmin || g.lmax != c->lmax || g.P != c->P ||
        g.N != c->N || g.sg != c->proj_sg || g.cpb != c->proj_cpb || g.tc != c->proj_tc)
        return false;
    for (int s = 0; s < S; s++)
        if (g.kinds[s] != shapes[s].kind || (shapes[s].kind == MODAL_SHAPE_SEPARABLE && g.nterms[s] != shapes[s].nterms))
            return false;
    return g.ptrs == batch_ptrs(c);
}

// Plan, stage pinned buffers and capture the device work of one batch layout.
static modal_status batch_capture(modal_ctx *c, int S, const modal_shape *shapes, modal_prec prec)
{
    if (!c->batch) c->batch = new BatchGraph();
    BatchGraph &g = *c->batch;
    g.clear();
    MODAL_TRY(proj_plan(c, S, shapes, prec, g.plan));
    const size_t tab_bytes = sizeof(double) * (size_t)(g.plan.tab_total > 0 ? g.plan.tab_total : 1);
    MODAL_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&g.h_tab), tab_bytes, cudaHostAllocDefault));
    MODAL_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&g.h_desc), sizeof(DShape) * (size_t)S, cudaHostAllocDefault));
    MODAL_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&g.h_beta), sizeof(double) * (size_t)S * c->N,
                             cudaHostAllocDefault));
    MODAL_CUDA(cudaStreamSynchronize(c->stream));  // the plan's uploads are done before capture starts
    const long l0 = c->launches;
    MODAL_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    modal_status st = MODAL_OK;
    cudaError_t e = cudaMemcpyAsync(c->shape_tab.ptr, g.h_tab, tab_bytes, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->shape_desc.ptr, g.h_desc, sizeof(DShape) * S, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) {
        set_error("modal_project_batch: staging copy in capture: %s", cudaGetErrorString(e));
        st = MODAL_ERR_CUDA;
    }
    if (st == MODAL_OK) st = proj_record(c, g.plan);
    if (st == MODAL_OK) {
        e = cudaMemcpyAsync(g.h_beta, c->beta.ptr, sizeof(double) * (size_t)S * c->N, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) {
            set_error("modal_project_batch: result copy in capture: %s", cudaGetErrorString(e));
            st = MODAL_ERR_CUDA;
        }
    }
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(c->stream, &graph);  // always ends the capture, even after a failure
    g.kernels = c->launches - l0;
    c->launches = l0;
    if (st != MODAL_OK) {
        if (graph) cudaGraphDestroy(graph);
        g.clear();
        return st;
    }
    if (e != cudaSuccess || !graph) {
        set_error("modal_project_batch: capture failed: %s", cudaGetErrorString(e));
        g.clear();
        return MODAL_ERR_CUDA;
    }
    g.graph = graph;
    e = cudaGraphInstantiate(&g.exec, graph, 0);
    if (e != cudaSuccess) {
        set_error("modal_project_batch: graph instantiation: %s", cudaGetErrorString(e));
        g.clear();
        return MODAL_ERR_CUDA;
    }
    g.S = S;
    g.prec = (int)prec;
    g.lmin = c->lmin;
    g.lmax = c->lmax;
    g.P = c->P;
    g.N = c->N;
    g.sg = c->proj_sg;
    g.cpb = c->proj_cpb;
    g.tc = c->proj_tc;
    g.kinds.resize(S);
    g.nterms.resize(S);
    for (int s = 0; s < S; s++) {
        g.kinds[s] = shapes[s].kind;
        g.nterms[s] = shapes[s].nterms;
    }
    g.ptrs = batch_ptrs(c);
    c->captures++;
    return MODAL_OK;
}

}  // namespace modal

using namespace modal;

extern "C" {

modal_status modal_project_batch(modal_ctx *c, int S, const modal_shape *shapes, modal_prec prec, double *beta)
{
    if (!c || S < 1 || !shapes || !beta) { set_error("modal_project_batch: bad arguments (S=%d)", S); return MODAL_ERR_ARG; }
    if (!c->have_modes || !c->have_spec) { set_error("modal_project_batch: set basis, modes and spectrum first"); return MODAL_ERR_STATE; }
    if (c->lmin < 2) { set_error("modal_project_batch: lmin must be >= 2 (w_0 = w_1 = 0)"); return MODAL_ERR_ARG; }
    if (prec != MODAL_PREC_FP64 && prec != MODAL_PREC_SPLIT) { set_error("modal_project_batch: prec=%d", (int)prec); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    for (int s = 0; s < S; s++) {  // same validation as the planned path
        const modal_shape &m = shapes[s];
        if (m.kind == MODAL_SHAPE_SEPARABLE ? (m.nterms < 1 || !m.tab)
                                            : (m.kind != MODAL_SHAPE_BUMP || !(m.sigma > 0.0))) {
            set_error("shape %d: invalid (kind %d, nterms %d, sigma %g)", s, m.kind, m.nterms, m.sigma);
            return MODAL_ERR_ARG;
        }
    }
    if (!c->batch || !batch_matches(*c->batch, c, S, shapes, prec)) MODAL_TRY(batch_capture(c, S, shapes, prec));
    BatchGraph &g = *c->batch;
    // refresh the pinned staging buffers with this batch's values
    const int stride = c->lmax + 1;
    for (int s = 0; s < S; s++) {
        const modal_shape &m = shapes[s];
        DShape d = g.plan.desc[s];
        d.c1 = m.c[0];
        d.c2 = m.c[1];
        d.c3 = m.c[2];
        d.sigma = m.sigma;
        g.h_desc[s] = d;
        if (m.kind == MODAL_SHAPE_SEPARABLE)
            std::memcpy(g.h_tab + d.tab_off, m.tab, sizeof(double) * (size_t)m.nterms * 3 * stride);
    }
    {
        StageTimer t(c, MODAL_T_PROJECT);
        MODAL_CUDA(cudaGraphLaunch(g.exec, c->stream));
    }
    c->launches += g.kernels;
    MODAL_CUDA(cudaStreamSynchronize(c->stream));
    MODAL_TRY(oz_check(c));  // a bounded wait of the tensor-core slab kernel that expired
    std::memcpy(beta, g.h_beta, sizeof(double) * (size_t)S * c->N);
    c->have_beta = true;  // beta also stays on the device for modal_alpha
    c->beta_S = S;
    return MODAL_OK;
}

long modal_ctx_captures(const modal_ctx *c) { return c ? c->captures : 0; }

}  // extern "C"
