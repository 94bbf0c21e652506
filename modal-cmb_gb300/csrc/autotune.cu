// autotune.cu -- the library's own launch-configuration tuner.
//
// Two kernels have launch parameters whose best value depends on the problem
// size and the GPU:
//   * the FP32 projection slab kernel: shapes per CTA (8 or 4) and the grid
//     form (one CTA per (slab, shape group), or a persistent grid of 1 or 2
//     CTAs per SM taking work items from a counter);
//   * the FP64 Gamma kernel: mu steps staged per shared-memory load (KC).
// modal_autotune times every candidate with CUDA events on the context stream
// on the context's own basis (a fixed synthetic batch of 16 shapes for the
// projection; the first min(N, 1024) modes for Gamma), keeps the fastest, and
// appends it to a plain-text cache file keyed by GPU architecture and problem
// size, so that later contexts read it back instead of timing again.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "common.cuh"

namespace modal {

__global__ void k_gamma_fp64(int N, int P, int nmu, int KC, const int *triples, const double *mt, const double *wg,
                             double *gamma);
__global__ void k_wgt48(int nmu, const double *w, double *wg);

namespace {

struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    EventPair()
    {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    ~EventPair()
    {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

std::string arch_tag(int device)
{
    int ma = 0, mi = 0;
    cudaDeviceGetAttribute(&ma, cudaDevAttrComputeCapabilityMajor, device);
    cudaDeviceGetAttribute(&mi, cudaDevAttrComputeCapabilityMinor, device);
    return "sm_" + std::to_string(ma) + std::to_string(mi);
}

// Looks `key` up in the cache file; on a hit fills vals[0..n) and returns true.
bool cache_lookup(const char *path, const std::string &key, int *vals, int n)
{
    if (!path) return false;
    FILE *f = std::fopen(path, "r");
    if (!f) return false;
    char line[512];
    bool hit = false;
    while (std::fgets(line, sizeof line, f)) {
        std::string s(line);
        if (s.compare(0, key.size(), key) != 0 || s.size() <= key.size() || s[key.size()] != ' ') continue;
        int got = 0;
        const char *p = line + key.size();
        for (int i = 0; i < n; i++) {
            int v = 0, used = 0;
            if (std::sscanf(p, " %d%n", &v, &used) != 1) break;
            vals[i] = v;
            p += used;
            got++;
        }
        hit = (got == n);  // the last matching line wins
    }
    std::fclose(f);
    return hit;
}

void cache_append(const char *path, const std::string &key, const int *vals, int n, double ms)
{
    if (!path) return;
    FILE *f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%s", key.c_str());
    for (int i = 0; i < n; i++) std::fprintf(f, " %d", vals[i]);
    std::fprintf(f, "  # %.3f ms\n", ms);
    std::fclose(f);
}

// 8 separable (two power-law terms) and 8 bump shapes, deterministic.
void tune_shapes(int lmax, std::vector<double> &tab, std::vector<modal_shape> &sh)
{
    const int S = 16, T = 2;
    tab.assign((size_t)8 * T * 3 * (lmax + 1), 0.0);
    sh.assign(S, modal_shape{});
    for (int s = 0; s < 8; s++) {
        double *t = tab.data() + (size_t)s * T * 3 * (lmax + 1);
        for (int e = 0; e < T * 3; e++) {
            const double ex = -2.0 * ((s * 7 + e * 3) % 11) / 10.0;
            for (int l = 0; l <= lmax; l++) t[(size_t)e * (lmax + 1) + l] = std::pow(l < 1 ? 1.0 : (double)l, ex);
        }
        sh[s].kind = MODAL_SHAPE_SEPARABLE;
        sh[s].nterms = T;
        sh[s].tab = t;
    }
    for (int s = 8; s < S; s++) {
        const double a = 0.2 + 0.05 * (s - 8), b = 0.3 + 0.02 * (s - 8);
        sh[s].kind = MODAL_SHAPE_BUMP;
        sh[s].c[0] = a;
        sh[s].c[1] = b;
        sh[s].c[2] = 1.0 - a - b;
        sh[s].sigma = 0.05 + 0.03 * (s - 8);
    }
}

modal_status time_projection(modal_ctx *c, const std::vector<modal_shape> &sh, float *ms)
{
    EventPair ev;
    MODAL_TRY(project_dev(c, (int)sh.size(), sh.data(), MODAL_PREC_SPLIT));  // warm-up (also plans buffers)
    float best = 1e30f;
    for (int r = 0; r < 2; r++) {
        MODAL_CUDA(cudaEventRecord(ev.a, c->stream));
        MODAL_TRY(project_dev(c, (int)sh.size(), sh.data(), MODAL_PREC_SPLIT));
        MODAL_CUDA(cudaEventRecord(ev.b, c->stream));
        MODAL_CUDA(cudaEventSynchronize(ev.b));
        float t = 0.f;
        MODAL_CUDA(cudaEventElapsedTime(&t, ev.a, ev.b));
        best = std::min(best, t);
    }
    *ms = best;
    return MODAL_OK;
}

}  // namespace

}  // namespace modal

using namespace modal;

extern "C" {

modal_status modal_autotune(modal_ctx *c, const char *cache_path)
{
    if (!c) { set_error("modal_autotune: ctx is NULL"); return MODAL_ERR_ARG; }
    if (!c->have_modes || !c->have_spec) { set_error("modal_autotune: set basis, modes and spectrum first"); return MODAL_ERR_STATE; }
    if (c->lmin < 2) { set_error("modal_autotune: lmin must be >= 2"); return MODAL_ERR_ARG; }
    MODAL_CUDA(cudaSetDevice(c->device));
    const std::string arch = arch_tag(c->device);
    const int P = c->P;

    // ---- projection slab kernel: tensor-core kernel (P <= 32), or the CUDA-core
    // kernel with (shapes per CTA, persistent CTAs per SM)
    const std::string kp = "proj2 " + arch + " lmax=" + std::to_string(c->lmax) + " P=" + std::to_string(P);
    int pv[3] = {0, 0, 0};
    if (cache_lookup(cache_path, kp, pv, 3)) {
        c->proj_sg = pv[0];
        c->proj_cpb = pv[1];
        c->proj_tc = pv[2];
    } else {
        std::vector<double> tab;
        std::vector<modal_shape> sh;
        tune_shapes(c->lmax, tab, sh);
        struct Cand { int sg, cpb, tc; };
        std::vector<Cand> cands;
        if (P <= 32) cands.push_back({0, 0, 1});
        for (int sg : (P <= 32) ? std::vector<int>{8, 4} : std::vector<int>{4})
            for (int cpb : {0, 1, 2}) cands.push_back({sg, cpb, 0});
        float best = 1e30f;
        Cand b = cands[0];
        for (const Cand &cd : cands) {
            c->proj_sg = cd.sg;
            c->proj_cpb = cd.cpb;
            c->proj_tc = cd.tc;
            float ms = 0.f;
            MODAL_TRY(time_projection(c, sh, &ms));
            if (ms < best) { best = ms; b = cd; }
        }
        c->proj_sg = b.sg;
        c->proj_cpb = b.cpb;
        c->proj_tc = b.tc;
        pv[0] = b.sg;
        pv[1] = b.cpb;
        pv[2] = b.tc;
        cache_append(cache_path, kp, pv, 3, best);
    }

    // ---- FP64 Gamma kernel: mu steps per shared-memory stage
    if (!c->have_glint) MODAL_TRY(modal_init_glint(c));
    MODAL_TRY(mt_ready(c));
    const std::string kg = "gamma64 " + arch + " P=" + std::to_string(P) + " nmu=" + std::to_string(c->nmu);
    int gv[1] = {0};
    if (cache_lookup(cache_path, kg, gv, 1)) {
        c->gamma_kc = gv[0];
    } else {
        const int Ns = std::min(c->N, 1024), nmu = c->nmu;
        DevBuf out, wg;
        modal_status st = ensure(out, sizeof(double) * (size_t)Ns * Ns);
        if (st == MODAL_OK) st = ensure(wg, sizeof(double) * nmu);
        float best = 1e30f;
        int bkc = 0;
        if (st == MODAL_OK) {
            k_wgt48<<<ceil_div(nmu, 256), 256, 0, c->stream>>>(nmu, c->w.as<double>(), wg.as<double>());
            st = launched(c, "wgt48");
        }
        EventPair ev;
        for (int kc : {4, 8, 16, 32}) {
            if (st != MODAL_OK) break;
            const size_t smem = sizeof(double) * ((size_t)kc + (size_t)kc * P * P);
            if (smem > 200 * 1024) continue;
            if (cudaFuncSetAttribute(k_gamma_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            const int nt = ceil_div(Ns, 32);
            float t = 1e30f;
            for (int r = 0; r < 3 && st == MODAL_OK; r++) {
                cudaEventRecord(ev.a, c->stream);
                k_gamma_fp64<<<dim3(nt, nt), 256, smem, c->stream>>>(Ns, P, nmu, kc, c->triples.as<int>(),
                                                                     c->mt.as<double>(), wg.as<double>(),
                                                                     out.as<double>());
                st = launched(c, "gamma_fp64");
                cudaEventRecord(ev.b, c->stream);
                if (cudaEventSynchronize(ev.b) != cudaSuccess) { set_error("modal_autotune: gamma timing failed"); st = MODAL_ERR_CUDA; }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev.a, ev.b);
                if (r > 0) t = std::min(t, ms);
            }
            if (st == MODAL_OK && t < best) { best = t; bkc = kc; }
        }
        release(out);
        release(wg);
        MODAL_TRY(st);
        c->gamma_kc = bkc;
        gv[0] = bkc;
        if (bkc > 0) cache_append(cache_path, kg, gv, 1, best);
    }
    return MODAL_OK;
}

modal_status modal_get_tuning(const modal_ctx *c, int *proj_sg, int *proj_cpb, int *gamma_kc)
{
    if (!c) { set_error("modal_get_tuning: ctx is NULL"); return MODAL_ERR_ARG; }
    if (proj_sg) *proj_sg = c->proj_sg;
    if (proj_cpb) *proj_cpb = c->proj_cpb;
    if (gamma_kc) *gamma_kc = c->gamma_kc;
    return MODAL_OK;
}

}  // extern "C"
