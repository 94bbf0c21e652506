#!/usr/bin/env python
"""Benchmark: Modal-CMB mode-space hot path on GB300.

One step = one pass of the hot path over the synthetic workload at
l_max = 2000, 30 shifted-Legendre basis functions (4960 modes), n_mu = 3001,
16 seeded separable shapes:
  GL nodes + P_l(mu) table + l-contraction, Gamma (mu-contraction),
  orthogonalisation, projection of the shapes, alpha solve.
`value` = device seconds of "Gamma + ortho" per step (the first quantity of
the metric), with inputs resident in HBM and L2 flushed between steps;
`projections_per_s` is the second quantity.  `e2e` is the same quantity
measured through the C ABI with host buffers (copies inside the timed region).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's CPU path (the in-place build of its own
sources when present, else the C restatement in oracle/) on the host cores,
on bounded samples of the same workload, extrapolated per unit.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "modal-cmb_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

METRIC = "Gamma+ortho s and shape projections/s, split-prec vs FP64, GB300, rel err<=1e-6"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FP64_NOMINAL_TFLOPS = 1.25  # GB300 dense FP64 (nominal; no measured FP64 peak is available)
# DRAM bytes (read + write) of the tridiagonalisation's panel kernels in one
# eigen-decomposition at l <= 2000, P = 30 (N = 4960): an ncu capture of the 155
# panel launches of one eigen-decomposition (dram__bytes_read.sum 8.4596e10 +
# dram__bytes_write.sum 4.07e8), not measured by this run.
NCU_PANEL_TRAFFIC_CFG2 = 8.4596e10 + 4.07e8


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="cfg2")
    ap.add_argument("--prec", choices=["auto", "fp64", "split"], default="auto")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    # only the warm-up and timed steps, one short line (for profiler launch lists)
    ap.add_argument("--step-only", action="store_true")
    a = ap.parse_args()
    a.warmup = max(3, a.warmup)
    return a


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    try:
        with open(PEAKS_FILE) as f:
            p = json.load(f)
        return p, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# ------------------------------------------------------------------- clocks

class Clocks:
    """nvidia-smi sampler running while the timed region runs."""

    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        load = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# -------------------------------------------------------------- our GPU arm

def max_over_ranks(vals, ws, device="cpu"):
    """Element-wise maximum of per-rank timings after a barrier (replicas: the
    job takes as long as its slowest rank); the identity for one rank."""
    if ws <= 1:
        return [float(v) for v in vals]
    import torch
    import torch.distributed as td
    t = torch.tensor([float(v) for v in vals], dtype=torch.float64, device=device)
    td.barrier()
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return t.tolist()


def run_ours(a, ws, rank, local):
    import torch
    import modal_gb300 as mg

    cfgd = mg.CONFIGS[a.config]
    lmax, P = cfgd["lmax"], cfgd["P"]
    q, tr, cl = mg.workload(lmax, P)
    shapes = mg.config_shapes(lmax, cfgd["shapes"], seed=rank)
    S, N = len(shapes), len(tr)
    nmu = 3 * lmax // 2 + 1
    torch.cuda.set_device(local)
    ctx = mg.Context(local)
    ctx.set_basis(2, lmax, q)
    ctx.set_modes(tr)
    ctx.set_spectrum(cl)
    ctx.profile(True)
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    # the library's own launch-configuration tuner, before any timing (cached per machine)
    tuning = ctx.autotune(os.path.join(tempfile.gettempdir(), f"modal_gb300_tune_{local}.txt"))

    split_ok = True
    try:
        ctx.init_glint()
        ctx.gamma(mg.PREC_SPLIT, download=False)
    except mg.ModalError:
        split_ok = False
    prec = {"auto": mg.PREC_SPLIT if split_ok else mg.PREC_FP64, "fp64": mg.PREC_FP64, "split": mg.PREC_SPLIT}[a.prec]

    # the comparison pass in the other precision projects at most 16 shapes
    # (FP64 projection of 512 shapes at l <= 2500 would take minutes); its
    # projection time is scaled to S shapes
    S_cmp = min(S, 16)
    shapes_cmp = shapes[:S_cmp]

    def step(pr, sh=None):
        sh = shapes if sh is None else sh
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        e[0].record(stream)
        ctx.init_glint()
        ctx.gamma(pr, download=False)
        ctx.orthogonalise(None, download=False)
        e[1].record(stream)
        ctx.project(sh, pr, download=False)
        e[2].record(stream)
        ctx.alpha(len(sh), download=False)
        e[3].record(stream)
        return e

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    def run(pr, steps, warm, sh=None):
        for _ in range(warm):
            step(pr, sh)
            flush.zero_()
            torch.cuda.synchronize()
        ctx.timer_reset()
        times = []
        launches0 = ctx.launches
        barrier()
        torch.cuda.synchronize()
        clk = Clocks(local) if pr == prec else None
        t0 = time.perf_counter()
        for _ in range(steps):
            ev = step(pr, sh)
            torch.cuda.synchronize()
            times.append([ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2]), ev[2].elapsed_time(ev[3])])
            flush.zero_()  # L2 flush between steps (outside the events)
            torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        clocks = clk.stop() if clk else None
        barrier()
        launches = ctx.launches - launches0
        tm = {k: ctx.timer(k) for k in ("gl", "pl", "mij", "gamma", "lift", "tc", "ortho", "eig_trd", "eig_panel",
                                        "eig_dc", "eig_back", "project", "alpha")}
        return np.array(times), wall, launches, tm, clocks

    times, wall, launches, tm, clocks = run(prec, a.steps, a.warmup)
    go_ms = float(np.median(times[:, 0]))
    proj_ms = float(np.median(times[:, 1]))
    step_ms = float(np.median(times.sum(axis=1)))
    go_ms, proj_ms, step_ms = max_over_ranks([go_ms, proj_ms, step_ms], ws, f"cuda:{local}")
    stages = {k: {"ms": v[0] / a.steps, "launches": v[1] / a.steps} for k, v in tm.items()}
    if a.step_only:
        ctx.close()
        return {"metric": METRIC, "value": go_ms * 1e-3, "unit": "s", "mode": "step-only", "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": step_ms, "config": {"workload": a.config},
                "gpu_launches": int(launches), "stage_ms_per_step": stages}

    # the other precision, for the split-vs-FP64 ratio and the error against FP64
    extra = {}
    ctx.init_glint()
    ctx.gamma(mg.PREC_FP64, download=False)
    G64 = ctx.gamma(mg.PREC_FP64)
    ctx.orthogonalise(None, download=False)
    b64 = ctx.project(shapes_cmp, mg.PREC_FP64)
    a64, m64 = ctx.alpha(S_cmp)
    if split_ok:
        other = mg.PREC_FP64 if prec == mg.PREC_SPLIT else mg.PREC_SPLIT
        t2, _, _, tm2, _ = run(other, max(1, min(a.steps, 2)), 1 if other == mg.PREC_FP64 else 3, shapes_cmp)
        t2 = t2.copy()
        t2[:, 1] *= S / S_cmp  # projection time scaled to the S shapes of the timed steps
        Gs = ctx.gamma(mg.PREC_SPLIT)
        ctx.orthogonalise(None, download=False)
        bs = ctx.project(shapes_cmp, mg.PREC_SPLIT)
        as_, ms_ = ctx.alpha(S_cmp)
        fp = t2 if other == mg.PREC_FP64 else times
        sp = times if other == mg.PREC_FP64 else t2
        d = as_ - a64
        gnorm = lambda v: np.sqrt(np.abs(np.einsum("si,ij,sj->s", v, G64, v)))  # noqa: E731
        extra = {
            "comparison_shapes": S_cmp,
            "fp64_gamma_ortho_ms": float(np.median(fp[:, 0])), "split_gamma_ortho_ms": float(np.median(sp[:, 0])),
            "fp64_projection_ms": float(np.median(fp[:, 1])), "split_projection_ms": float(np.median(sp[:, 1])),
            "split_vs_fp64_gamma_ortho_projection": float(np.median(fp[:, :2].sum(1)) / np.median(sp[:, :2].sum(1))),
            "rel_err_vs_fp64": {
                "gamma_fro": float(np.linalg.norm(Gs - G64) / np.linalg.norm(G64)),
                "beta_fro": float(np.linalg.norm(bs - b64) / np.linalg.norm(b64)),
                "alpha_gamma_norm": float(np.max(gnorm(d) / np.maximum(gnorm(a64), 1e-300))),
                "modesR_fro": float(np.linalg.norm(ms_ - m64) / np.linalg.norm(m64)),
            },
        }
        # alpha with a PCA eigenvalue floor above the split form's Gamma error:
        # the same FP64 orthogonalisation of each Gamma, keeping eigenvalues > floor * e_max
        fl = {}
        probes = np.random.default_rng(7).standard_normal((4, N))
        for floor in (1e-6, 1e-4):
            ctx.set_pca_floor(floor)
            _, lam64, _, r64 = ctx.orthogonalise(G64)
            af64, _ = ctx.alpha(S_cmp, b64)
            _, lams, _, rs = ctx.orthogonalise(Gs)
            afs, _ = ctx.alpha(S_cmp, bs)
            # the kept-subspace operator lambda^T lambda (orthoinv) on random probes
            p64, ps = lam64.T @ (lam64 @ probes.T), lams.T @ (lams @ probes.T)
            fl["%g" % floor] = {"kept_fp64": r64, "kept_split": rs,
                                "alpha_fro": float(np.linalg.norm(afs - af64) / np.linalg.norm(af64)),
                                "alpha_gamma_norm": float(np.max(gnorm(afs - af64) / gnorm(af64))),
                                "orthoinv_probe_fro": float(np.linalg.norm(ps - p64) / np.linalg.norm(p64))}
            del lam64, lams
        ctx.set_pca_floor(0.0)
        extra["rel_err_vs_fp64"]["alpha_with_pca_floor"] = fl

    # the 256-shape batch at this size (128 separable sums of 1-4 terms + 128
    # Gaussian bumps), split form, through the graph-captured batch path (one
    # graph launch: staging copies, all shapes' slab work, reductions, beta
    # back to the host); the FP64 form is scaled from the timed shapes
    if split_ok and a.config in ("cfg2", "cfg3"):
        sh256 = mg.config_shapes(lmax, ("mix", 256, 1, 4), seed=rank)
        b_ref = ctx.project(sh256, mg.PREC_SPLIT)
        for _ in range(2):
            b256 = ctx.project_batch(sh256, mg.PREC_SPLIT)
        assert np.array_equal(b256, b_ref)
        torch.cuda.synchronize()
        p_ms = []
        for _ in range(3):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.project_batch(sh256, mg.PREC_SPLIT)
            e1.record(stream)
            torch.cuda.synchronize()
            p_ms.append(e0.elapsed_time(e1))
        p256 = float(np.median(p_ms))
        # the FP64 form of the same 256 shapes, timed once (device time on the context stream)
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b256_64 = ctx.project(sh256, mg.PREC_FP64)
        e1.record(stream)
        torch.cuda.synchronize()
        fp64_256 = e0.elapsed_time(e1)
        beta256_err = float(np.max(np.linalg.norm(b256 - b256_64, axis=1) / np.linalg.norm(b256_64, axis=1)))
        # the same batch with the slab contraction on the tensor cores (P <= 32)
        tc256 = None
        if P <= 32:
            tuned_tc = ctx.proj_kernel()
            ctx.set_proj_kernel(True)
            btc = ctx.project_batch(sh256, mg.PREC_SPLIT)
            t_tc = []
            for _ in range(2):
                flush.zero_()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                ctx.project_batch(sh256, mg.PREC_SPLIT)
                e1.record(stream)
                torch.cuda.synchronize()
                t_tc.append(e0.elapsed_time(e1))
            ctx.set_proj_kernel(tuned_tc)
            tc256 = {"ms": float(min(t_tc)), "beta_max_rel_err_vs_fp64": float(np.max(
                np.linalg.norm(btc - b256_64, axis=1) / np.linalg.norm(b256_64, axis=1))),
                     "kernel": "k_project_slab_tc (tcgen05, BF16 three-piece operands)"}
        go64 = extra.get("fp64_gamma_ortho_ms", go_ms)
        gos = extra.get("split_gamma_ortho_ms", go_ms)
        extra["projection_256_shapes"] = {
            "path": "modal_project_batch (captured CUDA graph, %d captures)" % ctx.captures,
            "split_ms": p256, "split_projections_per_s": 256.0 / (p256 * 1e-3),
            "fp64_ms": fp64_256, "split_beta_max_rel_err_vs_fp64": beta256_err,
            "split_vs_fp64_gamma_ortho_plus_256_projections": (go64 + fp64_256) / (gos + p256),
            "kernel": "k_project_slab_tc" if ctx.proj_kernel() else "k_project_slab_f32 (CUDA cores)",
            "tensor_core_form": tc256}

    # roofline of the dominant kernel of the timed step: the tridiagonalisation's
    # panel kernel (the FP64 matrix-vector product over the trailing matrix of
    # every column).  achieved = algorithmic bytes of one eigen-decomposition,
    # 8 * sum_{m=1}^{N-1} m^2 (the trailing matrix read once per column), / the
    # panel kernels' device time per eigen-decomposition (CUDA events).
    pk, pk_kind = peaks()
    flops = 18.0 * N * (N + 1) / 2.0 * nmu
    hbm = pk.get("hbm_gbs", 6800.0)
    p_ms, p_n = tm["eig_panel"]
    o_ms, o_n = tm["ortho"]
    roof = None
    if p_n > 0 and o_n > 0:
        t_ms = p_ms / o_n  # panel kernels per orthogonalisation
        alg_bytes = 8.0 * (N - 1) * N * (2 * N - 1) / 6.0
        achieved = alg_bytes / (t_ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": NCU_PANEL_TRAFFIC_CFG2 if a.config == "cfg2" else None,
                "traffic_source": "ncu capture of the panel kernels at this config, not this run",
                "kernel": "k_trd_panel (%d launches per eigen-decomposition)" % round(p_n / o_n), "kernel_ms": t_ms,
                "peak_kind": pk_kind + " HBM copy bandwidth",
                "algorithmic": "8 sum_{m<N} m^2 bytes per eigen-decomposition (trailing matrix read per column)",
                "note": "the product also runs at the FP64 rate: 2 sum m^2 flop = %.1f TFLOP/s of the nominal %.2f"
                        % (2.0 * alg_bytes / 8.0 / (t_ms * 1e-3) / 1e12, FP64_NOMINAL_TFLOPS)}
    # the mu-contraction on the tensor cores (split form): algorithmic and executed rates
    l_ms, l_n = tm["lift"]
    mu_contraction = None
    if prec == mg.PREC_SPLIT and l_n > 0:
        t_ms = l_ms / l_n
        U = P * (P + 1) // 2
        UV = U * (U + 1) // 2
        v_of = np.repeat(np.arange(U), np.arange(U, 0, -1))
        ntiles = 0
        for j in range((UV + 127) // 128):
            ntiles += min(v_of[min(UV, (j + 1) * 128) - 1] // 128 + 1, (U + 127) // 128)
        kpad = -(-nmu // 64) * 64
        executed = 2.0 * 28 * 128 * 128 * kpad * ntiles  # 7 slices: 28 digit products per tile
        peak = pk.get("bf16_tflops", 1900.0)
        mu_contraction = {"kernel": "k_oz_gemm (mu-contraction, 7 exact 7-bit slices)", "kernel_ms": t_ms,
                          "algorithmic_tflops": flops / (t_ms * 1e-3) / 1e12,
                          "executed_tensor_tflops": executed / (t_ms * 1e-3) / 1e12,
                          "executed_frac": executed / (t_ms * 1e-3) / 1e12 / peak, "peak": peak,
                          "peak_kind": pk_kind + " bf16 burst (FP16 dense rate is equal)",
                          "algorithmic": "18 N(N+1)/2 n_mu flop per launch"}

    # end to end through the C ABI with host buffers
    e2e = run_e2e(ctx, mg, q, tr, cl, shapes, prec, a.steps)
    cpu = None
    if rank == 0 and not a.no_cpu_baseline:
        cpu = cpu_baseline(a.config, lmax, P, q, tr, cl, shapes, gamma=G64)
    ctx.close()
    extras = run_extras(mg, local) if rank == 0 and a.config == "cfg2" else None
    next_rows = run_next_rows(mg, local, not a.no_cpu_baseline) if rank == 0 and a.config == "cfg2" else None
    line = {
        "metric": METRIC, "value": go_ms * 1e-3, "unit": "s", "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": step_ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == mg.PREC_FP64 else ("f64 orthogonalisation; Gamma on f16 tensor cores with exact 7-bit "
                                                     "integer slices (f32 tensor-memory sums exact, double-f32 across "
                                                     "node blocks), f64 gather"),
        "data": "synthetic (seeded shapes; synthetic C_l; shifted Legendre basis)",
        "config": {"workload": f"{a.config}: l=2..{lmax}, P={P}, N={N}, n_mu={nmu}, S={S} shapes",
                   "l2": "flushed (256 MB write between steps)", "parallelism": f"replicas x{ws}",
                   "precision": "fp64" if prec == mg.PREC_FP64 else "split"},
        "projections_per_s": S * ws / (proj_ms * 1e-3),
        "tuning": tuning,
        "extras": extras,
        "next_rows": next_rows,
        "stage_ms_per_step": stages,
        "roofline": roof,
        "mu_contraction": mu_contraction,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    line.update(extra)
    return line


def run_extras(mg, local):
    """The rows next to the path at the basis-optimisation size (lmax 1000, 12 functions
    of 64 cubic B-splines = 364 modes, n_mu 1501, 32 shapes): one objective + gradient
    (modal_adjoint_residual) and the full greedy pruning (modal_basis_prune), device
    time with CUDA events on the context stream."""
    import torch
    C, Bw, tri, cl = mg.bspline_workload(1000, 12, 64, seed=4)
    shapes = mg.separable_shapes(1000, 32, 40, 1, 2)
    out = {"workload": "lmax 1000, 64 B-splines x 12 functions, N=364, n_mu=1501, 32 shapes"}
    with mg.Context(local) as c:
        c.set_basis(2, 1000, Bw @ C.T)
        c.set_modes(tri)
        c.set_spectrum(cl)
        c.init_glint()
        c.gamma(mg.PREC_FP64, download=False)
        c.orthogonalise(None, download=False)
        stream = torch.cuda.ExternalStream(c.stream)
        c.adjoint_residual(shapes)  # warm-up
        ts = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            J, _ = c.adjoint_residual(shapes)
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        out["adjoint_residual_ms"] = float(np.median(ts))
        out["objective_J"] = J
        t0 = time.perf_counter()
        order, lam = c.basis_prune()
        out["basis_prune_364_s"] = time.perf_counter() - t0
    return out


def _dev_ms(c, fn, reps=3):
    """Median device time of fn() on the context stream (CUDA events), after one warm-up."""
    import torch
    stream = torch.cuda.ExternalStream(c.stream)
    fn()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def _fit_cpu(fn, n1, n2, N, power):
    """CPU time at size N from timings at n1 < n2, modelled as a + b n^power (a:
    the work that does not grow with the sample, such as tables or the grid walk)."""
    t = []
    for n in (n1, n2):
        t0 = time.perf_counter()
        fn(n)
        t.append(time.perf_counter() - t0)
    b = max(0.0, (t[1] - t[0]) / (n2 ** power - n1 ** power))
    a = max(0.0, t[0] - b * n1 ** power)
    return a + b * N ** power


def run_next_rows(mg, local, with_cpu):
    """The rows next to the hot path, each on one synthetic workload: device time
    through the C ABI and, with the CPU baseline, the CPU restatement of the
    reference's routine timed on a bounded sample of the same workload and scaled
    by that routine's cost law (stated per row).  The CPU restatement's OpenMP
    routines use every host core."""
    out = {}
    orc = None
    if with_cpu:
        import oracle
        orc = oracle.Oracle()
    cores = os.cpu_count() or 1

    # polarised Gamma: calculate_orthol results[1..3] (orthogonalisation_late.c:239-336)
    lmax, P = 1000, 16
    cl, qT, qE, ttt, tte, tee, eee = mg.pol_workload(lmax, lmax, 2, P, P)
    N = len(ttt)
    with mg.Context(local) as c:
        c.set_basis(2, lmax, qT)
        c.set_modes(ttt)
        c.set_basis_e(2, lmax, qE)
        c.set_modes_pol(tte, tee, eee)
        c.init_glint()
        row = {"workload": f"TTE+TEE+EEE Gamma, T and E on l=2..{lmax}, P_T=P_E={P}, N={N}",
               "gpu_ms": _dev_ms(c, c.gamma_pol)}
        x, w = c.get_gl()
    if orc is not None:
        pl = orc.legendre_table(x, lmax)
        MT, ME = orc.mij(pl, 2, lmax, qT), orc.mij(pl, 2, lmax, qE)
        row["cpu_s"] = _fit_cpu(lambda n: orc.gamma_pol(MT, ME, w, tte[:n], tee[:n], eee[:n]), 192, 384, N, 2)
        row["cpu_sample"] = f"192 and 384 of {N} modes of each family, fitted as a + b n^2; cores {cores}"
    out["polarised_gamma"] = row

    # late x primordial transfer Gamma: calculate_gamma_2d over all (m, n) (calculate_gamma.c:773-934)
    lmax, P, Pp, xsize = 600, 16, 8, 32
    q, tr, cl = mg.workload(lmax, P)
    xvec, qt = mg.transfer_workload(lmax, Pp, xsize)
    prim = mg.mode_triples(Pp)
    N, Np = len(tr), len(prim)
    with mg.Context(local) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        c.init_glint()
        c.set_transfer(xvec, qt, prim)
        row = {"workload": f"transfer Gamma, l=2..{lmax}, P={P} (N={N}), P_prim={Pp} (N_prim={Np}), {xsize} x points",
               "gpu_ms": _dev_ms(c, lambda: c.gamma_transfer(0.7))}
        x, w = c.get_gl()
    if orc is not None:
        row["cpu_s"] = _fit_cpu(lambda n: orc.gamma_transfer(2, lmax, q, tr[:n], cl, x, w, xvec, qt, prim, 0.7),
                                16, 64, N, 1)
        row["cpu_sample"] = f"16 and 64 of {N} late modes (rows), fitted as a + b n (a: the per-x M tables); cores {cores}"
    out["transfer_gamma"] = row

    # 3D transfer Gamma: calculate_gamma_TTT_3D_nested (calculate_gamma_3d.c:274-440)
    lmax, P, Pp, xsize = 300, 12, 8, 32
    q, tr, cl = mg.workload(lmax, P)
    xvec, qt = mg.transfer_workload(lmax, Pp, xsize)
    prim = mg.mode_triples(Pp)
    N, Np = len(tr), len(prim)
    with mg.Context(local) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        c.set_transfer(xvec, qt, prim)
        row = {"workload": f"3D transfer Gamma, l=2..{lmax}, P={P} (N={N}), P_prim={Pp} (N_prim={Np}), {xsize} x points",
               "gpu_ms": _dev_ms(c, lambda: c.gamma_transfer_3d(0.7))}
    if orc is not None:
        row["cpu_s"] = _fit_cpu(lambda n: orc.gamma_3d(2, lmax, q, tr, cl, xvec, qt, prim[:n], 0.7), 8, 32, Np, 1)
        row["cpu_sample"] = f"8 and 32 of {Np} primordial modes, fitted as a + b n; cores {cores}"
    out["transfer_gamma_3d"] = row

    # primordial k-space side: calculate_ortho (orthogonalisation.c:14-86) and calculate_eigen
    kmin, kmax_i, kmax, Pp = 1, 120, 0.5, 12
    basis, prim, shapes = mg.prim_workload(kmax_i, Pp)
    N = len(prim)
    npts = len(mg.prim_points(kmin, kmax_i))
    with mg.Context(local) as c:
        row = {"workload": f"k-grid Gram matrix and 2 shape projections, grid 1..{kmax_i} ({npts} points), P={Pp}, N={N}",
               "gpu_ms_ortho": _dev_ms(c, lambda: c.prim_ortho(kmin, kmax_i, kmax, basis, prim)),
               "gpu_ms_eigen": _dev_ms(c, lambda: c.prim_eigen(kmin, kmax_i, kmax, basis, prim, shapes))}
    if orc is not None:
        row["cpu_s_ortho"] = _fit_cpu(lambda n: orc.prim_ortho(kmin, kmax_i, kmax, basis, prim[:n]), 48, 96, N, 2)
        row["cpu_s_eigen"] = _fit_cpu(lambda n: [orc.prim_eigen(kmin, kmax_i, kmax, basis, prim[:n], sh) for sh in shapes],
                                      12, 48, N, 1)
        row["cpu_sample"] = (f"48 and 96 of {N} modes for the Gram matrix (a + b n^2), 12 and 48 for the "
                             "projections (a + b n); 1 core")
    out["primordial"] = row
    return out


def run_e2e(ctx, mg, q, tr, cl, shapes, prec, steps):
    """Gamma + ortho through the public C ABI from host inputs to host outputs
    (inputs and outputs in pinned host memory)."""
    import torch
    ts = []
    N = len(tr)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    qp, trp = pin(q), pin(tr.astype(np.int32))
    G, o, lam = (torch.empty((N, N), dtype=torch.float64).pin_memory().numpy() for _ in range(3))
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        ctx.set_basis(2, q.shape[0] + 1, qp)
        ctx.set_modes(trp)
        ctx.init_glint()
        ctx.gamma(prec, out=G)
        ctx.orthogonalise(None, out=(o, lam))
        ts.append(time.perf_counter() - t0)
    ctx.set_spectrum(cl)
    h2d = q.nbytes + tr.astype(np.int32).nbytes
    d2h = G.nbytes + o.nbytes + lam.nbytes
    return {"value": float(np.median(ts)), "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "what": "set_basis/set_modes (H2D) + init_glint + gamma (D2H Gamma) + orthogonalise (D2H orthol, lambdal); "
                    "pinned host buffers",
            "N": N}


# -------------------------------------------------------- CPU reference arm

_GAMMA_CACHE = {}


def cpu_baseline(config, lmax, P, q, tr, cl, shapes, gamma=None):
    """Reference CPU path on the host cores: Gamma (P_l table + l-contraction in
    full, calculate_orthol over a sample of pairs, extrapolated per pair), the
    orthogonalisation of the actual normalised Gamma at full size (the
    reference's gsl_eigen_symmv + PCA outputs, ortho_late_mpi.c:759-805, with
    LAPACK through numpy standing in for GSL), and the projection
    (calculate_mode_3D over a sample of tetrapyd points per thread).  gamma:
    the FP64 Gamma when the caller has it; otherwise it is computed once per
    process by the CPU restatement (setup, not timed)."""
    import oracle
    cores = os.cpu_count() or 1
    ref = None
    kind = "port"
    try:
        if os.path.exists(oracle.REF_SO):
            ref = oracle.Ref()
            kind = "reference"
    except Exception:
        ref = None
    orc = oracle.Oracle()
    N = len(tr)
    nmu = 3 * lmax // 2 + 1
    total_pairs = N * (N + 1) // 2
    npairs = min(total_pairs, 400000)
    if ref is not None:
        # the reference's own init_orthol_glint + calculate_orthoMij_T and calculate_orthol loop
        ref.setup(2, lmax, q, tr, cl)
        t0 = time.perf_counter()
        with oracle.quiet_stdout():
            ref.init_gamma()
        t_init = time.perf_counter() - t0
        t0 = time.perf_counter()
        ref.gamma(nranks=cores, npairs=npairs)
        t_pairs = time.perf_counter() - t0
        x = w = M = None
    else:
        t0 = time.perf_counter()
        x, w = orc.gl_nodes(nmu)
        pl = orc.legendre_table(x, lmax)
        M = orc.mij(pl, 2, lmax, q)
        t_init = time.perf_counter() - t0
        t0 = time.perf_counter()
        orc.gamma_sample(M, w, tr, npairs, nthreads=cores)
        t_pairs = time.perf_counter() - t0
    t_gamma = t_init + t_pairs * total_pairs / npairs
    # orthogonalisation of the actual normalised Gamma, full size
    if gamma is None:
        key = (lmax, P, N)
        if key not in _GAMMA_CACHE:
            if M is None:
                x, w = orc.gl_nodes(nmu)
                M = orc.mij(orc.legendre_table(x, lmax), 2, lmax, q)
            _GAMMA_CACHE[key] = orc.gamma(M, w, tr, nthreads=cores)
        gamma = _GAMMA_CACHE[key]
    t0 = time.perf_counter()
    inv, lam, r = oracle.ortho_pca(gamma)
    t_ortho = time.perf_counter() - t0
    # projection sample
    npts_total = orc.tetrapyd_count(2, lmax)
    per_thread = 2000 if N > 1000 else 20000
    sh = shapes[0]
    t0 = time.perf_counter()
    if ref is not None:
        ref.project(sh, nthreads=cores, max_points=per_thread)
    else:
        orc.project(2, lmax, q, tr, cl, sh, nthreads=cores, max_points=per_thread)
    t_proj = (time.perf_counter() - t0) * npts_total / (per_thread * cores)
    return {"value": t_gamma + t_ortho, "unit": "s", "cores": cores, "kind": kind,
            "sample": (f"Gamma: l-contraction in full + {npairs} of {total_pairs} pairs, per-pair extrapolation; "
                       f"ortho: eigen-decomposition and PCA outputs of the actual normalised Gamma at N={N} "
                       f"(LAPACK via numpy for GSL), in full; projection: {per_thread} points/thread of {npts_total}"),
            "gamma_s": t_gamma, "ortho_s": t_ortho, "projections_per_s": 1.0 / t_proj}


def run_reference(a, ws, rank):
    import modal_gb300 as mg
    cfgd = mg.CONFIGS[a.config]
    lmax, P = cfgd["lmax"], cfgd["P"]
    q, tr, cl = mg.workload(lmax, P)
    shapes = mg.config_shapes(lmax, cfgd["shapes"], seed=0)
    res = []
    for i in range(a.warmup // 3 + a.steps):
        r = cpu_baseline(a.config, lmax, P, q, tr, cl, shapes)
        if i >= a.warmup // 3:
            res.append(r)
    v = float(np.median([r["value"] for r in res]))
    c = dict(res[-1])
    c["value"] = v
    N = len(tr)
    return {"metric": METRIC, "value": v, "unit": "s", "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": f"{a.config}: l=2..{lmax}, P={P}, N={N}, n_mu={3 * lmax // 2 + 1}, S={len(shapes)} shapes"},
            "projections_per_s": float(np.median([r["projections_per_s"] for r in res])),
            "cpu_baseline": c, "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    a = parse()
    ws, rank, local = dist()
    if a.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(a, ws, rank)), flush=True)
        return
    if ws > 1:
        import torch
        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    line = run_ours(a, ws, rank, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
