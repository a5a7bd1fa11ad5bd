"""Benchmark: converged MOMFBD patches/s on the production workload (one GB300).

Workload (default): 225 patches of 88 x 88 px, 36 modes, 3 channels x 12 frames
(wide-band + narrow-band focus + narrow-band +1 wave defocus), per-patch Kolmogorov
wavefronts at D/r0 = 15, 100 CG iterations per patch (all modes at once, FTOL = 0),
seeded synthetic data.  One step = one complete solve of the batch: image preparation
(windowing, transforms, noise, regularisation) and 100 iterations of the reference's
conjugate-gradient/line-search for every patch.

value: patches/s with the cutouts resident in HBM: the batch split over handles of about one
       object per SM each (three for 225 patches of two objects on 152 SMs), each on its own
       stream, with evaluation work items of 16 images (eval_chunk)
       (rdxg_set_patches_device per handle, then rdxg_solve_many: one CUDA graph, a branch per
       handle).
e2e:   patches/s through the public API from pinned host memory (cutouts H2D per handle,
       rdxg_solve_many, coefficients/reports/metric histories D2H), per step.
--impl reference: the reference's CPU path timed on the host cores -- redux itself does not
       build here (Boost, FFTW3, GSL, OpenCV missing), so its FP64 restatement (oracle/) is
       timed with all host threads on a bounded sample (one patch, same settings).
Multi-GPU: independent replicas (patches are independent); value = all patches / max time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "converged MOMFBD patches/s at 1e-5 rel metric vs FP64: chosen vs plain GPU"
UNIT = "patches/s"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return dict(hbm=d.get("hbm_gbs", 6800.0), src="measured", sm_max=d.get("sm_max_mhz", 2070.0))
    return dict(hbm=6800.0, src="fallback", sm_max=2070.0)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                self.rows.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        sm = [float(r[0]) for r in self.rows if len(r) >= 7 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 7 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) >= 7:
                for k, nm in enumerate(names):
                    if r[3 + k].lower().startswith("active"):
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def workload(patches, frames, iterations):
    from redux_gb300 import synth
    cache = os.path.join("/tmp", f"rdxg_bench_w2kl_{patches}_{frames}.npz")
    job = synth.make_job(88, 36, synth.LAYOUT_WB_NB(frames), basis="kl")
    if os.path.exists(cache):
        d = np.load(cache)
        cut = d["cutouts"]
    else:
        rng = np.random.default_rng(20261203 + 2)
        pt = synth.make_patches(job, patches, 15.0, rng)
        cut = pt.cutouts
        try:
            np.savez(cache, cutouts=cut)
        except OSError:
            pass
    return job, np.ascontiguousarray(cut, np.float32)


def cpu_port(job, cut, iterations, threads, n_patches=1):
    """FP64 restatement of the reference CPU path on `n_patches` patches, one patch at a time
    with OpenMP over images (redux's thread pool over images), its transforms by the oracle's
    iterative Stockham FFT with precomputed tables and stages specialised per radix (radix 8
    first); returns seconds."""
    import oracle
    t = 0.0
    finals = []
    oracle.set_fast_fft(True)
    try:
        for p in range(n_patches):
            op = oracle.OraclePatch(job, threads=threads)
            op.set_images(cut[p], None, None)
            cfg = oracle.default_cfg(max_iterations=iterations, n_modes=job.n_modes)
            t0 = time.perf_counter()
            r = op.solve(cfg)
            t += time.perf_counter() - t0
            finals.append(r["report"].final_metric)
    finally:
        oracle.set_fast_fft(False)
    return t, finals


def run_reference(args, rank):
    if rank != 0:
        return
    job, cut = workload(args.patches, args.frames, args.iterations)
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup):
        pass   # the oracle has no warm-up state; each step is a fresh patch solve
    for s in range(args.steps):
        t, _ = cpu_port(job, cut[s % cut.shape[0]:s % cut.shape[0] + 1], args.iterations, threads)
        vals.append(1.0 / t)
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": f"{args.patches} patches 88x88, 36 modes, 3ch x {args.frames} frames, "
                                   f"{args.iterations} CG iterations (one patch per step on the CPU)",
                       "l2": "cpu"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"1 patch x {args.iterations} iterations per step, FP64 restatement "
                                       f"(iterative Stockham FFT), {threads} OpenMP threads over images "
                                       f"(redux does not build here)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_uneven(args):
    """The uneven batch: patches of sizes {64, 88, 128}, 8-24 frames per channel and 36-60 KL
    modes drawn uniformly per patch (the first M modes of one expansion), staged modes and
    per-patch convergence (FTOL 1e-6).  One ragged handle per OTF size holds every patch of
    that size, each with its own frames, modes and constraints (rdxg_set_patch_shapes); the
    three handles' rounds run in one CUDA graph launch (rdxg_solve_many).  Against per-patch
    launches (each patch in a handle of its own geometry, solved one after the other) on a
    sample, whose results must be the same bits.  Not the headline line:
    `python bench.py --workload uneven` (`--levels 3` draws from three levels instead)."""
    import torch
    from redux_gb300 import solver as S, synth
    torch.cuda.set_device(0)
    n = args.patches if args.patches != 225 else 400
    t0 = time.perf_counter()
    ws = synth.uneven_batch(n, levels=args.levels or None)
    # one handle per OTF size: the largest frames and modes drawn for it, a shape per geometry
    by_size = {}
    for w in ws:
        N = w.job.otf_size
        by_size.setdefault(N, []).append(w)
    groups = []
    for N, wl in sorted(by_size.items()):
        F_max = max(int(w.job.img_wavefront.max()) + 1 for w in wl)
        M_max = max(w.job.n_modes for w in wl)
        big = synth.make_job(N, M_max, synth.LAYOUT_WB_NB(F_max), basis="kl", kl_last=synth.UNEVEN_KL_LAST)
        shapes, assign, cuts, members = [], [], [], []
        for k, w in enumerate(wl):
            F = int(w.job.img_wavefront.max()) + 1
            shapes.append((F, w.job.n_modes, w.job.nullspace))
            for i in range(w.patches.cutouts.shape[0]):
                c = np.zeros((big.n_images, big.cutout_size, big.cutout_size), np.float32)
                c[:w.job.n_images] = w.patches.cutouts[i]
                cuts.append(c)
                assign.append(k)
                members.append((w, i))
        groups.append(dict(N=N, big=big, shapes=shapes, assign=assign, cut=np.stack(cuts), members=members))
    t_gen = time.perf_counter() - t0
    st = S.SolveSettings(mode_start=5, mode_step=5, max_iterations=args.iterations if args.iterations != 100 else 30,
                         min_iterations=5, ftol=1e-6, max_metrics=4096)
    hs = []
    for g in groups:
        h = S.Solver(g["big"], max_patches=len(g["assign"]))
        h.set_patch_shapes(g["shapes"], g["assign"])
        h.set_patches(g["cut"])
        hs.append(h)
    for _ in range(args.warmup):
        S.solve_many(hs, st)
    torch.cuda.synchronize()
    times = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            for h, g in zip(hs, groups):
                h.set_patches(g["cut"])
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            outs = S.solve_many(hs, st)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
    iters, evals = [], []
    for out in outs:
        iters += [r.iterations for r in out["reports"]]
        evals += [r.n_f_evals + r.n_df_evals for r in out["reports"]]
    t_many = statistics.median(times)
    launches = sum(h.launch_count() for h in hs)
    # per-patch launches on a sample (3 patches of each size), each its own geometry's handle;
    # their results against the batch's
    t_single, n_single, identical = 0.0, 0, True
    for g, out in zip(groups, outs):
        for pi in range(min(3, len(g["members"]))):
            w, i = g["members"][pi]
            h1 = S.Solver(w.job, max_patches=1)
            for rep in range(2):     # the first solve of a handle plans its launch shapes: time the second
                h1.set_patches(w.patches.cutouts[i:i + 1])
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                o1 = h1.run(st)
                torch.cuda.synchronize()
                if rep:
                    t_single += time.perf_counter() - t0
            I, M = w.job.n_images, w.job.n_modes
            identical &= bool(np.array_equal(out["alpha"][pi][:I, :M], o1["alpha"][0]))
            r, r1 = out["reports"][pi], o1["reports"][0]
            identical &= bool(np.array_equal(out["metrics"][pi, :r.n_metrics], o1["metrics"][0, :r1.n_metrics]))
            n_single += 1
            h1.close()
    line = {"metric": "uneven-batch converged patches/s", "value": n / t_many, "unit": UNIT,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_many * 1000.0,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (FP64 sums and CG scalars)", "data": "synthetic",
            "config": {"workload": f"{n} patches, sizes {{64, 88, 128}}, frames 8-24, 36-60 KL modes"
                                   + (f" ({args.levels} levels)" if args.levels else " (uniform draws)")
                                   + ", staged modes, FTOL 1e-6, at most "
                                   + f"{st.max_iterations} iterations per stage",
                       "geometries": len(ws), "handles": len(hs),
                       "patches_per_handle": {g["N"]: len(g["assign"]) for g in groups},
                       "iterations_median": float(np.median(iters)),
                       "evaluations_per_patch": float(np.mean(evals)), "generation_s": t_gen},
            "gpu_launches": int(launches),
            "launch_shapes": {g["N"]: h.launch_shape() for g, h in zip(groups, hs)},
            "per_patch_launches": {"value": n_single / t_single, "unit": UNIT,
                                   "sample": f"{n_single} patches (3 per size), each in a handle of its own geometry",
                                   "results_identical_to_batch": identical},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    for h in hs:
        h.close()


def _dist(v):
    v = np.asarray(v, np.float64)
    if v.size == 0:
        return None
    return {"n": int(v.size), "median": float(np.median(v)), "p90": float(np.percentile(v, 90)),
            "min": float(v.min()), "max": float(v.max())}


def run_convergence(args):
    """Converged parity on the production batch (225 patches 88 x 88, 36 KL modes, 3 x 12
    images): every patch solved to convergence (all modes at once, FTOL on the relative metric
    change, at least 5 iterations, 3 consecutive changes below FTOL) in FP32 and in FP64, and:
      * FP64 continuation: an FP64 handle takes each FP32 solution as its starting point (same
        images, rdxg_set_start_alpha) and solves on with the same settings; the relative
        metric drop it still finds says whether FP32 stopped at an FP64-converged point;
      * the same continuation from the FP64 solutions (the control: how far FP64's own
        converged points are from converged);
      * the signed difference of the FP32 and FP64 converged metrics (both evaluated in
        FP64) and, as the noise floor of the problem, of the FP64 GPU and the FP64 oracle on a
        sample of patches (two FP64 implementations that differ only in rounding order).
    Not the headline line: `python bench.py --workload convergence`."""
    import torch
    from redux_gb300 import solver as S
    torch.cuda.set_device(0)
    job, cut = workload(args.patches, args.frames, args.iterations)
    P, M = cut.shape[0], job.n_modes
    lam = job.wavelength
    conv = S.SolveSettings(mode_start=M, mode_step=M, max_iterations=args.conv_max_iterations, min_iterations=5,
                           target_iterations=3, ftol=args.conv_ftol, max_metrics=args.conv_max_iterations + 16)

    def timed(s, settings):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = s.run(settings)
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    # FP32 (the chosen form), the whole batch in one handle; one warm-up solve (launch planner,
    # graph capture)
    s32 = S.Solver(job, max_patches=P)
    s32.set_patches(cut)
    s32.run(conv)
    s32.set_patches(cut)
    o32, t32 = timed(s32, conv)
    a32 = o32["alpha"]
    it32 = [r.iterations for r in o32["reports"]]
    # FP64, the whole batch in one handle
    s64 = S.Solver(job, max_patches=P, precision="fp64")
    s64.set_patches(cut)
    L64_at32 = s64.metric(a32)
    o64, t64 = timed(s64, conv)
    a64 = o64["alpha"]
    L64 = np.array([r.final_metric for r in o64["reports"]])
    it64 = [r.iterations for r in o64["reports"]]
    # continuations in FP64 from both endpoints
    s64.set_start_alpha(a32)
    oc32, tc32 = timed(s64, conv)
    s64.set_start_alpha(a64)
    oc64, _ = timed(s64, conv)
    s64.set_start_alpha(None)

    def drops(o):
        return [(r.initial_metric - r.final_metric) / abs(r.initial_metric) for r in o["reports"]]

    drop32, drop64 = drops(oc32), drops(oc64)
    init_check = float(np.max(np.abs(np.array([r.initial_metric for r in oc32["reports"]]) - L64_at32)
                              / np.abs(L64_at32)))
    signed = (L64_at32 - L64) / np.abs(L64)
    rms = lambda a, b: np.sqrt(np.mean((a - b) ** 2, axis=(1, 2))) / lam
    # plain FP64 GPU form (one patch per launch sequence) on a sample, for the speed ratio
    nplain = min(4, P)
    s1 = S.Solver(job, max_patches=1, precision="fp64")
    t_plain = 0.0
    for p in range(nplain):
        s1.set_patches(cut[p:p + 1])
        _, t = timed(s1, conv)
        t_plain += t
    s1.close()
    # noise floor: the FP64 oracle (CPU) on a sample, same settings
    import oracle
    threads = os.cpu_count() or 1
    noise, f32_vs_oracle = [], []
    t_or = 0.0
    for p in range(min(args.conv_oracle_patches, P)):
        op = oracle.OraclePatch(job, threads=threads)
        op.set_images(cut[p], None, None)
        cfg = oracle.Cfg(n_initial_modes=M, n_mode_increment=M, max_iterations=conv.max_iterations,
                         min_iterations=conv.min_iterations, target_iterations=conv.target_iterations,
                         fd_first=1, ftol=conv.ftol, eps=conv.eps, brent_tol=0.1)
        t0 = time.perf_counter()
        ro = op.solve(cfg)
        t_or += time.perf_counter() - t0
        Lo = ro["report"].final_metric
        noise.append((L64[p] - Lo) / abs(Lo))
        f32_vs_oracle.append((L64_at32[p] - Lo) / abs(Lo))
    line = {"metric": "converged patches/s, FP32 against FP64 (continuation drop <= 1e-5)",
            "value": P / t32, "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": t32 * 1000.0,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (FP64 sums and CG scalars)", "data": "synthetic",
            "config": {"workload": f"{P} patches 88x88, 36 KL modes, 3ch x {args.frames} frames, D/r0=15, "
                                   f"all modes at once, FTOL {args.conv_ftol:g} (3 consecutive), MIN_ITER 5, "
                                   f"MAX_ITER {args.conv_max_iterations}"},
            "fp32": {"patches_per_s": P / t32, "iterations": _dist(it32)},
            "fp64_batch": {"patches_per_s": P / t64, "iterations": _dist(it64)},
            "plain_fp64_gpu": {"patches_per_s": nplain / t_plain, "sample": f"{nplain} patches, per-patch launches"},
            "speedup_fp32_vs_plain_fp64": (P / t32) / (nplain / t_plain),
            "continuation_from_fp32": {
                "rel_metric_drop": _dist(drop32),
                "within_1e-5": int(sum(1 for d in drop32 if d <= 1e-5)),
                "within_1e-6": int(sum(1 for d in drop32 if d <= 1e-6)),
                "alpha_moved_rms_rad": _dist(rms(oc32["alpha"], a32)),
                "iterations": _dist([r.iterations for r in oc32["reports"]]),
                "start_metric_vs_fp64_at_fp32_alpha_max_rel": init_check,
                "seconds": tc32},
            "continuation_from_fp64": {
                "rel_metric_drop": _dist(drop64),
                "within_1e-5": int(sum(1 for d in drop64 if d <= 1e-5)),
                "within_1e-6": int(sum(1 for d in drop64 if d <= 1e-6))},
            "fp32_minus_fp64_final_rel": {"signed": _dist(signed), "abs": _dist(np.abs(signed)),
                                           "within_1e-5": int(np.sum(np.abs(signed) <= 1e-5)),
                                           "fp32_lower": int(np.sum(signed < 0)),
                                           "alpha_rms_rad": _dist(rms(a32, a64))},
            "noise_floor_fp64_gpu_minus_oracle_rel": {"signed": noise, "fp32_minus_oracle": f32_vs_oracle,
                                                      "oracle_seconds": t_or, "oracle_threads": threads}}
    # restarted solves: each precision continues from its own endpoint (a CG restart: beta from
    # zero, steepest descent first) until a whole restart cycle lowers no patch's metric by more
    # than the restart tolerance; then both endpoints are compared again, in FP64
    if args.conv_restarts > 0:
        def restart_loop(s, a0, L0):
            a, L = a0, np.asarray(L0, np.float64)
            cycles, tot_it, t = 0, 0, 0.0
            hist = []
            for _ in range(args.conv_restarts):
                s.set_start_alpha(a)
                o, dt = timed(s, conv)
                t += dt
                cycles += 1
                Ln = np.array([r.final_metric for r in o["reports"]])
                tot_it += int(np.sum([r.iterations for r in o["reports"]]))
                d = (L - Ln) / np.abs(L)
                hist.append(float(np.max(d)))
                a, L = o["alpha"], Ln
                if np.max(d) <= args.conv_restart_tol:
                    break
            s.set_start_alpha(None)
            return a, L, cycles, tot_it, t, hist
        ra32, rL32, cyc32, tit32, rt32, h32 = restart_loop(s32, a32, [r.final_metric for r in o32["reports"]])
        ra64, rL64, cyc64, tit64, rt64, h64 = restart_loop(s64, a64, L64)
        rL64_at32 = s64.metric(ra32)
        rs = (rL64_at32 - rL64) / np.abs(rL64)
        line["restarted"] = {
            "restart_tol": args.conv_restart_tol,
            "fp32": {"cycles": cyc32, "max_drop_per_cycle": h32, "extra_iterations_per_patch": tit32 / P,
                     "seconds": rt32, "patches_per_s_total": P / (t32 + rt32)},
            "fp64": {"cycles": cyc64, "max_drop_per_cycle": h64, "extra_iterations_per_patch": tit64 / P,
                     "seconds": rt64, "patches_per_s_total": P / (t64 + rt64)},
            "fp32_minus_fp64_final_rel": {"signed": _dist(rs), "abs": _dist(np.abs(rs)),
                                           "within_1e-5": int(np.sum(np.abs(rs) <= 1e-5)),
                                           "within_1e-4": int(np.sum(np.abs(rs) <= 1e-4)),
                                           "fp32_lower": int(np.sum(rs < 0)),
                                           "alpha_rms_rad": _dist(rms(ra32, ra64))}}
    print(json.dumps(line), flush=True)
    if args.conv_save:
        np.savez(args.conv_save, a32=a32, a64=a64, ac32=oc32["alpha"], ac64=oc64["alpha"], L64_at32=L64_at32,
                 L64=L64, drop32=drop32, drop64=drop64, it32=it32, it64=it64)
    s32.close()
    s64.close()


def run_large(args):
    """Large patches, mixed precision: 128 x 128 patches, 3 channels x 32
    frames, 100 KL modes at D/r0 = 25; mode expansion on the tensor cores (tcgen05, BF16-split
    FP32 operands, 6xBF16 by default; `--phase-mode 2` for the 3xBF16 split, 0 for the CUDA
    cores), FP32 transforms, FP64 metric sums and CG scalars.  `--iterations` CG iterations per patch with all modes at once, as the
    headline workload.  Reports patches/s and CG iterations/s, the kernel times with their
    nominal FP32 rates and HBM fractions, and the errors against the FP64 restatement on one
    patch: the metric, gradient and restored object at the same alpha (per-evaluation
    precision) and the metric history, alpha and restored object after a short solve of both.
    Defaults to 1 warm-up and 2 timed solves.  Not the headline line: `python bench.py --workload large`."""
    import torch
    from redux_gb300 import solver as S, synth
    torch.cuda.set_device(0)
    P = args.patches if args.patches != 225 else 256
    t0 = time.perf_counter()
    w = synth.workload("large128", n_patches=P)
    t_gen = time.perf_counter() - t0
    job, cut = w.job, np.ascontiguousarray(w.patches.cutouts, np.float32)
    settings = S.fixed_iterations(job.n_modes, args.iterations, max_metrics=args.iterations + 8)
    s = S.Solver(job, max_patches=P)
    if args.phase_mode is not None:
        s.set_phase_mode(args.phase_mode)
    for _ in range(args.warmup):
        s.set_patches(cut)
        s.run(settings)
    torch.cuda.synchronize()
    times = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            s.set_patches(cut)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = s.run(settings)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
    t_solve = statistics.median(times)
    reps = out["reports"]
    nf = sum(r.n_f_evals for r in reps) / P
    ndf = sum(r.n_df_evals for r in reps) / P
    launches = s.launch_count()
    # kernel times on the loaded batch at its last point
    kt = s.profile_kernels(reps=3)
    peaks = _peaks()
    N, n, M, I = job.otf_size, job.pupil_pixels, job.n_modes, job.n_images
    G = P * I
    fft_flops = 5.0 * N * N * math.log2(N * N)
    flops = {"forward": G * (2 * fft_flops + 2.0 * M * n * n), "accum": G * 16.0 * N * N,
             "adjoint": G * (2 * fft_flops + 2.0 * M * n * n)}
    # compulsory HBM bytes per launch: forward reads nothing per image but writes S (8 N^2);
    # the accumulation reads D and S twice and writes O and Q; the adjoint reads D, S, X, O, Q, PF
    hbm = {"forward": G * 8.0 * N * N, "accum": G * 4 * 8.0 * N * N, "adjoint": G * (4 * 8.0 * N * N + 8.0 * n * n)}
    kern = {k: {"ms": kt[k], "fp32_tflops": flops[k] / (kt[k] / 1e3) / 1e12,
                "hbm_gbs": hbm[k] / (kt[k] / 1e3) / 1e9, "hbm_frac": hbm[k] / (kt[k] / 1e3) / 1e9 / peaks["hbm"]}
            for k in ("forward", "accum", "adjoint")}
    # errors against the FP64 restatement (CPU) on one patch: the metric, gradient and restored
    # object at the same alpha, and a short solve of both
    import oracle
    threads = os.cpu_count() or 1
    check_iters = args.check_iterations
    s1 = S.Solver(job, max_patches=1)
    s1.set_patches(cut[:1])
    op = oracle.OraclePatch(job, threads=threads)
    op.set_images(cut[0], None, None)
    at = w.patches.alpha_true[:1]
    fc = N / 2.0
    m_o = op.metric(at[0])
    _, g_o = op.gradient(at[0], method="vogel")
    g_1, _ = s1.gradient(at)
    obj_o = op.restore(at[0], fc)
    obj_1 = s1.restore(at, fc)[0]
    st_short = S.fixed_iterations(M, check_iters, max_metrics=check_iters + 8)
    r1 = s1.run(st_short)
    t0 = time.perf_counter()
    ro = op.solve(oracle.default_cfg(max_iterations=check_iters, n_modes=M))
    t_cpu = time.perf_counter() - t0
    obj_1s = s1.restore(r1["alpha"], fc)[0]
    obj_os = op.restore(ro["alpha"], fc)
    fin_1, fin_o = r1["reports"][0].final_metric, ro["report"].final_metric
    nm = min(r1["reports"][0].n_metrics, len(ro["metrics"]))
    hist_rel = np.abs(r1["metrics"][0, :nm] - ro["metrics"][:nm]) / np.abs(ro["metrics"][:nm])
    errors = {
        "reference": "FP64 restatement of the reference (CPU), 1 patch",
        "metric_rel_same_alpha": abs(s1.metric(at)[0] - m_o) / abs(m_o),
        "gradient_rel_norm_same_alpha": float(np.linalg.norm(g_1[0] - g_o) / np.linalg.norm(g_o)),
        "object_rel_peak_same_alpha": float(np.abs(obj_1 - obj_o).max() / np.abs(obj_o).max()),
        "short_solve_iterations": check_iters,
        "short_solve_metric_history_rel_max": float(hist_rel.max()) if nm else None,
        "short_solve_final_metric_rel": abs(fin_1 - fin_o) / abs(fin_o),
        "short_solve_alpha_rms_rad": float(np.sqrt(np.mean((r1["alpha"][0] - ro["alpha"]) ** 2)) / job.wavelength),
        "short_solve_object_rel_peak": float(np.abs(obj_1s - obj_os).max() / np.abs(obj_os).max()),
    }
    s1.close()
    # the plain FP64 GPU form at N = 128 (the general path in double, its work tiles in global
    # memory): the same solve with per-patch launches on a sample of patches, and the FP32
    # path's errors against it at the same alpha on the same patches
    nb = max(1, min(args.large_fp64_patches, P))
    s64 = S.Solver(job, max_patches=1, precision="fp64")
    t64, fin64 = 0.0, []
    for p in range(nb):
        s64.set_patches(cut[p:p + 1])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r64 = s64.run(settings)
        torch.cuda.synchronize()
        t64 += time.perf_counter() - t0
        fin64.append(r64["reports"][0].final_metric)
    s64.close()
    plain_v = nb / t64
    sb32 = S.Solver(job, max_patches=nb)
    sb32.set_patches(cut[:nb])
    sb64 = S.Solver(job, max_patches=nb, precision="fp64")
    sb64.set_patches(cut[:nb])
    a_same = w.patches.alpha_true[:nb]
    m32, m64 = sb32.metric(a_same), sb64.metric(a_same)
    g32, _ = sb32.gradient(a_same)
    g64, _ = sb64.gradient(a_same)
    o32, o64 = sb32.restore(a_same, fc), sb64.restore(a_same, fc)
    errors["fp64_gpu"] = {
        "reference": f"FP64 GPU form, {nb} patches, at the true alpha",
        "metric_rel": (np.abs(m32 - m64) / np.abs(m64)).tolist(),
        "gradient_rel_norm": [float(np.linalg.norm(g32[p] - g64[p]) / np.linalg.norm(g64[p])) for p in range(nb)],
        "object_rel_peak": [float(np.abs(o32[p] - o64[p]).max() / np.abs(o64[p]).max()) for p in range(nb)],
        "final_metric_signed_rel_after_solve": [(reps[p].final_metric - fin64[p]) / abs(fin64[p]) for p in range(nb)],
    }
    # converged: the whole batch to convergence (FTOL 1e-6 three times in a row, all modes at
    # once), then FP64 continuations from the FP32 endpoints and from FP64's own on the sample
    conv = S.SolveSettings(mode_start=M, mode_step=M, max_iterations=args.conv_max_iterations, min_iterations=5,
                           target_iterations=3, ftol=args.conv_ftol, max_metrics=4096)
    s.set_patches(cut)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc = s.run(conv)
    torch.cuda.synchronize()
    t_conv = time.perf_counter() - t0
    a32c = rc["alpha"]
    t0 = time.perf_counter()
    r64c = sb64.run(conv)
    torch.cuda.synchronize()
    t64c = time.perf_counter() - t0

    def continuation(a):
        sb64.set_start_alpha(a)
        rr = sb64.run(conv)["reports"]
        return [(r.initial_metric - r.final_metric) / r.initial_metric for r in rr]

    d32 = continuation(a32c[:nb])
    d64 = continuation(r64c["alpha"])
    sb32.close()
    sb64.close()
    fin32c = [rc["reports"][p].final_metric for p in range(nb)]
    fin64c = [r.final_metric for r in r64c["reports"]]
    its = [r.iterations for r in rc["reports"]]
    converged = {
        "settings": f"all modes at once, FTOL {args.conv_ftol} (3 consecutive), MIN_ITER 5, "
                    f"MAX_ITER {args.conv_max_iterations}",
        "patches_per_s": P / t_conv, "iterations_median": float(np.median(its)), "iterations_max": int(max(its)),
        "fp64_batch_patches_per_s": nb / t64c,
        "continuation_drop_from_fp32": d32, "continuation_drop_from_fp64": d64,
        "fp32_minus_fp64_final_signed_rel": [(a - b) / abs(b) for a, b in zip(fin32c, fin64c)],
    }
    line = {"metric": "large-patch patches/s", "value": P / t_solve, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_solve * 1000.0, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 sums and CG scalars)", "data": "synthetic",
            "config": {"workload": f"{P} patches 128x128, 100 KL modes, 3ch x 32 frames, D/r0=25, "
                                   f"{args.iterations} CG iterations, all modes at once",
                       "metric_evals_per_patch": nf, "gradient_evals_per_patch": ndf,
                       "cg_iterations_per_s": P * args.iterations / t_solve, "generation_s": t_gen,
                       "mode_expansion": {0: "CUDA cores, FP32 (inside the transform kernel)",
                                          2: "tensor cores, 3xBF16 split, FP32 accumulation (k_phase_tc)",
                                          3: "tensor cores, 6xBF16 split, FP32 accumulation (k_phase_tc)"}[
                                              s.phase_mode()],
                       "l2": "inputs larger than L2 (D, S: 2 x %.1f GB)" % (G * 8.0 * N * N / 1e9)},
            "gpu_launches": int(launches), "kernels": kern, "peak_hbm_gbs": peaks["hbm"],
            "launch_shapes": s.launch_shape(),
            "errors_vs_fp64": errors,
            "plain_fp64_gpu": {"value": plain_v, "unit": UNIT, "sample": f"{nb} patches, per-patch launches",
                               "speedup_chosen_vs_plain": P / t_solve / plain_v},
            "converged": converged,
            "cpu_baseline": {"value": 1.0 / t_cpu * check_iters / args.iterations, "unit": UNIT, "cores": threads,
                             "kind": "port", "sample": f"1 patch x {check_iters} iterations, FP64 restatement, "
                                                       f"{threads} OpenMP threads over images, scaled to "
                                                       f"{args.iterations} iterations"},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    s.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default 5; 2 for --workload large)")
    ap.add_argument("--warmup", type=int, default=None, help="warm-up steps (default 3; 1 for --workload large)")
    ap.add_argument("--impl", default="ours")
    ap.add_argument("--patches", type=int, default=225)
    ap.add_argument("--frames", type=int, default=12)
    ap.add_argument("--iterations", type=int, default=100)
    ap.add_argument("--no-baselines", action="store_true")
    ap.add_argument("--handles", type=int, default=0,
                    help="handles (each on its own stream) the batch is split over, solved together "
                         "(0: about one object per SM in each)")
    ap.add_argument("--chunk", type=int, default=0,
                    help="images of an object per evaluation work item (eval_chunk; 0: 16 when the batch "
                         "is split over several handles, else the library's 6)")
    ap.add_argument("--workload", default="production", choices=("production", "uneven", "large", "convergence"),
                    help="production: the headline batch (225 patches 88 x 88); uneven: 400 patches of "
                         "{64, 88, 128} px; large: 256 patches 128 x 128 with 100 modes; convergence: the "
                         "headline batch solved to convergence in FP32 and FP64 with FP64 continuations")
    ap.add_argument("--phase-mode", type=int, default=None, choices=(0, 2, 3),
                    help="large patches: mode expansion (3: tensor cores 6xBF16, the default; 2: 3xBF16; "
                         "0: CUDA cores)")
    ap.add_argument("--conv-ftol", type=float, default=1e-6, help="convergence: FTOL")
    ap.add_argument("--conv-max-iterations", type=int, default=2000, help="convergence: MAX_ITER")
    ap.add_argument("--conv-oracle-patches", type=int, default=4,
                    help="convergence: patches also solved by the FP64 oracle (noise floor)")
    ap.add_argument("--conv-save", default="", help="convergence: write the coefficients to this .npz")
    ap.add_argument("--conv-restarts", type=int, default=0,
                    help="convergence: restart cycles (continuations from the own endpoint) at most")
    ap.add_argument("--conv-restart-tol", type=float, default=1e-6,
                    help="convergence: stop restarting once no patch's metric drops by more than this")
    ap.add_argument("--levels", type=int, default=0,
                    help="uneven batch: frames and modes from this many values (0: uniform draws)")
    ap.add_argument("--large-fp64-patches", type=int, default=4,
                    help="large patches: patches solved by the plain FP64 GPU form and compared with it")
    ap.add_argument("--check-iterations", type=int, default=10,
                    help="large patches: CG iterations of the solve compared with the FP64 restatement")
    ap.add_argument("--kernels-only", action="store_true",
                    help="load the batch and time each kernel once (profiling target)")
    args = ap.parse_args()
    large = args.workload == "large" and args.impl != "reference"
    if args.warmup is None:
        args.warmup = 1 if large else 3
    if args.steps is None:
        args.steps = 2 if large else 5
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)
    if args.workload == "convergence":
        return run_convergence(args)
    if args.workload == "uneven":
        return run_uneven(args)
    if args.workload == "large":
        return run_large(args)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from redux_gb300 import solver as S

    job, cut = workload(args.patches, args.frames, args.iterations)
    P = cut.shape[0]
    settings = S.fixed_iterations(job.n_modes, args.iterations, max_metrics=args.iterations + 8)
    if args.kernels_only:
        solver = S.Solver(job, max_patches=P, device=local)
        solver.set_patches(cut)
        tuned = solver.autotune(reps=3)     # the shapes a solve would use
        kt = solver.profile_kernels(reps=1)
        torch.cuda.synchronize()
        print(json.dumps({"kernel_ms": kt, "patches": P, "launch_shapes": tuned}), flush=True)
        solver.close()
        return
    # the batch split over H handles, each on its own stream, solved together (one CUDA graph,
    # a branch per handle): one handle's latency-bound kernels of a round overlap the others'
    # evaluations.  With about one object per SM in each handle, large evaluation work items
    # (fewer per-item overheads) pay, as the handles' evaluations fill each other's tails.
    # Measured on the 225-patch batch (objects of 12 and 24 images), ms per step, by work-item
    # size: 1 handle 709 (6), 743 (12), 858 (18); 3 handles 688 (6), 678 (12), 668.7 (16),
    # 669.7 (18), 672 (20), 694 (24); 4 handles 688 (12, 16); 5 handles 696 (6), 687 (18).
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    H = args.handles or max(1, round(P * job.n_objects / sms))
    H = max(1, min(H, P))
    chunk = args.chunk or (16 if H > 1 else 0)
    bounds = [int(round(P * k / H)) for k in range(H + 1)]
    parts = [(bounds[k], bounds[k + 1]) for k in range(H)]
    solvers, streams = [], []
    for b0, b1 in parts:
        sk = S.Solver(job, max_patches=b1 - b0, device=local, eval_chunk=chunk)
        st = torch.cuda.Stream()
        sk.set_stream(st.cuda_stream)
        solvers.append(sk)
        streams.append(st)
    stream = streams[0]           # the graph runs on the first handle's stream
    cut_dev = torch.from_numpy(cut).to(f"cuda:{local}")
    cut_pin = torch.from_numpy(cut).pin_memory()
    cut_pin_np = cut_pin.numpy()
    torch.cuda.synchronize()

    def load_device():
        for sk, (b0, b1) in zip(solvers, parts):
            sk.set_patches_device(b1 - b0, cut_dev[b0:b1].data_ptr())

    def step_device():
        load_device()
        S.solve_many(solvers, settings, fetch=False)

    def fetch_all(max_metrics):
        outs = [sk.fetch(max_metrics) for sk in solvers]
        return dict(alpha=np.concatenate([o["alpha"] for o in outs]),
                    reports=[r for o in outs for r in o["reports"]])

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step_device()
    barrier()
    launches = 0
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            step_device()
            launches += sum(sk.launch_count() for sk in solvers) + H   # + one preparation each
        e1.record(stream)
        e1.synchronize()
        barrier()
        ms_dev = e0.elapsed_time(e1) / args.steps
    rounds = solvers[0].launch_count() / 6.0
    out = fetch_all(settings.max_metrics)
    reps = out["reports"]
    iters = [r.iterations for r in reps]
    nf = sum(r.n_f_evals for r in reps) / P
    ndf = sum(r.n_df_evals for r in reps) / P

    # end to end through the public API from pinned host memory
    ms_e2e = []
    alpha_bytes = P * job.n_images * job.n_modes * 8
    for _ in range(args.steps):
        barrier()
        t0 = time.perf_counter()
        for sk, (b0, b1) in zip(solvers, parts):
            sk.set_patches(cut_pin_np[b0:b1])
        S.solve_many(solvers, settings)
        torch.cuda.synchronize()
        ms_e2e.append((time.perf_counter() - t0) * 1000.0)
    e2e_ms = statistics.median(ms_e2e)
    h2d = cut.nbytes
    d2h = alpha_bytes + P * 48 + P * settings.max_metrics * 8

    from redux_gb300.replicas import max_over_ranks
    ms_dev, e2e_ms = max_over_ranks([ms_dev, e2e_ms], device=f"cuda:{local}")
    value = world * P / (ms_dev / 1000.0)
    e2e_value = world * P / (e2e_ms / 1000.0)

    # roofline of the dominant kernel, measured on the whole batch in one handle (6-image
    # evaluation work items)
    solver = S.Solver(job, max_patches=P, device=local)
    solver.set_patches_device(P, cut_dev.data_ptr())
    solver.autotune(reps=3)
    kt = solver.profile_kernels(reps=5)
    peaks = _peaks()
    N, n, M = job.otf_size, job.pupil_pixels, job.n_modes
    G = P * job.n_images
    # per image and metric evaluation: the transforms of the OTF and the mode expansion
    fft_flops = 5.0 * N * N * math.log2(N * N)
    f_eval_flops = 2 * fft_flops + 2.0 * M * n * n
    per_launch = {
        "forward": dict(bytes=G * 8.0 * N * N, flops=G * f_eval_flops),
        "accum": dict(bytes=G * 2 * 8.0 * N * N, flops=G * 16.0 * N * N),
        "adjoint": dict(bytes=G * 4 * 8.0 * N * N, flops=G * (2 * fft_flops + 2.0 * M * n * n)),
    }
    # time share per step: forward and accumulation run every round, the adjoint only does
    # work in rounds where a patch needs a gradient (about one in ten)
    share = {"forward": rounds * kt["forward"], "accum": rounds * kt["accum"], "adjoint": ndf * kt["adjoint"]}
    dom = max(share, key=share.get)
    hbm_achieved = per_launch[dom]["bytes"] / (kt[dom] / 1000.0) / 1e9
    fp32_tflops = {k: per_launch[k]["flops"] / (kt[k] / 1000.0) / 1e12 for k in per_launch}
    # DRAM bytes per image of the forward pass from ncu captures of the 64-patch batch
    # (k_eval: 80.9 MB read + 3.4 MB written for 2304 images; k_phase_tc: 0.95 MB read, its
    # phases stay in L2), scaled to this launch by the images it evaluates: a constant, not
    # measured in this run
    traffic = {"forward": G * (84.3e6 + 0.95e6) / 2304.0} if (N, M) == (88, 36) else {}
    # the evaluation is bound by FP32 issue and shared-memory traffic of its transforms, not
    # by HBM (ncu: issue-bound, DRAM well below its peak): the primary fraction is its nominal
    # FFT flops (5 P log2 P per transform) plus the mode expansion against the FP32 CUDA-core
    # peak (SMs x 128 lanes x 2 flops x maximum SM clock; computed, there is no measured FP32
    # peak), the HBM fraction of its algorithmic bytes (8 N^2 per image) beside it
    props = torch.cuda.get_device_properties(local)
    fp32_peak = props.multi_processor_count * 128 * 2 * peaks["sm_max"] * 1e6 / 1e12
    roofline = {"bound": "fp32", "achieved": fp32_tflops[dom], "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": fp32_tflops[dom] / fp32_peak,
                "peak_source": "computed: SMs x 128 FP32 lanes x 2 flops x maximum SM clock",
                "traffic": traffic.get(dom),
                "traffic_source": "constant: ncu dram__bytes_read.sum + dram__bytes_write.sum of a 64-patch capture "
                                  "(profiles/k_eval_88x88_64patches.md), scaled by images" if dom in traffic else None,
                "kernel": dom, "kernel_ms": kt, "share_ms_per_step": share,
                "hbm": {"achieved": hbm_achieved, "peak": peaks["hbm"], "unit": "GB/s",
                        "frac": hbm_achieved / peaks["hbm"], "peak_source": peaks["src"]},
                "fp32_tflops": fp32_tflops,
                "fp32_frac": {k: v / fp32_peak for k, v in fp32_tflops.items()}}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_dev, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (FP64 sums and CG scalars)", "data": "synthetic",
            "config": {"workload": f"{P} patches 88x88, 36 KL modes, 3ch x {args.frames} frames, D/r0=15, "
                                   f"{args.iterations} CG iterations, all modes at once",
                       "patches_per_gpu": P, "iterations": args.iterations,
                       "handles": H, "handle_patches": [b1 - b0 for b0, b1 in parts],
                       "eval_chunk": chunk or 6,
                       "l2": "inputs larger than L2 (D, OTF: 2 x 500 MB per batch)",
                       "metric_evals_per_patch": nf, "gradient_evals_per_patch": ndf,
                       "cg_iterations_per_s": world * P * args.iterations / (ms_dev / 1000.0)},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches), "roofline": roofline, "clocks": clk.summary(),
            "launch_shapes": solvers[0].launch_shape()}

    if rank == 0 and not args.no_baselines:
        # plain FP64 GPU form: same algorithm in double precision, one patch per launch sequence
        nplain = min(4, P)
        s64 = S.Solver(job, max_patches=1, precision="fp64", device=local)
        t_plain = 0.0
        finals64, alphas64 = [], []
        for p in range(nplain):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s64.set_patches(cut[p:p + 1])
            r64 = s64.run(settings)
            torch.cuda.synchronize()
            t_plain += time.perf_counter() - t0
            finals64.append(r64["reports"][0].final_metric)
            alphas64.append(r64["alpha"][0])
        plain_v = nplain / t_plain
        f32 = [reps[p].final_metric for p in range(nplain)]
        rel = [abs(a - b) / abs(b) for a, b in zip(f32, finals64)]
        # the metric at the chosen path's final alpha, evaluated by both forms on fresh handles
        s32c = S.Solver(job, max_patches=nplain, device=local)
        s32c.set_patches(cut[:nplain])
        s64c = S.Solver(job, max_patches=nplain, precision="fp64", device=local)
        s64c.set_patches(cut[:nplain])
        m32c, m64c = s32c.metric(out["alpha"][:nplain]), s64c.metric(out["alpha"][:nplain])
        s32c.close(); s64c.close()
        line["plain_fp64_gpu"] = {"value": plain_v, "unit": UNIT, "sample": f"{nplain} patches, per-patch launches",
                                  "speedup_chosen_vs_plain": value / world / plain_v,
                                  "final_metric_rel_diff_vs_fp64": rel,
                                  "final_metric_signed_rel_vs_fp64": [(a - b) / abs(b) for a, b in zip(f32, finals64)],
                                  "within_1e-5": sum(1 for x in rel if x <= 1e-5),
                                  "metric_rel_fp64_at_final_alpha": (np.abs(m32c - m64c) / np.abs(m64c)).tolist(),
                                  # alpha is in the reference's units (wavefront, lambda * rad)
                                  "alpha_rms_diff_rad": [float(np.sqrt(np.mean((out["alpha"][p] - alphas64[p]) ** 2))
                                                               / job.wavelength) for p in range(nplain)],
                                  "note": "per-evaluation metric and gradient agree with FP64 to ~1e-7; the "
                                          "reference's CG line search amplifies rounding along the trajectory "
                                          "(FP64 GPU vs FP64 CPU: <5e-6 after 100 iterations, 1e-4 after 400)"}
        s64.close()
        # converged solves with the reference's default settings (MODE_START 5, MODE_STEP 5,
        # MIN_ITER 5, MAX_ITER 500, N_DONE_ITER 3, FTOL 1e-3: staged modes, re-shifts between
        # stages, per-patch stop), the batch against the plain FP64 form on a sample
        # Patches stop at different rounds, so the late rounds carry few objects: these solves
        # run on handles of their own with the library's default 6-image evaluation work items
        # (the same split; 16-image items: 670.6 against 688.8 patches/s)
        conv = S.SolveSettings(max_metrics=4096)
        conv_solvers = []
        for (b0, b1), st in zip(parts, streams):
            sk = S.Solver(job, max_patches=b1 - b0, device=local)
            sk.set_stream(st.cuda_stream)
            conv_solvers.append(sk)

        def solve_conv():
            for sk, (b0, b1) in zip(conv_solvers, parts):
                sk.set_patches_device(b1 - b0, cut_dev[b0:b1].data_ptr())
            S.solve_many(conv_solvers, conv, fetch=False)

        solve_conv()                                       # warm-up (graph capture)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        solve_conv()
        torch.cuda.synchronize()
        t_conv = time.perf_counter() - t0
        outs = [sk.fetch(conv.max_metrics) for sk in conv_solvers]
        rc = dict(reports=[r for o in outs for r in o["reports"]])
        for sk in conv_solvers:
            sk.close()
        s64 = S.Solver(job, max_patches=1, precision="fp64", device=local)
        t64, sr = 0.0, []
        for p in range(nplain):
            s64.set_patches(cut[p:p + 1])
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r64 = s64.run(conv)
            torch.cuda.synchronize()
            t64 += time.perf_counter() - t0
            b = r64["reports"][0].final_metric
            sr.append((rc["reports"][p].final_metric - b) / abs(b))
        s64.close()
        line["converged_reference_settings"] = {
            "value": world * P / t_conv, "unit": UNIT,
            "settings": "MODE_START 5, MODE_STEP 5, MIN_ITER 5, MAX_ITER 500, N_DONE_ITER 3, FTOL 1e-3",
            "iterations_median": float(np.median([r.iterations for r in rc["reports"]])),
            "evaluations_per_patch": float(np.mean([r.n_f_evals + r.n_df_evals for r in rc["reports"]])),
            "plain_fp64_gpu": {"value": nplain / t64, "unit": UNIT, "sample": f"{nplain} patches, per-patch launches"},
            "speedup_chosen_vs_plain": P / t_conv / (nplain / t64),
            "final_metric_signed_rel_vs_fp64": sr,
            "within_1e-5": sum(1 for x in sr if abs(x) <= 1e-5)}
        # CPU baseline: the FP64 restatement on all host cores, one patch
        threads = os.cpu_count() or 1
        ncpu = min(4, P)
        tc, finals_cpu = cpu_port(job, cut, args.iterations, threads, ncpu)
        line["cpu_baseline"] = {"value": ncpu / tc, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{ncpu} patches x {args.iterations} iterations, FP64 restatement "
                                          f"(iterative Stockham FFT), {threads} OpenMP threads over images",
                                "final_metric_rel_diff_gpu_vs_cpu": [abs(reps[p].final_metric - finals_cpu[p]) /
                                                                     abs(finals_cpu[p]) for p in range(ncpu)]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    solver.close()
    for sk in solvers:
        sk.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
