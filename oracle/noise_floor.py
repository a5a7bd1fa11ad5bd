"""Noise floor of converged MOMFBD metrics: the FP64 restatement (the oracle) solved to
convergence twice per patch, once as it is and once with every metric evaluation multiplied by
(1 + sigma * N(0, 1)) -- relative noise of the size of the FP32 evaluation's rounding error
(1e-7 ... 3e-7 against FP64, measured by the GPU parity tests).  The signed relative difference
of the two converged metrics (both evaluated without noise at the final points) is what
rounding of that size alone does to a converged solve of this non-convex problem: the spread
against which the FP32 path's converged metrics are compared with FP64's.

TEST AND STUDY INFRASTRUCTURE ONLY (CPU); the product never imports it.

    python oracle/noise_floor.py --patches 0:24 --sigma 2e-7
prints one JSON line: per-patch clean and noisy metrics, iterations, and the distribution.
Workload: the production batch's patches (225 patches 88 x 88, 36 KL modes, 3 x 12 images,
seeded generator), all modes at once, FTOL 1e-6 (3 consecutive), MIN_ITER 5, MAX_ITER 2000.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import oracle  # noqa: E402


def solve(job, cutout, cfg, sigma, seed, threads):
    op = oracle.OraclePatch(job, threads=threads)
    op.set_images(cutout, None, None)
    M = job.n_modes
    off = np.zeros(job.n_images * M)
    rng = np.random.default_rng(seed)
    n_tot = job.n_images * job.patch_size ** 2

    def f(x):
        v = op.metric(op.cons_reverse_add(x, off))
        return v * (1.0 + sigma * rng.standard_normal()) if sigma > 0 else v

    def df(x, method, mc):
        en = np.zeros(M, np.uint8)
        en[:mc] = 1
        _, g = op.gradient(op.cons_reverse_add(x, off), "vogel" if method == 2 else "fd", en)
        return op.cons_apply(g)

    o = oracle.cg_minimize(job.nullspace.n_free, M, cfg, 1.0 / n_tot ** 2, f, df)
    return op.metric(op.cons_reverse_add(o["x"], off)), o["report"].iterations


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--patches", default="0:8", help="first:last (exclusive) patch indices of the batch")
    ap.add_argument("--sigma", type=float, default=2e-7, help="relative noise of each metric evaluation")
    ap.add_argument("--ftol", type=float, default=1e-6)
    ap.add_argument("--max-iterations", type=int, default=2000)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    import bench
    job, cut = bench.workload(225, 12, 100)
    M = job.n_modes
    cfg = oracle.Cfg(n_initial_modes=M, n_mode_increment=M, max_iterations=args.max_iterations, min_iterations=5,
                     target_iterations=3, fd_first=1, ftol=args.ftol, eps=1e-10, brent_tol=0.1)
    a, b = (int(v) for v in args.patches.split(":"))
    rows = []
    t0 = time.time()
    for p in range(a, b):
        Lc, ic = solve(job, cut[p], cfg, 0.0, 0, args.threads)
        Ln, inn = solve(job, cut[p], cfg, args.sigma, 20261203 + p, args.threads)
        rows.append({"patch": p, "clean": Lc, "noisy": Ln, "it_clean": ic, "it_noisy": inn,
                     "rel": (Ln - Lc) / abs(Lc)})
        print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
    rel = np.array([r["rel"] for r in rows])
    out = {"study": "noise floor of converged metrics (FP64 oracle, relative metric noise)", "sigma": args.sigma,
           "ftol": args.ftol, "patches": f"{a}:{b}", "seconds": time.time() - t0, "threads": args.threads,
           "rel_noisy_minus_clean": {"median": float(np.median(rel)), "abs_median": float(np.median(np.abs(rel))),
                                     "p90_abs": float(np.percentile(np.abs(rel), 90)), "min": float(rel.min()),
                                     "max": float(rel.max()), "noisy_lower": int(np.sum(rel < 0)), "n": int(rel.size),
                                     "within_1e-5": int(np.sum(np.abs(rel) <= 1e-5))},
           "rows": rows}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
