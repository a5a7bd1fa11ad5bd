"""Writes the oracle's golden vectors (tests/golden/oracle_golden.npz): regression fixtures
of the FP64 C restatement on the seeded synthetic workloads, so that a change to the oracle
(which every GPU test compares against) shows up on the CPU.  The reference itself does not build
here, so these pin the restatement to itself, not to redux.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from redux_gb300 import synth  # noqa: E402

OUT = os.path.join(HERE, "oracle_golden.npz")


def cases():
    """(name, workload): the plain 64 x 64 patch, and one 88 x 88 production patch with 4 frames."""
    return [("plain64", synth.workload("plain64")),
            ("production88", synth.workload("production88", n_patches=1, frames=4))]


def compute(name, w):
    job = w.job
    fg = None if w.patches.fixed_gamma is None else w.patches.fixed_gamma[0]
    op = oracle.OraclePatch(job)
    op.set_images(w.patches.cutouts[0], None, fg)
    a = w.patches.alpha_true[0]
    out = {}
    out[f"{name}_gamma"] = op.gamma()
    out[f"{name}_metric"] = np.array([op.metric(a * s) for s in (0.0, 0.5, 1.0)])
    out[f"{name}_grad_vogel"] = op.gradient(a * 0.5, method="vogel")[1]
    out[f"{name}_grad_fd"] = op.gradient(a * 0.5, method="fd")[1]
    out[f"{name}_restore"] = op.restore(a, job.otf_size / 2.0)[:, ::3, ::3]   # every third pixel
    r = op.solve(oracle.default_cfg(max_iterations=5, n_modes=job.n_modes))
    out[f"{name}_solve_metrics"] = r["metrics"]
    out[f"{name}_solve_alpha"] = r["alpha"]
    return out


def main():
    data = {}
    for name, w in cases():
        data.update(compute(name, w))
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT}: {len(data)} arrays")


if __name__ == "__main__":
    main()
