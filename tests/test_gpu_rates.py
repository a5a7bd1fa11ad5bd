"""The FP64 issue cost this GPU's per-round kernels are designed around (marked gpu): a warp's
FP64 FMA takes tens of cycles and a double-to-float conversion more, against about one for
FP32, and masking all lanes but one does not make them cheaper.  That is why the solver
kernel stages its data and forms alphaEff in FP32, and why the reduction and the adjoint's
projection add their partial sums as float-float numbers (tests/cuda/fp64_rate.cu prints the
figures: cycles per warp instruction)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _nvcc():
    n = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(n):
        pytest.skip("nvcc not found")
    return n


def test_fp64_issue_cost(tmp_path):
    exe = str(tmp_path / "fp64_rate")
    subprocess.run([_nvcc(), "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe,
                    os.path.join(HERE, "cuda", "fp64_rate.cu")], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    print(out)
    cyc = {}
    for line in out.split("\n"):
        if line.strip():
            kind, lanes, c = line.split()
            cyc[(kind, int(lanes))] = float(c)
    ffma = cyc[("ffma", 32)]
    # FP64 far slower than FP32, and no cheaper with one lane active
    assert cyc[("dfma", 32)] > 16 * ffma
    assert cyc[("f2f", 32)] > cyc[("dfma", 32)]
    assert cyc[("dfma", 1)] > 0.8 * cyc[("dfma", 32)]
