"""Builds libredux_gb300.so in place: every CUDA source for sm_103a with nvcc, in parallel.

No CMake and no torch: the library is a plain C ABI over the CUDA runtime (linked
statically), so the same build runs here and on the GPU host.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libredux_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC"]

CU_SOURCES = ["rdxg_api.cu", "rdxg_inst_common.cu", "rdxg_inst_32.cu", "rdxg_inst_64.cu",
              "rdxg_inst_88.cu", "rdxg_inst_128.cu", "rdxg_noalloc.cu", "rdxg_phase_tc.cu"]
CXX_SOURCES = ["rdxg_host_cg.cpp", "rdxg_setup.cpp"]


def _nvcc():
    n = shutil.which("nvcc")
    if n:
        return n
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(HERE, "..", "include", "rdxg.h"))
    return hs


def build(verbose: bool = False, force: bool = False) -> str:
    """Compiles what changed (everything with force).  RDXG_NVCC_FLAGS adds nvcc options,
    e.g. -DRDXG_EVAL_THREADS=384 for the block size of the evaluation kernels."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    extra = os.environ.get("RDXG_NVCC_FLAGS", "").split()
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append([nvcc] + NVCC_FLAGS + extra + ["-c", s, "-o", o])
    cxx = os.environ.get("CXX", "g++")
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append([cxx] + CXX_FLAGS + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _newer(LIB, objs):
        run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
