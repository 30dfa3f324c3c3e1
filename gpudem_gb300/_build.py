"""In-tree build of libgdem.so (the engine) and liboracle.so (the CPU
restatement used only by tests and the CPU-baseline leg of bench.py).

Each CUDA translation unit is compiled for sm_103a only, in parallel, then
linked into one shared library under gpudem_gb300/_build/.  Kernels whose
FP64 results must match the reference CPU build are compiled with
-fmad=false (no multiply-add contraction), matching the reference makefile
(makefile:5); the mixed-precision kernels keep contraction on.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgdem.so")
ORACLE_SRC = os.path.join(ROOT, "oracle", "gdem_oracle.cpp")
ORACLE_LIB = os.path.join(OUT, "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I" + os.path.join(ROOT, "include")]
# translation unit -> whether FP64 contraction must stay off
UNITS = {
    "gdem_api.cu": True,
    "gdem_rebuild.cu": True,
    "gdem_step_fp64.cu": True,
    "gdem_step_mixed.cu": False,
    "gdem_stats.cu": True,
    "gdem_noalloc.cu": True,
    "gdem_output.cu": True,
    "gdem_init.cu": True,
    "gdem_settings.cpp": True,
}
# the mixed-precision step: FP32 contact law with the hardware's approximate
# reciprocal and square root (its error is measured against the FP64 mode)
EXTRA = {"gdem_step_mixed.cu": ["-prec-div=false", "-prec-sqrt=false"]}


def _nvcc():
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if os.path.exists(cand) else "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.exists(s) and os.path.getmtime(s) > t for s in sources)


def build_engine(verbose=False, ptxas_info=False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(ROOT, "include", "gdem.h"))
    nvcc = _nvcc()
    objs = []
    jobs = []
    for unit, nofma in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OUT, os.path.splitext(unit)[0] + ".o")
        objs.append(obj)
        if _stale(obj, [src, *headers, __file__]):
            cmd = [nvcc, *ARCH, *COMMON, "-fmad=false" if nofma else "-fmad=true", *EXTRA.get(unit, []), "-c", src,
                   "-o", obj]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out, file=sys.stderr)
    if _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", *objs, "-o", LIB, "-lcudart"])
    return LIB


def build_oracle() -> str:
    """Compile the CPU restatement (test infrastructure) with the host
    compiler, no FMA contraction, OpenMP for the timed CPU baseline."""
    os.makedirs(OUT, exist_ok=True)
    if _stale(ORACLE_LIB, [ORACLE_SRC, __file__]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-fno-fast-math", ORACLE_SRC, "-o", ORACLE_LIB])
    return ORACLE_LIB


def build_all(verbose=False):
    return build_engine(verbose), build_oracle() if os.path.exists(ORACLE_SRC) else None


if __name__ == "__main__":
    print(build_all(verbose="-v" in sys.argv))
