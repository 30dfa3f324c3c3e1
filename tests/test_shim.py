"""The reference-side binding (gpudem_gb300/shim/gdem_device_dem.cu) compiles
against the reference's own headers and include/gdem.h, with the reference's
compile flags (makefile:3-5).  Runs only where the reference checkout exists
(oracle/build_ref.sh --where); no GPU needed.  Its body,
gpudem_gb300/shim/gdem_shim_core.h, is run on the GPU by
tests/test_shim_gpu.py through stand-in structs with the same members."""
from __future__ import annotations

import os
import subprocess

import pytest

from conftest import ROOT


def _reference_dir():
    from oracle.refharness import reference_dir
    return reference_dir()


def test_shim_compiles_against_reference_headers():
    ref = _reference_dir()
    if ref is None:
        pytest.skip("reference checkout absent")
    from gpudem_gb300 import _build
    out = os.path.join(_build.OUT, "shim_check.o")
    os.makedirs(_build.OUT, exist_ok=True)
    cmd = [_build._nvcc(), "-O3", "-DUSE_GPU=1", "-fmad=false", "-std=c++17",
           "-gencode", "arch=compute_103a,code=sm_103a", "-I" + ref, "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "gpudem_gb300", "shim"),
           "-c", os.path.join(ROOT, "gpudem_gb300", "shim", "gdem_device_dem.cu"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    nm = subprocess.run(["nm", "-C", out], capture_output=True, text=True).stdout
    assert "gdem_device_dem_verlet_verlet(ParticleSys<DeviceMemory>*, BoundingBox*, TriangleMesh*, BVH*, int, int)" in nm
    assert "gdem_copy_from_device(ParticleSys<DeviceMemory>*, ParticleSys<HostMemory>*)" in nm
    os.remove(out)
