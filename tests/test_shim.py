"""The reference-side binding (gpudem_gb300/shim/gdem_device_dem.cu) compiles
against the reference's own headers and include/gdem.h, with the reference's
compile flags (makefile:3-5).  Runs only where the reference checkout exists
(GDEM_REFERENCE_DIR); no GPU needed."""
from __future__ import annotations

import os
import subprocess

import pytest

from conftest import ROOT

REF = os.environ.get("GDEM_REFERENCE_DIR", os.path.join(os.sep, "root", "reference"))


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "device_dem.h")), reason="reference checkout absent")
def test_shim_compiles_against_reference_headers():
    from gpudem_gb300 import _build
    out = os.path.join(_build.OUT, "shim_check.o")
    os.makedirs(_build.OUT, exist_ok=True)
    cmd = [_build._nvcc(), "-O3", "-DUSE_GPU=1", "-fmad=false", "-std=c++17",
           "-gencode", "arch=compute_103a,code=sm_103a", "-I" + REF, "-I" + os.path.join(ROOT, "include"),
           "-c", os.path.join(ROOT, "gpudem_gb300", "shim", "gdem_device_dem.cu"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    nm = subprocess.run(["nm", "-C", out], capture_output=True, text=True).stdout
    assert "gdem_device_dem_verlet_verlet(ParticleSys<DeviceMemory>*, BoundingBox*, TriangleMesh*, BVH*, int, int)" in nm
    assert "gdem_copy_from_device(ParticleSys<DeviceMemory>*, ParticleSys<HostMemory>*)" in nm
    os.remove(out)
