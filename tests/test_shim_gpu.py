"""The reference-side binding's body (gpudem_gb300/shim/gdem_shim_core.h)
stepping the 100-sphere box drop on the GPU, as main.cu would through
gdem_device_dem_verlet_verlet / gdem_copy_from_device (main.cu:270, :279).

The reference's own headers are not on the GPU host, so
tests/shim_standin.cu gives the binding structs with the reference's member
names and device arrays in its layout (MAX_NEI-strided history rows), filled
from the golden inputs, the BoundingBox values and the welded mesh arrays the
reference itself produced (tests/golden).  The states it copies back must be
the reference CPU path's, bit for bit.  (tests/test_shim.py compiles the
same body against the real headers where the reference checkout exists.)"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import MAX_NEI, ROOT, compact_rows, load_golden

pytestmark = pytest.mark.gpu


def _build_standin():
    from gpudem_gb300 import _build
    lib = _build.build_engine()
    out = os.path.join(_build.OUT, "libshim_standin.so")
    src = os.path.join(ROOT, "tests", "shim_standin.cu")
    core = os.path.join(ROOT, "gpudem_gb300", "shim", "gdem_shim_core.h")
    if _build._stale(out, [src, core, lib]):
        cmd = [_build._nvcc(), *_build.ARCH, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
               "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "gpudem_gb300", "shim"),
               src, "-o", out, "-L" + _build.OUT, "-lgdem", "-Xlinker", "-rpath," + _build.OUT]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-3000:]
    return C.CDLL(out)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def test_binding_steps_the_box_drop_like_the_reference():
    L = _build_standin()
    for f in ("standin_setup", "standin_step", "standin_copy_back", "standin_release"):
        getattr(L, f).restype = C.c_int
    g = load_golden("box_drop_100")
    mesh = dict(np.load(os.path.join(ROOT, "tests", "golden", "meshes.npz")))
    assert np.array_equal(mesh["box_tris"].reshape(-1), g["in_tris"].reshape(-1))
    n = g["in_r"].size
    bd = g["box_d"]
    box9 = np.array([*bd[0:6], bd[6], bd[12], bd[13]], np.float64)  # min, max, dx, skinR, refreshThresh
    x = np.ascontiguousarray(g["in_x"].reshape(-1), np.float64)
    zeros = np.zeros(3 * n)
    arr = {k: np.ascontiguousarray(mesh["box_" + k]) for k in
           ("mx", "my", "mz", "tri_i0", "tri_i1", "tri_i2", "tri_e0", "tri_e1", "tri_e2", "d")}
    for k in ("tri_i0", "tri_i1", "tri_i2", "tri_e0", "tri_e1", "tri_e2"):
        arr[k] = arr[k].astype(np.int32)
    L.standin_setup.argtypes = [C.c_int] + [C.c_void_p] * 7 + [C.c_double, C.c_double] + [C.c_void_p] * 2 + \
        [C.c_int, C.c_int] + [C.c_void_p] * 10
    rc = L.standin_setup(n, _p(x), _p(zeros), _p(zeros), _p(g["in_r"]), _p(g["in_m"]), _p(g["in_k"]),
                         _p(g["in_eta"]), float(g["in_dt"]), float(g["in_mu"]), _p(np.ascontiguousarray(g["in_g"])),
                         _p(box9), arr["mx"].size, arr["d"].size,
                         *[_p(arr[k]) for k in ("mx", "my", "mz", "tri_i0", "tri_i1", "tri_i2", "tri_e0",
                                                 "tri_e1", "tri_e2", "d")])
    assert rc == 0
    H = n * MAX_NEI
    out = {k: np.zeros(3 * n) for k in ("x", "v", "angv")}
    out.update({k: np.zeros(n, np.int32) for k in ("isActive", "numCont", "numContWall")})
    out.update({k: np.zeros(H, np.int32) for k in ("indHis", "indHisWall")})
    out.update({k: np.zeros(H) for k in ("hx", "hy", "hz", "hwx", "hwy", "hwz")})
    done = 0
    compared = 0
    try:
        for c in g["checkpoints"]:
            c = int(c)
            if c > 10000:
                break
            assert L.standin_step(c - done) == 0
            done = c
            assert L.standin_copy_back(*[_p(out[k]) for k in (
                "x", "v", "angv", "isActive", "numCont", "indHis", "hx", "hy", "hz", "numContWall",
                "indHisWall", "hwx", "hwy", "hwz")]) == 0
            tag = f"s{c}"
            for k in ("x", "v", "angv", "isActive", "numCont", "numContWall"):
                assert np.array_equal(out[k], g[f"{tag}_{k}"]), (tag, k)
            nc, ncw = out["numCont"], out["numContWall"]
            assert np.array_equal(compact_rows(out["indHis"], nc), g[f"{tag}_indHis"]), tag
            assert np.array_equal(compact_rows(out["indHisWall"], ncw), g[f"{tag}_indHisWall"]), tag
            dh = np.stack([compact_rows(out[k], nc) for k in ("hx", "hy", "hz")], 1)
            dhw = np.stack([compact_rows(out[k], ncw) for k in ("hwx", "hwy", "hwz")], 1)
            assert np.array_equal(dh, g[f"{tag}_deltHis"]), tag
            assert np.array_equal(dhw, g[f"{tag}_deltHisWall"]), tag
            compared += 1
    finally:
        L.standin_release()
    assert compared >= 6 and done == 10000
