"""Failure detection through the C ABI, made on the host (the reference
checks nothing: its CUDA error checks are commented out, device_dem.cu:1230,
and a list overflow only prints, BoundingBox.cu:1146):

* a NaN imported into the velocities sets GDEM_EW_NONFINITE in the step that
  meets it, and gdem_synchronize then returns GDEM_ERR_DEVICE;
* a corrupt or degenerate mesh is refused with GDEM_ERR_ARG before anything
  reaches the device, and the engine keeps the mesh it had;
* a bulk-copy wait of the persistent mixed step kernels that runs out of
  tries (GDEM_TEST_WAIT_TRIES=0: the first wait gives up at once) sets
  GDEM_EW_TIMEOUT; the kernel lets its copies in flight land first, and the
  context stays usable.

No kernel here faults, traps or hangs: every failure is made on the host or
by a wait whose bound is lowered."""
from __future__ import annotations

import os
from dataclasses import replace

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GDEM_ERR_ARG, GDEM_ERR_DEVICE = 1, 6
EW_NONFINITE, EW_TIMEOUT = 0x20, 0x80


def _scene(n=2_000):
    from gpudem_gb300 import scenes
    return scenes.config3_helical_chute(n=n, n_tri=2_000, v_sigma=0.5)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_velocity_sets_nonfinite_and_fails_synchronize(precision):
    from gpudem_gb300 import _lib, engine
    sc = _scene()
    v = np.array(sc.v, np.float64).reshape(-1, 3).copy()
    v[123, 1] = np.nan
    E = engine.Engine(replace(sc, v=v), precision=precision, model="hertz_mindlin")
    E.step(3)
    rc = E.L.gdem_synchronize(E.h)
    assert rc == GDEM_ERR_DEVICE
    st = E.stats()
    assert st["error_word"] & EW_NONFINITE, hex(st["error_word"])
    with pytest.raises(_lib.GdemError, match="GDEM_ERR_DEVICE"):
        E.sync()
    E.close()
    # the process goes on: a clean engine steps without error
    F = engine.Engine(sc, precision=precision, model="hertz_mindlin")
    F.step(3)
    F.sync()
    assert F.stats()["error_word"] == 0


@pytest.mark.parametrize("fault", ["nan_corner", "inf_corner", "repeated_corner", "collinear"])
def test_corrupt_mesh_is_refused_and_the_old_mesh_stays(fault):
    from gpudem_gb300 import _lib, engine
    sc = _scene(n=1_000)
    E = engine.Engine(sc, precision="fp64", model="hertz_mindlin")
    ref = engine.Engine(sc, precision="fp64", model="hertz_mindlin")
    bad = np.array(sc.tris, np.float64).reshape(-1, 3, 3).copy()
    if fault == "nan_corner":
        bad[7, 1, 2] = np.nan
    elif fault == "inf_corner":
        bad[3, 0, 0] = np.inf
    elif fault == "repeated_corner":
        bad[11, 2] = bad[11, 0]
    else:
        bad[5, 2] = 2.0 * bad[5, 1] - bad[5, 0]
    with pytest.raises(_lib.GdemError, match="GDEM_ERR_ARG"):
        E.set_mesh(bad)
    E.ntri = ref.ntri
    E.step(200)
    ref.step(200)
    a, b = E.export(history=True), ref.export(history=True)
    for k in ("x", "v", "numContWall", "indHisWall"):
        assert np.array_equal(a[k], b[k]), k


def test_indexed_mesh_with_bad_ids_is_refused():
    from gpudem_gb300 import _lib, engine, scenes
    sc = _scene(n=500)
    E = engine.Engine(sc, precision="fp64", import_scene=False)
    tris = scenes.box_mesh()
    v = tris.reshape(-1, 3)
    mx, my, mz = v[:, 0], v[:, 1], v[:, 2]
    ti = np.arange(v.shape[0], dtype=np.int32).reshape(-1, 3)
    te = 3 * ti.shape[0] + np.arange(ti.size, dtype=np.int32).reshape(-1, 3)
    d = np.zeros(ti.shape[0])
    E.set_mesh_indexed(mx, my, mz, ti, te, d)  # sound
    for broken in ({"ti": ti[:, ::-1]}, {"ti": ti + 1000}, {"te": -te}, {"d": np.full_like(d, np.nan)}):
        args = dict(ti=ti, te=te, d=d)
        args.update(broken)
        with pytest.raises(_lib.GdemError, match="GDEM_ERR_ARG"):
            E.set_mesh_indexed(mx, my, mz, args["ti"], args["te"], args["d"])


@pytest.mark.parametrize("kernel", [1, 2])  # warp-cooperative, warp-staged
def test_bulk_copy_wait_that_gives_up_reports_timeout(kernel, monkeypatch):
    from gpudem_gb300 import engine
    sc = _scene(n=4_000)
    monkeypatch.setenv("GDEM_TEST_WAIT_TRIES", "0")
    E = engine.Engine(sc, precision="mixed", model="hertz_mindlin", mixed_kernel=kernel)
    monkeypatch.delenv("GDEM_TEST_WAIT_TRIES")
    E.step(1)
    assert E.L.gdem_synchronize(E.h) == GDEM_ERR_DEVICE
    assert E.stats()["error_word"] & EW_TIMEOUT
    E.close()
    # same process, same context: an engine with the normal bound runs clean
    F = engine.Engine(sc, precision="mixed", model="hertz_mindlin", mixed_kernel=kernel)
    F.step(20)
    F.sync()
    assert F.stats()["error_word"] == 0
