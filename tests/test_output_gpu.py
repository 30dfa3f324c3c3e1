"""Output frames (write_frame_bin's files, built on the device and written by
a host thread while the steps go on) and checkpoint/restart snapshots."""
from __future__ import annotations

import os
from dataclasses import replace

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def scene_with_inactive(n=5000, seed=2):
    from gpudem_gb300 import scenes
    sc = scenes.config2_tilted_box(n=n, seed=seed)
    act = np.ones(sc.n, bool)
    act[np.random.default_rng(seed).choice(sc.n, sc.n // 10, replace=False)] = False
    return replace(sc, active=act)


def read_frame(path):
    """write_frame_bin's file (solver_output.cu:259-316)."""
    raw = open(path, "rb").read()
    count = int(np.frombuffer(raw[:4], np.int32)[0])
    pos = np.frombuffer(raw[4:4 + 12 * count], np.float32).reshape(count, 3)
    rad = np.frombuffer(raw[4 + 12 * count:4 + 16 * count], np.float32)
    assert len(raw) == 4 + 16 * count
    return count, pos, rad


def expected_frame(st, r, lf):
    """The reference writer restated on the exported state: active particles
    in pId order, (float)(x * lf) and (float)(r * lf)."""
    a = st["isActive"] == 1
    x = st["x"].reshape(-1, 3)[a]
    return int(a.sum()), (x * lf).astype(np.float32), (np.asarray(r)[a] * lf).astype(np.float32)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_frames_are_write_frame_bin_files(tmp_path, precision):
    from gpudem_gb300 import engine
    sc = scene_with_inactive()
    E = engine.Engine(sc, precision=precision, model="hertz_mindlin")
    E.step(200)
    E.frame_write_async(str(tmp_path), 200, length_factor=2.0)
    E.frames_flush()
    count, pos, rad = read_frame(os.path.join(tmp_path, "result_000000000200.bin"))
    ec, ep, er = expected_frame(E.export(history=False), sc.r, 2.0)
    assert count == ec == sc.n - sc.n // 10
    assert np.array_equal(pos, ep)
    assert np.array_equal(rad, er)


def test_frames_overlap_the_steps(tmp_path):
    """Frames queued every 25 steps without waiting: each file holds the state
    of its own step (checked against a second engine stepping the same run
    and exporting at those steps)."""
    from gpudem_gb300 import engine
    sc = scene_with_inactive()
    A = engine.Engine(sc, precision="mixed", model="hertz_mindlin")
    B = engine.Engine(sc, precision="mixed", model="hertz_mindlin")
    want = {}
    for k in range(1, 9):
        A.step(25)
        A.frame_write_async(str(tmp_path), 25 * k)
        B.step(25)
        want[25 * k] = expected_frame(B.export(history=False), sc.r, 1.0)
    A.frames_flush()
    for step, (ec, ep, er) in want.items():
        count, pos, rad = read_frame(os.path.join(tmp_path, f"result_{step:012d}.bin"))
        assert count == ec
        assert np.array_equal(pos, ep), step
        assert np.array_equal(rad, er), step


def test_frames_report_a_bad_directory(tmp_path):
    from gpudem_gb300 import _lib, engine
    sc = scene_with_inactive(n=1000)
    E = engine.Engine(sc, precision="mixed", model="hertz_mindlin")
    E.frame_write_async(str(tmp_path / "missing"), 1)
    with pytest.raises(_lib.GdemError, match="cannot open"):
        E.frames_flush()
    E.frame_write_async(str(tmp_path), 2)      # the engine goes on
    E.frames_flush()
    assert os.path.exists(os.path.join(tmp_path, "result_000000000002.bin"))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_snapshot_restart_continues_bit_for_bit(tmp_path, precision):
    """Checkpoint after 300 steps of 20,000 colliding spheres over the chute
    (contact histories, some particles inactive), go on 300 steps; a fresh engine loading the checkpoint reaches
    the same state bit for bit, spring histories included."""
    from gpudem_gb300 import engine, scenes
    sc = scenes.config3_helical_chute(n=20_000, n_tri=5_000, v_sigma=0.5)
    act = np.ones(sc.n, bool)
    act[::17] = False
    sc = replace(sc, active=act)
    path = str(tmp_path / "snap.bin")
    A = engine.Engine(sc, precision=precision, model="hertz_mindlin")
    A.step(300)
    A.save_snapshot(path)
    A.step(300)
    a = A.export(history=True)
    B = engine.Engine(sc, precision=precision, model="hertz_mindlin")
    B.load_snapshot(path)
    B.step(300)
    b = B.export(history=True)
    assert A.stats()["steps"] == B.stats()["steps"] == 600
    for key in ("x", "v", "angv", "isActive", "numCont", "indHis", "deltHisx", "deltHisy", "deltHisz",
                "numContWall", "indHisWall", "deltHisxWall"):
        assert np.array_equal(a[key], b[key]), key
    assert int(a["numCont"].sum()) > 100


def test_snapshot_refuses_another_engine(tmp_path):
    from gpudem_gb300 import _lib, engine
    sc = scene_with_inactive(n=1000)
    path = str(tmp_path / "snap.bin")
    engine.Engine(sc, precision="mixed", model="hertz_mindlin").save_snapshot(path)
    E = engine.Engine(sc, precision="fp64", model="hertz_mindlin")
    with pytest.raises(_lib.GdemError, match="precision"):
        E.load_snapshot(path)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_snapshot_with_a_corrupt_history_key_is_refused(tmp_path, precision):
    """A partner id outside [0, n) in a saved snapshot is refused on the host
    before anything is uploaded: the engine that tried to load it goes on
    exactly as an engine that never saw the file."""
    import struct
    from gpudem_gb300 import _lib, engine, scenes
    sc = scenes.config3_helical_chute(n=20_000, n_tri=5_000, v_sigma=0.5)
    path = str(tmp_path / "snap.bin")
    A = engine.Engine(sc, precision=precision, model="hertz_mindlin")
    A.step(900)
    A.save_snapshot(path)
    assert _lib.load().gdem_check_snapshot(path.encode(), A.ntri) == 0
    raw = bytearray(open(path, "rb").read())
    n = sc.n
    state = n * (7 * 16 if precision == "mixed" else 4 * 32)
    counts = np.frombuffer(bytes(raw[56 + state:56 + state + 4 * n]), np.int32)
    assert counts.sum() > 0
    first_key = 56 + state + 4 * n
    raw[first_key:first_key + 4] = struct.pack("<i", n + 7)
    bad = str(tmp_path / "bad.bin")
    open(bad, "wb").write(bytes(raw))
    B = engine.Engine(sc, precision=precision, model="hertz_mindlin")
    C = engine.Engine(sc, precision=precision, model="hertz_mindlin")
    with pytest.raises(_lib.GdemError, match="history partner"):
        B.load_snapshot(bad)
    B.step(50)
    C.step(50)
    b, c = B.export(history=True), C.export(history=True)
    for key in ("x", "v", "angv", "numCont", "indHis", "deltHisx"):
        assert np.array_equal(b[key], c[key]), key


def test_async_position_exports_hold_their_steps():
    """gdem_export_positions_async: each copy holds the positions of the step
    it was queued after, though later steps ran meanwhile."""
    import torch
    from gpudem_gb300 import engine
    sc = scene_with_inactive()
    A = engine.Engine(sc, precision="mixed", model="hertz_mindlin")
    B = engine.Engine(sc, precision="mixed", model="hertz_mindlin")
    bufs = [torch.empty(3 * sc.n, dtype=torch.float64).pin_memory().numpy() for _ in range(3)]
    want = []
    for k in range(3):
        A.step(40)
        A.export_positions_async(bufs[k % 2] if k < 2 else bufs[2])
        B.step(40)
        want.append(B.export_positions())
    A.step(40)
    A.sync()
    for k in range(3):
        assert np.array_equal(bufs[k % 2] if k < 2 else bufs[2], want[k]), k
