"""bench.py's workload defaults: the chute bed runs 2,000 steps with the mesh
tree rebuilt every step and a 1,000-step position comparison; the periodic
channel runs its 500 steps over a static mesh whose tree is built once."""
from __future__ import annotations

import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402


def test_bed_defaults():
    a = bench.parse_args([])
    assert (a.workload, a.steps, a.error_steps, a.bvh_once, a.n, a.ntri) == ("poured", 2000, 1000, False,
                                                                            1_000_000, 50_000)
    assert a.warmup >= 3


def test_channel_defaults():
    a = bench.parse_args(["--workload", "channel"])
    assert (a.steps, a.error_steps, a.bvh_once, a.n, a.ntri) == (500, 500, True, 10_000_000, 200_000)
    a = bench.parse_args(["--workload", "channel", "--tree-every-step", "--steps", "40"])
    assert (a.steps, a.bvh_once) == (40, False)


def test_warmup_floor():
    assert bench.parse_args(["--warmup", "1"]).warmup == 3


def test_sort_launch_count():
    # up to 32 tiles of 2048 keys the digit scan folds into the scatter kernel
    assert bench.sort_launches(50_768) == 8
    assert bench.sort_launches(32 * 2048) == 8
    assert bench.sort_launches(32 * 2048 + 1) == 12
    assert bench.sort_launches(1_000_000) == 12


def test_reference_arm_loads_the_bed_from_another_process(monkeypatch):
    """The reference arm takes the engine arm's bed from a file that a
    separate process writes, and maps no part of the engine itself."""
    import numpy as np
    from gpudem_gb300 import _lib, scenes
    want = scenes.config1_box_drop()

    def fake_run(cmd, check):
        path = cmd[cmd.index("--save-bed") + 1]
        np.savez(path, **{f: np.asarray(getattr(want, f)) for f in bench._BED_FIELDS
                          if getattr(want, f) is not None})

    monkeypatch.setattr(bench.subprocess, "run", fake_run)
    monkeypatch.setattr(_lib, "_lib", None)
    got = bench.load_bed(bench.parse_args(["--impl", "reference"]))
    for f in bench._BED_FIELDS:
        a, b = getattr(got, f), getattr(want, f)
        assert (a is None and b is None) or np.array_equal(np.asarray(a), np.asarray(b)), f
    assert _lib._lib is None
