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
