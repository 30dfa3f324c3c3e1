"""Shared test helpers.  Tests marked ``gpu`` need a GB300 and the built
libgdem.so; everything else runs on the CPU."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
MAX_NEI = 100


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def scene_from_golden(g):
    """Rebuild the exact Scene a golden fixture was generated from."""
    from gpudem_gb300.scenes import Scene
    return Scene(x=g["in_x"], r=g["in_r"], m=g["in_m"], k=g["in_k"], eta=g["in_eta"],
                 mu=float(g["in_mu"]), dt=float(g["in_dt"]), tris=g["in_tris"],
                 inlet_lo=g["in_inlet_lo"], inlet_hi=g["in_inlet_hi"], g=g["in_g"],
                 v=g.get("in_v"), w=g.get("in_w"), skin=float(g["in_skin"]),
                 refresh=float(g["in_refresh"]))


def compact_rows(rows, counts, stride=MAX_NEI):
    rows = np.asarray(rows).reshape(-1, stride)
    if counts.size == 0:
        return rows[:0, 0]
    return np.concatenate([rows[i, :counts[i]] for i in range(counts.size)])


def assert_rel(a, b, rtol, what):
    """max |a-b| <= rtol * max |b| (array-wise relative error)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    scale = np.max(np.abs(b)) if b.size else 0.0
    err = np.max(np.abs(a - b)) if b.size else 0.0
    assert err <= rtol * max(scale, 1e-300), f"{what}: max abs err {err:.3e} (scale {scale:.3e}, rtol {rtol})"
