"""The 30,000-sphere tilted box as its workload states it: radii uniform in
[0.8, 1.2] x 2 mm, seeded packing in a closed box tilted 30 degrees,
Hertz-Mindlin (E = 5 MPa, nu = 0.3, e = 0.6, mu = 0.4), dt = 2e-6 s,
10,000 steps.

* FP64: the engine against the oracle's FP64 restatement at five
  checkpoints up to step 10,000: positions, velocities, spins, forces,
  torques and tangential histories within 1e-12 relative, and identical
  integer results (activity, contact counts and partners, Verlet and wall
  rows).
* Mixed precision: its per-step force and torque error against FP64.  At
  sampled steps the FP64 run's exact state (with its contact histories) is
  imported into a fresh FP64 engine and a fresh mixed engine, each takes one
  step, and the forces are compared particle by particle.  The error of
  particle i is |f_mixed - f_FP64| / max(|f_FP64|, m_i |g|), the weight being
  the floor for a particle whose contact forces nearly cancel; torques the
  same with m_i |g| r_i.  Bounds, over particles in contact: max 2e-3,
  p99.99 2e-4, median 1e-5.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

from conftest import MAX_NEI, assert_rel, compact_rows

pytestmark = pytest.mark.gpu

CHECKPOINTS = (1, 500, 2500, 6000, 10_000)
FORCE_SAMPLES = (1, 2500, 10_000)
F_MAX, F_P9999, F_MEDIAN = 2e-3, 2e-4, 1e-5


def _history_scene(sc, st):
    """The scene with an exported state (pId order, MAX_NEI-strided rows)."""
    hist = {k: st[k] for k in ("numCont", "indHis", "deltHisx", "deltHisy", "deltHisz", "numContWall",
                               "indHisWall", "deltHisxWall", "deltHisyWall", "deltHiszWall")}
    return replace(sc, x=st["x"].reshape(-1, 3), v=st["v"].reshape(-1, 3), w=st["angv"].reshape(-1, 3),
                   active=st["isActive"].astype(bool), history=hist, hist_stride=MAX_NEI)


def _one_step_forces(sc, precision):
    from gpudem_gb300 import engine
    E = engine.Engine(sc, precision=precision, model="hertz_mindlin", store_forces=True, hist_capacity=32,
                      hist_wall_capacity=16)
    E.step(1)
    st = E.export(history=False, forces=True)
    assert E.stats()["error_word"] == 0
    E.close()
    return st["f"].reshape(-1, 3), st["mom"].reshape(-1, 3)


def _rel_err(a, b, floor):
    num = np.linalg.norm(a - b, axis=1)
    den = np.maximum(np.linalg.norm(b, axis=1), floor)
    return num / den


def test_config2_fp64_matches_oracle_and_mixed_force_error():
    from gpudem_gb300 import engine, scenes
    from oracle import port
    sc = scenes.config2_tilted_box()
    assert sc.n == 30_000
    E = engine.Engine(sc, precision="fp64", model="hertz_mindlin", store_forces=True)
    O = port.OracleScene(sc, model="hertz_mindlin")
    g = float(np.linalg.norm(sc.g))
    done = 0
    report = []
    for c in CHECKPOINTS:
        E.step(c - done)
        O.step(c - done)
        done = c
        st = E.export(history=True, forces=True)
        for nm in ("isActive", "numCont", "numContWall"):
            assert np.array_equal(st[nm], O.get(nm)), (c, nm)
        nc, ncw = st["numCont"], st["numContWall"]
        assert np.array_equal(compact_rows(st["indHis"], nc), compact_rows(O.get("indHis"), nc)), c
        assert np.array_equal(compact_rows(st["indHisWall"], ncw), compact_rows(O.get("indHisWall"), ncw)), c
        nn, nl, nw, wl = E.lists()
        assert np.array_equal(nn, O.get("numNei")) and np.array_equal(nw, O.get("numNeiWall")), c
        assert np.array_equal(compact_rows(nl, nn), compact_rows(O.get("neiList"), nn)), c
        assert np.array_equal(compact_rows(wl, nw), compact_rows(O.get("neiListWall"), nw)), c
        for nm in ("x", "v", "angv", "f", "mom"):
            assert_rel(st[nm], O.get(nm), 1e-12, f"step {c} {nm}")
        for sfx, cnt in (("", nc), ("Wall", ncw)):
            dh = np.stack([compact_rows(st["deltHis" + a + sfx], cnt) for a in "xyz"])
            dho = np.stack([compact_rows(O.get("deltHis" + a + sfx), cnt) for a in "xyz"])
            assert_rel(dh, dho, 1e-12, f"step {c} history{sfx}")
        if c in FORCE_SAMPLES:
            hs = _history_scene(sc, st)
            f64, t64 = _one_step_forces(hs, "fp64")
            fmx, tmx = _one_step_forces(hs, "mixed")
            touching = (st["numCont"] + st["numContWall"]) > 0
            weight = sc.m * g
            ef = _rel_err(fmx, f64, weight)[touching]
            et = _rel_err(tmx, t64, weight * sc.r)[touching]
            row = dict(step=c, n_touching=int(touching.sum()), f_max=float(ef.max()),
                       f_p9999=float(np.quantile(ef, 0.9999)), f_median=float(np.median(ef)),
                       t_max=float(et.max()), t_p9999=float(np.quantile(et, 0.9999)),
                       t_median=float(np.median(et)))
            report.append(row)
            print("config2 mixed force error", row)
    s = E.stats()
    assert s["error_word"] == 0 and s["n_contacts"] > 10_000
    assert E.stats()["rebuilds"] == 1 + O.counter("rebuilds")
    for row in report:
        assert row["n_touching"] > 1000, row
        for q in ("f", "t"):
            assert row[q + "_max"] <= F_MAX, row
            assert row[q + "_p9999"] <= F_P9999, row
            assert row[q + "_median"] <= F_MEDIAN, row
