"""The 30,000-sphere tilted box (radii uniform in [0.8, 1.2] x 2 mm, seeded
packing in a closed box tilted 30 degrees, Hertz-Mindlin E = 5 MPa,
nu = 0.3, e = 0.6, mu = 0.4, dt = 2e-6 s, 10,000 steps), two ways:

* as stated: the packing dropped from rest.  10,000 steps of 2e-6 s are
  0.02 s of free fall (2 mm), so few contacts form; the FP64 engine must
  match the oracle's FP64 restatement at every checkpoint.
* landed: the same spheres first poured into the box on the GPU (mixed
  precision, dt = 2e-5 s, restitution 0.1), then from that state (positions,
  velocities, spins; springs start empty) the stated material and time step
  for 10,000 steps, FP64 engine against the oracle, with a dense contact
  network.

At every checkpoint: positions, velocities, spins, forces, torques and
tangential histories within 1e-12 relative, identical integer results
(activity, contact counts and partners, Verlet and wall rows), the same
rebuild count.

On the landed bed, the mixed mode's per-step force and torque error against
FP64: at sampled steps the FP64 run's exact state (with its contact
histories) is imported into a fresh FP64 engine and a fresh mixed engine,
each takes one step, and the forces are compared particle by particle.  The
error of particle i is |f_mixed - f_FP64| / max(|f_FP64|, m_i |g|), the
weight being the floor for a particle whose contact forces nearly cancel;
torques the same with m_i |g| r_i.  Bounds, over particles in contact:
p99.99 2e-4, median 1e-5, and at most 3 particles in 30,000 above 1e-3.
Those few are contacts at the Coulomb cap: the reference's law adds the
dashpot term only while a contact sticks (cpu_dem.cu:783-951), so a contact
within rounding of |f_t| = mu |f_n| can stick in one precision and slip in
the other, a jump of the damping force (7 % of one particle's force was
seen).  The largest error is reported, not bounded.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

from conftest import MAX_NEI, assert_rel, compact_rows

pytestmark = pytest.mark.gpu

CHECKPOINTS = (1, 500, 2500, 6000, 10_000)
FORCE_SAMPLES = (1, 2500, 10_000)
F_P9999, F_MEDIAN = 2e-4, 1e-5
F_FLIP, N_FLIP = 1e-3, 3


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


def _landed_scene(sc):
    """The spheres poured into the box and at rest, springs empty."""
    from gpudem_gb300 import scenes
    landed = scenes.settle_scene(sc, steps=24_000, dt=2e-5, e=0.1, chunk=24_000)
    keep = landed.active.astype(bool)
    return replace(sc, x=landed.x[keep], v=landed.v[keep], w=landed.w[keep], r=sc.r[keep], m=sc.m[keep],
                   k=sc.k[keep], eta=sc.eta[keep], history=None, hist_stride=0, active=None,
                   inlet_lo=landed.inlet_lo, inlet_hi=landed.inlet_hi, box=landed.box)


def _run_against_oracle(sc, force_samples=()):
    from gpudem_gb300 import engine
    from oracle import port
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
            if int(cnt.sum()) == 0:
                continue
            dh = np.stack([compact_rows(st["deltHis" + a + sfx], cnt) for a in "xyz"])
            dho = np.stack([compact_rows(O.get("deltHis" + a + sfx), cnt) for a in "xyz"])
            assert_rel(dh, dho, 1e-12, f"step {c} history{sfx}")
        if c in force_samples:
            hs = _history_scene(sc, st)
            f64, t64 = _one_step_forces(hs, "fp64")
            fmx, tmx = _one_step_forces(hs, "mixed")
            touching = (st["numCont"] + st["numContWall"]) > 0
            weight = sc.m * g
            ef = _rel_err(fmx, f64, weight)[touching]
            et = _rel_err(tmx, t64, weight * sc.r)[touching]
            row = dict(step=c, n_touching=int(touching.sum()), f_max=float(ef.max()),
                       n_above=int((ef > F_FLIP).sum() + (et > F_FLIP).sum()),
                       f_p9999=float(np.quantile(ef, 0.9999)), f_median=float(np.median(ef)),
                       t_max=float(et.max()), t_p9999=float(np.quantile(et, 0.9999)),
                       t_median=float(np.median(et)))
            report.append(row)
            print("config2 mixed force error", row)
    s = E.stats()
    assert s["error_word"] == 0
    assert s["rebuilds"] == 1 + O.counter("rebuilds")
    return s, report


def test_config2_as_stated_fp64_matches_oracle():
    from gpudem_gb300 import scenes
    sc = scenes.config2_tilted_box()
    assert sc.n == 30_000
    _run_against_oracle(sc)


def test_config2_landed_fp64_matches_oracle_and_mixed_force_error():
    from gpudem_gb300 import scenes
    sc = _landed_scene(scenes.config2_tilted_box())
    assert sc.n >= 29_900
    s, report = _run_against_oracle(sc, FORCE_SAMPLES)
    assert s["n_contacts"] > 3 * sc.n
    assert len(report) == len(FORCE_SAMPLES)
    for row in report:
        assert row["n_touching"] > 0.9 * sc.n, row
        assert row["n_above"] <= 2 * N_FLIP, row
        for q in ("f", "t"):
            assert row[q + "_p9999"] <= F_P9999, row
            assert row[q + "_median"] <= F_MEDIAN, row
