"""Hertz-Mindlin (with rolling resistance) against the oracle's FP64
restatement, and the mixed-precision mode against the FP64 engine.

Hertz-Mindlin is not in the reference: its parity is against the oracle's
restatement of the published law (oracle/gdem_oracle.cpp), bit for bit in
FP64.  The mixed mode has no bit-level counterpart: its error is measured
against the FP64 engine on the same inputs, with the tolerances written here.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_rel, compact_rows

pytestmark = pytest.mark.gpu

# mixed-precision acceptance: positions after 1000 steps within 1e-4 r_min of
# FP64; kinetic energy, coordination number and packing fraction within 0.5 %
POS_TOL_RMIN = 1e-4
OBS_RTOL = 5e-3


def _hm_scene(n, seed, mu_roll=0.05):
    from gpudem_gb300 import scenes
    rng = np.random.default_rng(seed)
    r0 = 2e-3
    radii = r0 * rng.uniform(0.8, 1.2, n)
    half = 0.1
    s = half / 1.37
    lo, hi = np.array([-s, -s, -s]), np.array([s, s, s])
    x = scenes.lattice_packing(n, radii, lo, hi, rng, gap=0.02)
    m = scenes.sphere_mass(2500.0, radii)
    k = np.full(n, 2000.0)
    return scenes.Scene(x=x, r=radii, m=m, k=k, eta=scenes.eta_const(k, 0.6), mu=0.4, dt=2e-6,
                        tris=scenes.tilted_box_mesh(half, 30.0, 2), inlet_lo=lo, inlet_hi=hi,
                        v=rng.normal(0.0, 0.5, (n, 3)), w=rng.normal(0.0, 40.0, (n, 3)),
                        E=5e6, nu=0.3, e=0.6, mu_roll=mu_roll)


@pytest.mark.parametrize("mu_roll", [0.0, 0.05])
def test_hertz_mindlin_fp64_matches_oracle(mu_roll):
    from gpudem_gb300 import engine
    from oracle import port
    sc = _hm_scene(20_000, seed=31, mu_roll=mu_roll)
    E = engine.Engine(sc, model="hertz_mindlin", store_forces=True)
    O = port.OracleScene(sc, model="hertz_mindlin")
    done = 0
    for c in (1, 50, 400):
        E.step(c - done)
        O.step(c - done)
        done = c
        st = E.export(history=True, forces=True)
        assert np.array_equal(st["isActive"], O.get("isActive"))
        nc, ncw = st["numCont"], st["numContWall"]
        assert np.array_equal(nc, O.get("numCont")) and np.array_equal(ncw, O.get("numContWall"))
        assert np.array_equal(compact_rows(st["indHis"], nc), compact_rows(O.get("indHis"), nc))
        for nm in ("x", "v", "angv", "f", "mom"):
            assert_rel(st[nm], O.get(nm), 1e-12, f"HM step {c} {nm}")
        dh = np.stack([compact_rows(st["deltHis" + a], nc) for a in "xyz"])
        dho = np.stack([compact_rows(O.get("deltHis" + a), nc) for a in "xyz"])
        assert_rel(dh, dho, 1e-12, f"HM step {c} history")
    s = E.stats()
    assert s["error_word"] == 0 and s["n_contacts"] > 500


@pytest.mark.parametrize("model", ["linear", "hertz_mindlin"])
def test_mixed_close_to_fp64_small(model):
    """20k spheres, 300 steps: mixed positions stay within 1e-4 r_min of FP64."""
    from gpudem_gb300 import engine
    sc = _hm_scene(20_000, seed=41)
    A = engine.Engine(sc, precision="fp64", model=model)
    B = engine.Engine(sc, precision="mixed", model=model)
    A.step(300)
    B.step(300)
    xa = A.export(history=False)["x"]
    xb = B.export(history=False)["x"]
    err = np.max(np.abs(xa - xb))
    assert err <= POS_TOL_RMIN * sc.r.min(), f"max position error {err:.3e} m"
    sa, sb = A.stats(), B.stats()
    assert sb["error_word"] == 0
    assert abs(sb["kinetic_energy"] - sa["kinetic_energy"]) <= OBS_RTOL * sa["kinetic_energy"]


def test_mixed_history_keys_follow_reorders():
    """Mixed mode keys its contact history by storage index and remaps the
    keys when a rebuild reorders the particles; exported, the keys are pIds
    and the rows match the FP64 engine's (same contacts, encounter order)."""
    from gpudem_gb300 import engine
    sc = _hm_scene(20_000, seed=43)
    A = engine.Engine(sc, precision="fp64", model="hertz_mindlin")
    B = engine.Engine(sc, precision="mixed", model="hertz_mindlin")
    for E in (A, B):
        E.step(60)
        E.rebuild()          # reorder with live histories
        E.step(60)
        E.rebuild()
        E.step(30)
    ha, hb = A.export(history=True), B.export(history=True)
    assert B.stats()["error_word"] == 0
    assert np.array_equal(ha["numCont"], hb["numCont"])
    assert np.array_equal(compact_rows(ha["indHis"], ha["numCont"]), compact_rows(hb["indHis"], hb["numCont"]))
    assert int(ha["numCont"].sum()) > 300


def test_mixed_kernels_rebuild_with_fp64_while_pouring():
    """300,000 spheres poured into the chute at dt = 2e-5 s, so the lists are
    rebuilt every few steps.  Every mixed step kernel rebuilds at the steps
    FP64 does: the persistent kernels integrate many particles per thread, and
    every particle's refresh vote counts.  The three kernels step
    bit-identical trajectories, and a repeat gives the same bits, with the
    inner rows or the list rows scanned."""
    from dataclasses import replace
    from gpudem_gb300 import engine, scenes
    sc = replace(scenes.config3_chute_pour(n=300_000), dt=2e-5, e=0.1)
    kw = dict(model="hertz_mindlin", hist_capacity=32, hist_wall_capacity=16)

    def run(precision, **k):
        E = engine.Engine(sc, precision=precision, **kw, **k)
        E.step(600)
        x = E.export_positions()
        st = E.stats()
        E.close()
        assert st["error_word"] == 0
        return x, st["rebuilds"]

    _, rf = run("fp64")
    runs = [run("mixed", mixed_kernel=k) for k in (1, 2, 3, 1)]
    # the step scanning the list rows instead of the inner rows
    runs += [run("mixed", mixed_kernel=k, inner_skin=-1.0) for k in (1, 3)]
    print(f"pour, rebuilds in 600 steps: fp64 {rf}, mixed kernels {[r for _, r in runs]}")
    assert rf >= 10
    for x, rb in runs:
        assert abs(rb - rf) <= 1
        assert np.array_equal(x, runs[0][0])


def test_mixed_error_on_the_poured_bed():
    """The benchmark workload: 1M lognormal spheres poured into the helical
    chute and settled (about 4.6 contacts per sphere), Hertz-Mindlin, the
    LBVH rebuilt every step.  After 1000 steps every sphere of the mixed run
    is within 1e-4 r_min of the FP64 run, and kinetic energy, coordination
    number and packing fraction agree to 0.5 %."""
    from gpudem_gb300 import engine, scenes
    sc = scenes.settle_scene(scenes.config3_chute_pour(n=1_000_000), steps=12_000)
    kw = dict(model="hertz_mindlin", hist_capacity=32, bvh_every_step=True)
    A = engine.Engine(sc, precision="fp64", **kw)
    A.step(1000)
    xa = A.export_positions()
    sa = A.stats()
    A.close()
    B = engine.Engine(sc, precision="mixed", **kw)
    B.step(1000)
    xb = B.export_positions()
    sb = B.stats()
    B.close()
    e = np.linalg.norm((xa - xb).reshape(-1, 3), axis=1)
    rmin = float(sc.r.min())
    print(f"poured bed, |x_mixed - x_fp64| / r_min after 1000 steps: max {e.max() / rmin:.2e}, "
          f"p99.99 {np.percentile(e, 99.99) / rmin:.2e}; contacts/sphere {sa['coordination']:.3f}")
    assert sa["coordination"] > 3.0
    assert e.max() <= POS_TOL_RMIN * rmin
    assert sb["error_word"] == 0
    for key in ("kinetic_energy", "packing_fraction", "coordination"):
        assert abs(sb[key] - sa[key]) <= OBS_RTOL * abs(sa[key]), key


def test_mixed_error_at_benchmark_size():
    """1M lognormal spheres on a loose lattice over the helical chute,
    Hertz-Mindlin, seeded random velocities so collisions happen: after 1000
    steps every sphere of the mixed run is within 1e-4 r_min of the FP64 run,
    and kinetic energy, coordination number and packing fraction agree to
    0.5 %."""
    from gpudem_gb300 import engine, scenes
    sc = scenes.config3_helical_chute(n=1_000_000, v_sigma=0.5)
    A = engine.Engine(sc, precision="fp64", model="hertz_mindlin")
    A.step(1000)
    xa = A.export(history=False)["x"]
    sa = A.stats()
    A.close()
    B = engine.Engine(sc, precision="mixed", model="hertz_mindlin")
    B.step(1000)
    xb = B.export(history=False)["x"]
    sb = B.stats()
    B.close()
    e = np.linalg.norm((xa - xb).reshape(-1, 3), axis=1)
    rmin = float(sc.r.min())
    q = {p_: float(np.percentile(e, p_)) / rmin for p_ in (50, 99, 99.99)}
    print(f"|x_mixed - x_fp64| / r_min after 1000 steps: median {q[50]:.2e}, p99 {q[99]:.2e}, "
          f"p99.99 {q[99.99]:.2e}, max {e.max() / rmin:.2e}, above 1e-4: {int((e > 1e-4 * rmin).sum())}; "
          f"contacts fp64 {sa['n_contacts']} mixed {sb['n_contacts']}")
    assert q[99.99] <= POS_TOL_RMIN
    assert e.max() <= POS_TOL_RMIN * rmin
    for key in ("kinetic_energy", "packing_fraction"):
        assert abs(sb[key] - sa[key]) <= OBS_RTOL * abs(sa[key]), key
    assert abs(sb["coordination"] - sa["coordination"]) <= OBS_RTOL * max(sa["coordination"], 1e-9) + 1e-6
