"""Independent scenes packed into one engine (config 4's batched form) give
the same motion as the same scenes stepped one by one, each in its own
engine: every scene keeps its own friction and restitution, and no scene
sees another.  Packing translates each scene, so the runs agree to the
rounding of the translated coordinates (grown over 400 steps of
collisions), not bit for bit; a wrong material or a contact across scenes
would show at 1e-4 r and above.

The packed scene itself is pinned to the oracle: its FP64 restatement with
per-particle friction and restitution steps the same packed scene, and the
FP64 engine must match it bit for bit in its integer results and to 1e-12
in its states, forces and histories."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_packed_scenes_match_separate_engines(precision):
    from gpudem_gb300 import engine, scenes
    scs = scenes.config4_batched(n_scenes=6, seed=7, n_min=300, n_max=3000)
    for sc in scs:   # start them moving so contacts form quickly
        rng = np.random.default_rng(sc.n)
        sc.v = rng.normal(0.0, 0.3, (sc.n, 3))
    packed, offs, starts = scenes.pack_scenes(scs)
    steps = 400
    P = engine.Engine(packed, precision=precision, model="hertz_mindlin")
    P.step(steps)
    xp = P.export(history=False)["x"].reshape(-1, 3)
    sp = P.stats()
    P.close()
    assert sp["error_word"] == 0
    n_contacts = 0
    for s, sc in enumerate(scs):
        E = engine.Engine(sc, precision=precision, model="hertz_mindlin")
        E.step(steps)
        xs = E.export(history=False)["x"].reshape(-1, 3)
        st = E.stats()
        E.close()
        n_contacts += st["n_contacts"] + st["n_wall_contacts"]
        d = np.abs((xp[starts[s]:starts[s + 1]] - offs[s]) - xs)
        tol = (1e-7 if precision == "fp64" else 1e-5) * float(sc.r.min())
        assert d.max() <= tol, (s, float(d.max()))
    assert n_contacts > 100


def test_packed_scenes_match_the_oracle_fp64():
    from conftest import assert_rel, compact_rows
    from gpudem_gb300 import engine, scenes
    from oracle import port
    scs = scenes.config4_batched(n_scenes=8, seed=9, n_min=300, n_max=4000)
    for sc in scs:
        rng = np.random.default_rng(sc.n + 1)
        sc.v = rng.normal(0.0, 0.3, (sc.n, 3))
    packed, offs, starts = scenes.pack_scenes(scs)
    assert len(set(np.round(packed.mu_p, 12))) == 8
    E = engine.Engine(packed, precision="fp64", model="hertz_mindlin", store_forces=True)
    O = port.OracleScene(packed, model="hertz_mindlin")
    done = 0
    for c in (1, 100, 600):
        E.step(c - done)
        O.step(c - done)
        done = c
        st = E.export(history=True, forces=True)
        for nm in ("isActive", "numCont", "numContWall"):
            assert np.array_equal(st[nm], O.get(nm)), (c, nm)
        nc = st["numCont"]
        assert np.array_equal(compact_rows(st["indHis"], nc), compact_rows(O.get("indHis"), nc)), c
        for nm in ("x", "v", "angv", "f", "mom"):
            assert_rel(st[nm], O.get(nm), 1e-12, f"packed step {c} {nm}")
        dh = np.stack([compact_rows(st["deltHis" + a], nc) for a in "xyz"])
        dho = np.stack([compact_rows(O.get("deltHis" + a), nc) for a in "xyz"])
        assert_rel(dh, dho, 1e-12, f"packed step {c} history")
    s = E.stats()
    assert s["error_word"] == 0 and s["n_contacts"] > 200
    assert s["rebuilds"] == 1 + O.counter("rebuilds")
