"""Independent scenes packed into one engine (config 4's batched form) give
the same motion as the same scenes stepped one by one, each in its own
engine: every scene keeps its own friction and restitution, and no scene
sees another.  Packing translates each scene, so the runs agree to the
rounding of the translated coordinates (grown over 400 steps of
collisions), not bit for bit; a wrong material or a contact across scenes
would show at 1e-4 r and above."""
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
