"""Periodic x (gdem_desc.periodic_x): the box's x extent is one period.

No reference counterpart exists (its box deactivates what leaves it), so the
oracle's periodic restatement is checked by a size-independent property --
a pair colliding across the period's faces moves exactly like the same pair
colliding inside -- and the engine is checked against the oracle: FP64
bit-identical, mixed precision within the position tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

from gpudem_gb300 import scenes

POS_TOL_RMIN = 1e-4


def pair_scene(xc):
    """Two spheres (r = 1 mm) approaching head-on-ish at 0.5 m/s each, their
    mid-point at x = xc, in a channel of period 0.02 m."""
    r = 1e-3
    m = scenes.sphere_mass(2500.0, np.full(2, r))
    k = np.full(2, scenes.stiffness_from_E(5e6, r))
    x = np.array([[xc - 1.5e-3, 0.0, 0.0], [xc + 1.5e-3, 4e-4, 0.0]])
    v = np.array([[0.5, 0.0, 0.1], [-0.5, 0.0, 0.0]])
    lo, hi = np.array([-0.01, -0.01, -0.01]), np.array([0.01, 0.01, 0.01])
    sc = scenes.Scene(x=x, r=np.full(2, r), m=m, k=k, eta=scenes.eta_const(k, 0.5), mu=0.5, dt=2e-6,
                      tris=np.zeros((0, 3, 3)), inlet_lo=lo, inlet_hi=hi, g=np.zeros(3), v=v, w=np.zeros((2, 3)),
                      E=5e6, nu=0.3, e=0.5, mu_roll=0.05, box=(lo, hi), periodic_x=True)
    return sc


def wrap(x, lo=-0.01, L=0.02):
    return (x - lo) % L + lo


def test_oracle_pair_across_the_faces_moves_like_the_pair_inside():
    from oracle.port import OracleScene
    inside = OracleScene(pair_scene(0.0), model="hertz_mindlin")
    seam = OracleScene(pair_scene(0.01), model="hertz_mindlin")   # mid-point on the x faces
    for _ in range(5):
        inside.step(400)
        seam.step(400)
        xa, xb = inside.get("x").reshape(-1, 3), seam.get("x").reshape(-1, 3)
        assert np.all(xb[:, 0] >= -0.01) and np.all(xb[:, 0] < 0.01)
        shifted = xa.copy()
        shifted[:, 0] = wrap(xa[:, 0] + 0.01)
        d = shifted - xb
        d[:, 0] = (d[:, 0] + 0.01) % 0.02 - 0.01      # compare on the circle
        assert np.abs(d).max() < 1e-12
        for name in ("v", "angv"):
            assert np.allclose(inside.get(name), seam.get(name), rtol=1e-9, atol=1e-12), name
    # they did collide, and spun up (friction)
    assert np.abs(inside.get("angv")).max() > 1.0
    assert inside.get("v")[0] < 0.5


def test_oracle_channel_wraps_particles():
    from oracle.port import OracleScene
    sc = scenes.config5_periodic_channel(n=3000, length=0.1, width=0.05, n_tri=2000, v_drift=1.0, dt=5e-6)
    o = OracleScene(sc, model="hertz_mindlin")
    x0 = o.get("x").reshape(-1, 3).copy()
    o.step(1500)
    x = o.get("x").reshape(-1, 3)
    assert o.get("isActive").sum() == sc.n
    assert np.all(x[:, 0] >= -0.05) and np.all(x[:, 0] < 0.05)
    assert int((np.abs(x[:, 0] - x0[:, 0]) > 0.05).sum()) > 50        # crossed a face


def test_triangles_must_be_narrower_than_a_quarter_period():
    sc = scenes.config5_periodic_channel(n=100, length=0.1, width=0.05, n_tri=200)
    tx = sc.tris[:, :, 0]
    assert (tx.max(1) - tx.min(1)).max() < 0.025


# ---------------------------------------------------------------- GPU

def channel(n=5000):
    return scenes.config5_periodic_channel(n=n, length=0.1, width=0.05, n_tri=2000, v_drift=1.0, dt=5e-6)


@pytest.mark.gpu
def test_periodic_fp64_engine_is_the_oracle():
    from gpudem_gb300 import engine
    from oracle.port import OracleScene
    sc = channel()
    o = OracleScene(sc, model="hertz_mindlin")
    e = engine.Engine(sc, precision="fp64", model="hertz_mindlin")
    for _ in range(4):
        o.step(500)
        e.step(500)
        d = e.export(history=False)
        for name in ("x", "v", "angv"):
            assert np.array_equal(o.get(name), d[name]), name
    assert e.stats()["error_word"] == 0
    x0 = sc.x
    assert int((np.abs(d["x"].reshape(-1, 3)[:, 0] - x0[:, 0]) > 0.05).sum()) > 50


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_periodic_mixed_close_to_fp64(kernel):
    from gpudem_gb300 import engine
    sc = channel()
    a = engine.Engine(sc, precision="fp64", model="hertz_mindlin")
    b = engine.Engine(sc, precision="mixed", model="hertz_mindlin", mixed_kernel=kernel)
    a.step(1000)
    b.step(1000)
    xa, xb = a.export_positions().reshape(-1, 3), b.export_positions().reshape(-1, 3)
    d = xa - xb
    d[:, 0] = (d[:, 0] + 0.05) % 0.1 - 0.05
    err = np.linalg.norm(d, axis=1).max() / float(sc.r.min())
    print(f"periodic channel, kernel {kernel}: |x_mixed - x_fp64| max {err:.2e} r_min after 1000 steps")
    assert err <= POS_TOL_RMIN
    assert b.stats()["error_word"] == 0
    assert a.stats()["rebuilds"] == b.stats()["rebuilds"]
