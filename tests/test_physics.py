"""Physics-level checks of the contact law and integrator, the comparisons the
reference itself keeps (it has no numeric tests):

* the LIGGGHTS 3.8.0 two-sphere collision (liggghtsCases/testCases/in.collision,
  dump.txt), against the fixture tests/golden/liggghts_collision.json;
* python/compareDrop.py (restitution of a bouncing sphere), python/compareRoll.py
  (slip and roll down an incline) and python/compareCollision.py (Walton's
  oblique impact in its sticking regime).

The CPU tests run the oracle (the FP64 restatement of the reference's CPU
path); the gpu tests run the engine through the C ABI, FP64 (bit-identical to
the oracle) and mixed precision.

Spin sign: the reference's contact normal points toward particle i
(device_dem.cu:589), but the relative surface velocity (device_dem.cu:832) and
the torque (device_dem.cu:716) use it as if it pointed away from i.  The two
sign errors cancel in positions and velocities; the stored angular velocity is
the negative of the physical one, so it is compared with LIGGGHTS' omega
negated.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np
import pytest

from gpudem_gb300 import scenes

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "liggghts_collision.json")
FRAMES = (18000, 19000, 20000, 22000, 50000, 100000)
# agreement with LIGGGHTS: velocities to 1e-4 m/s (0.01 % of the impact
# speed), positions to 1e-4 m (1 % of the radius), |omega| to 5e-4 relative;
# the two codes differ in the contact radius of the relative velocity and in
# the order of the velocity-Verlet half steps
V_ATOL, X_ATOL, W_RTOL = 1e-4, 1e-4, 5e-4


class OracleRun:
    def __init__(self, sc, box):
        from oracle.port import OracleScene
        self.o = OracleScene(sc, box=box)

    def step(self, n):
        self.o.step(n)

    def state(self):
        g = lambda k: self.o.get(k).reshape(-1, 3).copy()
        return g("x"), g("v"), g("angv")


class EngineRun:
    def __init__(self, sc, box, precision):
        from gpudem_gb300 import engine
        self.e = engine.Engine(sc, precision=precision, model="linear", box=box)

    def step(self, n):
        self.e.step(n)

    def state(self):
        d = self.e.export(history=False)
        return d["x"].reshape(-1, 3), d["v"].reshape(-1, 3), d["angv"].reshape(-1, 3)


def make_run(kind, sc, box):
    return OracleRun(sc, box) if kind == "oracle" else EngineRun(sc, box, kind)


def liggghts_case():
    gold = json.load(open(GOLD))
    d = gold["deck"]
    r = [0.5 * x for x in d["diameter"]]
    m = [rho * 4.0 / 3.0 * math.pi * ri ** 3 for rho, ri in zip(d["density"], r)]
    kn = scenes.hooke_stiffness(d["youngs_modulus"], d["poisson_ratio"], r[0], r[1], m[0], m[1],
                                d["characteristic_velocity"])
    eta = scenes.hooke_eta_const(kn, d["restitution"])
    sc = scenes.two_sphere_scene(d["x0"], d["v0"], r, m, [kn, kn], [eta, eta], d["friction"], d["timestep"])
    return sc, gold["frames"]


def check_liggghts(kind):
    sc, frames = liggghts_case()
    box = (np.full(3, -1.0), np.full(3, 1.0))
    run = make_run(kind, sc, box)
    done = 0
    out = {}
    for f in FRAMES:
        run.step(f - done)
        done = f
        x, v, w = run.state()
        out[f] = (x, v, w)
        for pid in (1, 2):
            ref = np.array(frames[str(f)][str(pid)])
            i = pid - 1
            assert np.allclose(x[i], ref[0:3], rtol=0, atol=X_ATOL), (f, pid, x[i], ref[0:3])
            assert np.allclose(v[i], ref[3:6], rtol=0, atol=V_ATOL), (f, pid, v[i], ref[3:6])
            wl = ref[6:9]
            if np.linalg.norm(wl) > 0:
                assert abs(np.linalg.norm(w[i]) - np.linalg.norm(wl)) <= W_RTOL * np.linalg.norm(wl), (f, pid)
                assert np.allclose(w[i], -wl, rtol=W_RTOL, atol=1e-9), (f, pid, w[i], wl)
            else:
                assert np.linalg.norm(w[i]) == 0.0
    return out


def pair_impact(kind, e, theta_deg=0.0, mu=0.7, dt=1e-6):
    """Two equal spheres (r = 0.01 m, rho = 1000, k = 1e5), one at rest, the
    other at 1 m/s with its centre offset by 2 r sin(theta) across the line of
    motion.  Returns the restitution along the final line of centres (the
    normal one for a head-on impact), the tangential and normal impulses on
    the struck sphere, its spin and the mass."""
    r = 0.01
    m = float(scenes.sphere_mass(1000.0, np.full(1, r))[0])
    k = np.full(2, 1e5)
    th = math.radians(theta_deg)
    x = [[0.0, 0.0, 0.0], [-0.05, 2 * r * math.sin(th), 0.0]]
    sc = scenes.two_sphere_scene(x, [[0.0, 0, 0], [1.0, 0, 0]], [r, r], [m, m], k, scenes.eta_const(k, e), mu, dt,
                                 half=0.2)
    run = make_run(kind, sc, (np.full(3, -0.2), np.full(3, 0.2)))
    run.step(int(round(0.08 / dt)))
    X, V, W = run.state()
    n0 = np.array([math.cos(th), -math.sin(th), 0.0])      # initial line of centres, from 2 to 1
    t0 = np.array([math.sin(th), math.cos(th), 0.0])
    dd = X[0] - X[1]
    n1 = dd / np.linalg.norm(dd)
    e_n = -((V[1] - V[0]) @ n1) / (np.array([1.0, 0, 0]) @ n1)
    return e_n, m * (V[0] @ t0), m * (V[0] @ n0), W[0, 2], m


# ---------------------------------------------------------------- CPU (oracle)

def test_fixture_is_the_deck():
    sc, frames = liggghts_case()
    assert sc.n == 2 and sc.mu == 0.7 and sc.dt == 1e-5
    assert set(map(int, frames)) >= set(FRAMES)
    # the stiffness LIGGGHTS' hooke model gives this pair
    assert abs(sc.k[0] - 127966.3287545) < 1e-6


def test_oracle_matches_liggghts_collision():
    check_liggghts("oracle")


@pytest.mark.parametrize("e", [0.3, 0.7])
def test_oracle_head_on_restitution(e):
    e_n, _, _, w, _ = pair_impact("oracle", e)
    assert abs(e_n - e) <= 0.01 * e
    assert w == 0.0


def test_oracle_oblique_impact_sticks():
    """compareCollision.py's 30-degree impact with mu = 0.7, where Walton's
    impulse model sticks: the tangential impulse is m/7 of the tangential
    approach speed for equal solid spheres (within 5 % below, 2 % above: the
    tangential spring overshoots a little, and the line of centres turns
    during the contact), and the spin takes its moment r J_t / I (within 5 %).
    (Sliding is checked on the incline, where the Coulomb limit holds the
    whole time; in a short impact the reference's cap follows |f_n| including
    its damping term, so no clean mu J_n law applies.)"""
    r = 0.01
    _, jt, _, w, m = pair_impact("oracle", 0.3, theta_deg=30.0, mu=0.7, dt=2e-6)
    stick = m / 7.0 * math.sin(math.radians(30.0))
    assert 0.95 <= jt / stick <= 1.02, jt / stick
    inertia = 0.4 * m * r * r
    assert abs(abs(w) * inertia / (jt * r) - 1.0) <= 0.05


def test_oracle_bouncing_sphere():
    """compareDrop.py: free fall y0 - g t^2 / 2 until the impact, and a
    rebound to e^2 of the drop height."""
    sc = scenes.bouncing_sphere_scene()
    dt, r, floor, y0 = sc.dt, float(sc.r[0]), -1.0, 0.5
    run = make_run("oracle", sc, (np.array([-0.2, -1.2, -0.2]), np.array([0.2, 0.7, 0.2])))
    n = int(0.5 / dt)
    run.step(n)
    x, v, _ = run.state()
    t = n * dt
    assert abs(x[0, 1] - (y0 - 9.81 * t * t / 2)) <= 9.81 * t * dt
    assert abs(v[0, 1] + 9.81 * t) <= 1e-9
    run.step(int(0.056 / dt))
    ymax = -1e9
    for _ in range(400):
        run.step(int(1e-3 / dt))
        x, v, _ = run.state()
        ymax = max(ymax, x[0, 1])
        if v[0, 1] < 0:
            break
    e = math.sqrt((ymax - (floor + r)) / (y0 - (floor + r)))
    assert abs(e - 0.3) <= 0.015 * 0.3


@pytest.mark.parametrize("mu", [0.2, 0.6])
def test_oracle_incline_slip_and_roll(mu):
    check_incline("oracle", mu)


def check_incline(kind, mu, rtol=1e-3):
    """compareRoll.py at 60 degrees: mu = 0.2 < 2/7 tan 60 slides with
    a = g (sin - mu cos); mu = 0.6 rolls with a = 5/7 g sin and |omega| r = |v|."""
    th = math.radians(60.0)
    sc = scenes.incline_scene(60.0, mu)
    d = np.array([math.cos(th), -math.sin(th), 0.0])
    run = make_run(kind, sc, (np.array([-0.1, -0.7, -0.1]), np.array([0.4, 0.1, 0.1])))
    t, u, w = [], [], []
    for k in range(20):
        run.step(1000)
        _, v, om = run.state()
        t.append((k + 1) * 1000 * sc.dt)
        u.append(float(v[0] @ d))
        w.append(float(om[0, 2]))
    a = np.polyfit(t[5:], u[5:], 1)[0]
    rolls = mu >= 2.0 / 7.0 * math.tan(th)
    a_ref = 5.0 / 7.0 * 9.81 * math.sin(th) if rolls else 9.81 * (math.sin(th) - mu * math.cos(th))
    assert abs(a - a_ref) <= rtol * a_ref, (a, a_ref)
    if rolls:
        assert abs(abs(w[-1]) * sc.r[0] / u[-1] - 1.0) <= rtol


# ---------------------------------------------------------------- GPU (engine)

@pytest.mark.gpu
def test_engine_fp64_is_the_oracle_on_the_liggghts_collision():
    sc, _ = liggghts_case()
    box = (np.full(3, -1.0), np.full(3, 1.0))
    a, b = make_run("oracle", sc, box), make_run("fp64", sc, box)
    done = 0
    for f in FRAMES:
        a.step(f - done)
        b.step(f - done)
        done = f
        for p, q in zip(a.state(), b.state()):
            assert np.array_equal(p, q), f


@pytest.mark.gpu
def test_engine_mixed_matches_liggghts_collision():
    check_liggghts("mixed")


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("mu", [0.2, 0.6])
def test_engine_incline_slip_and_roll(precision, mu):
    check_incline(precision, mu)
