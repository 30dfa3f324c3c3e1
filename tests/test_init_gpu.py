"""Device-side particle initialisation (gdem_init_particles): the reference's
shuffle inlet (ParticleSystem.cu:189-340) without the O(N^2) host loop, with
polydisperse radii."""
from __future__ import annotations

import math

import numpy as np
import pytest

from gpudem_gb300 import scenes

pytestmark = pytest.mark.gpu

BOX = (np.array([-0.05, 0.0, -0.05]), np.array([0.05, 0.1, 0.05]))


def empty_engine(n, precision="mixed", model="linear"):
    """An engine of n particles over a closed 0.2 m box, particles not yet set."""
    from gpudem_gb300 import engine
    half = 0.1
    sc = scenes.Scene(x=np.zeros((n, 3)), r=np.full(n, 1e-3), m=np.ones(n), k=np.ones(n), eta=np.ones(n), mu=0.5,
                      dt=2e-6, tris=scenes.box_mesh(half), inlet_lo=BOX[0], inlet_hi=BOX[1], E=5e6, nu=0.3, e=0.5)
    return engine.Engine(sc, precision=precision, model=model, box=(np.full(3, -half * 1.1), np.full(3, half * 1.1)),
                         import_scene=False)


def min_gap(x, r):
    """min over pairs of |x_i - x_j| - r_i - r_j (nearest neighbours by KD tree)."""
    spatial = pytest.importorskip("scipy.spatial")
    tree = spatial.cKDTree(x)
    d, j = tree.query(x, k=2)
    return float(np.min(d[:, 1] - r - r[j[:, 1]]))


def test_random_placement_matches_the_shuffle_inlet():
    n = 20_000
    E = empty_engine(n, precision="fp64")
    E.init_particles(*BOX, placement="random", radius=("mono", 1e-3), density=2500.0, youngs_modulus=9.487e7,
                     restitution=0.5, seed=7)
    st = E.export(history=False)
    x = st["x"].reshape(-1, 3)
    r = np.full(n, 1e-3)
    assert np.array_equal(st["r"], r)
    assert np.all(x >= BOX[0]) and np.all(x <= BOX[1])
    assert min_gap(x, r) >= 0.0          # no two closer than 2 r (ParticleSystem.cu:262)
    # uniform over the region: the centre of mass sits near the region's centre
    assert np.all(np.abs(x.mean(0) - 0.5 * (BOX[0] + BOX[1])) < 2e-3)
    assert np.array_equal(st["isActive"], np.ones(n, np.int32))
    # mass, stiffness and damping constant by the reference's formulas (main.cu:67,
    # ParticleSystem.cu:202, :301); the mass comes back as 1 / (1 / m)
    assert np.allclose(st["m"], scenes.sphere_mass(2500.0, r), rtol=2e-16, atol=0)
    assert np.array_equal(st["k"], np.full(n, scenes.stiffness_from_E(9.487e7, 1e-3)))
    assert np.allclose(st["etaconst"], scenes.eta_const(st["k"], 0.5), rtol=1e-15, atol=0)


def test_lattice_placement_with_lognormal_radii_and_seeds():
    n = 20_000                           # of the region's 28^3 = 21,952 sites
    E = empty_engine(n)
    E.init_particles(*BOX, placement="lattice", radius=("lognormal", 1e-3, 0.15, 0.6e-3, 1.6e-3), gap=0.1, seed=3)
    a = E.export(history=False)["x"].reshape(-1, 3)
    E.init_particles(*BOX, placement="lattice", radius=("lognormal", 1e-3, 0.15, 0.6e-3, 1.6e-3), gap=0.1, seed=3)
    b = E.export(history=False)["x"].reshape(-1, 3)
    E.init_particles(*BOX, placement="lattice", radius=("lognormal", 1e-3, 0.15, 0.6e-3, 1.6e-3), gap=0.1, seed=4)
    c = E.export(history=False)["x"].reshape(-1, 3)
    assert np.array_equal(a, b)          # the seed decides everything
    assert not np.array_equal(a, c)
    assert min_gap(a, np.full(n, 1.6e-3)) >= -1e-12   # sites 2 r_max (1 + gap) apart, jitter gap r_max / 2
    assert np.all(a >= BOX[0]) and np.all(a <= BOX[1])


def test_too_many_particles_is_a_range_error():
    from gpudem_gb300 import _lib
    E = empty_engine(200_000)
    with pytest.raises(_lib.GdemError, match="RANGE"):
        E.init_particles(*BOX, placement="random", radius=("mono", 1.5e-3), seed=1)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_initialised_particles_step(precision):
    n = 20_000
    E = empty_engine(n, precision=precision, model="hertz_mindlin")
    E.init_particles(*BOX, placement="random", radius=("bidisperse", 1.0e-3, 1.5e-3, 0.7), density=2500.0,
                     velocity=(0.0, -0.2, 0.0), velocity_sigma=0.3, seed=11)
    E.step(500)
    s = E.stats()
    assert s["error_word"] == 0 and s["n_active"] == n
    assert s["n_contacts"] > 0


@pytest.mark.parametrize("c", range(5))
def test_device_constants_match_the_reference_initialiser(c):
    """Mass, stiffness and damping constant of gdem_init_particles against the
    reference's own initializeParticles (tests/golden/init_particles.npz, made
    by the reference harness), bit for bit.  The mass comes back as
    1 / (1 / m): the engine stores 1 / m."""
    import os
    from conftest import GOLDEN
    from gpudem_gb300 import engine
    z = dict(np.load(os.path.join(GOLDEN, "init_particles.npz")))
    r, rho, E, e = (float(a) for a in z["cases"][c])
    n = 200
    half = 40 * r
    lo, hi = np.array([-20 * r, 0.0, -20 * r]), np.array([20 * r, 20 * r, 20 * r])
    sc = scenes.Scene(x=np.zeros((n, 3)), r=np.full(n, r), m=np.ones(n), k=np.ones(n), eta=np.ones(n), mu=0.5,
                      dt=1e-6, tris=scenes.box_mesh(half), inlet_lo=lo, inlet_hi=hi)
    Eng = engine.Engine(sc, precision="fp64", box=(np.full(3, -1.1 * half), np.full(3, 1.1 * half)),
                        import_scene=False)
    Eng.init_particles(lo, hi, placement="random", radius=("mono", r), density=rho, youngs_modulus=E,
                       restitution=e, seed=1)
    st = Eng.export(history=False)
    assert np.all(st["k"] == float(z[f"c{c}_k"]))
    assert np.all(st["etaconst"] == float(z[f"c{c}_etaconst"]))
    assert np.all(st["m"] == 1.0 / float(z[f"c{c}_invm"]))
