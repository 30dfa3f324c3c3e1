"""Wall lists from the mesh tree on a mesh of more than 256 x 256 triangles,
where the tree's upper levels are built through L2 before the last tile is
reduced in shared memory (k_mesh_tree), checked against a brute-force scan:
every triangle whose AABB comes within r + skin of the sphere, kept when the
reference's closest-feature test (dist_triangle, cpu_dem.cu:12, run through
gdem_dist_triangle) finds it within r + skin (BVH.cu:576-622)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import compact_rows

pytestmark = pytest.mark.gpu


def _floor_scene(n=300, seed=3):
    from gpudem_gb300 import scenes
    tris = scenes.corrugated_floor_mesh(length=1.0, width=0.2, amp=5e-4, n_target=600_000, seed=seed)
    rng = np.random.default_rng(seed)
    r = rng.uniform(3e-4, 4e-4, n)
    x = np.stack([rng.uniform(-0.49, 0.49, n), rng.uniform(-8e-4, 8e-4, n), rng.uniform(-0.09, 0.09, n)], 1)
    k = np.full(n, 1e4)
    sc = scenes.Scene(x=x, r=r, m=scenes.sphere_mass(2500.0, r), k=k, eta=scenes.eta_const(k, 0.5), mu=0.5,
                      dt=1e-6, tris=tris, inlet_lo=np.array([-0.5, -0.01, -0.1]),
                      inlet_hi=np.array([0.5, 0.01, 0.1]))
    return sc


def _brute_rows(E, sc, x, skin):
    tris = sc.tris
    lo, hi = tris.min(1), tris.max(1)
    rows = []
    for i in range(sc.n):
        R = sc.r[i] + skin
        d = np.maximum(np.maximum(lo - x[i], x[i] - hi), 0.0)
        cand = np.nonzero((d * d).sum(1) <= R * R)[0].astype(np.int32)
        if cand.size == 0:
            rows.append(cand)
            continue
        out, hit = E.dist_triangle(np.repeat(x[i][None], cand.size, 0), np.full(cand.size, R), cand)
        rows.append(cand[hit != -2])
    return rows


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_wall_lists_large_mesh(precision):
    from gpudem_gb300 import engine
    sc = _floor_scene()
    assert sc.tris.shape[0] > 256 * 256 * 2
    E = engine.Engine(sc, precision=precision, box=(np.array([-0.55, -0.05, -0.15]), np.array([0.55, 0.05, 0.15])),
                      wall_capacity=48)
    skin = float(sc.r.max())
    for rebuild_tree in (False, True):
        want = _brute_rows(E, sc, E.export(history=False)["x"].reshape(-1, 3), skin)
        assert sum(w.size for w in want) > sc.n  # most spheres reach the floor
        nn, nl, nw, wl = E.lists()
        got = compact_rows(wl, nw)
        starts = np.concatenate([[0], np.cumsum(nw)[:-1]])
        for i in range(sc.n):
            row = got[starts[i]:starts[i] + nw[i]]
            if precision == "fp64":
                assert np.array_equal(row, want[i]), i
            else:
                # FP32 boxes and features with a widened cutoff: a superset,
                # sorted, and only triangles just beyond the cutoff added
                assert np.all(np.diff(row) > 0), i
                assert np.all(np.isin(want[i], row)), i
                assert row.size <= want[i].size + 4, i
        assert E.stats()["error_word"] == 0
        if not rebuild_tree:
            # rows from the tree rebuilt in every step (beside the step
            # kernel), at the positions two steps later
            E.close()
            E = engine.Engine(sc, precision=precision,
                              box=(np.array([-0.55, -0.05, -0.15]), np.array([0.55, 0.05, 0.15])),
                              wall_capacity=48, bvh_every_step=True)
            E.step(2)
            E.rebuild()
    E.close()

