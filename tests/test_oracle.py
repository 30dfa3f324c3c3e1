"""The CPU restatement (oracle/gdem_oracle.cpp) pinned bit for bit to the
golden vectors the unmodified reference produced (tests/golden).  CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import compact_rows, load_golden, scene_from_golden


@pytest.fixture(scope="module")
def port():
    from oracle import port as p
    return p


def test_radix_sort_and_morton(port):
    g = load_golden("components")
    names = sorted({k.split("_")[1] for k in g if k.startswith("sort_")})
    for nm in names:
        ko, po = port.radix_sort(g[f"sort_{nm}_keys"])
        assert np.array_equal(ko, g[f"sort_{nm}_sorted"]), nm
        assert np.array_equal(po, g[f"sort_{nm}_perm"]), nm
    for c, k in zip(g["morton_coords"], g["morton_keys"]):
        assert port.morton3d(*c) == k


def test_cell_lists(port):
    g = load_golden("components")
    sc = scene_from_golden(g)
    O = port.OracleScene(sc)
    d, iv = O.box()
    assert np.array_equal(iv[:4], g["box_i"]) and d[0] == g["box_d"][0]
    pNum, pStart, pList = O.plist()
    assert np.array_equal(pNum, g["plist_pNum"])
    assert np.array_equal(pStart, g["plist_pStart"])
    assert np.array_equal(pList, g["plist_pList"])
    assert np.array_equal(O.get("cellId"), g["plist_cellId"])
    keys, order, pNum, pStart, pList = O.plist_withsort()
    assert np.array_equal(keys, g["wsort_keys"])
    assert np.array_equal(order, g["wsort_order"])
    assert np.array_equal(pNum, g["wsort_pNum"])
    assert np.array_equal(pStart, g["wsort_pStart"])
    assert np.array_equal(pList, g["wsort_pList"])


@pytest.mark.parametrize("case", ["tilted", "chute", "box"])
def test_mesh_bvh_and_closest_feature(port, case):
    from gpudem_gb300.scenes import Scene, eta_const, sphere_mass
    g = load_golden("meshes")
    tris = g[f"{case}_tris"]
    x, r = g[f"{case}_probe_x"], g[f"{case}_probe_r"]
    n = r.size
    sc = Scene(x=x, r=r, m=sphere_mass(2500.0, r), k=np.full(n, 1e5), eta=eta_const(np.full(n, 1e5), 0.5),
               mu=0.5, dt=1e-5, tris=tris, inlet_lo=np.zeros(3), inlet_hi=np.zeros(3))
    box_d = g[f"{case}_box_d"]
    O = port.OracleScene(sc, box=(box_d[0:3], box_d[3:6]))
    for f in ["nx", "ny", "nz", "d", "e01x", "e01y", "e01z", "e02x", "e02y", "e02z", "e12x", "e12y", "e12z",
              "d00", "d00inv", "d01", "d11", "d11inv", "d22", "d22inv", "denom", "minx", "maxx", "miny",
              "maxy", "minz", "maxz", "cx", "cy", "cz", "tri_i0", "tri_i1", "tri_i2", "tri_e0", "tri_e1",
              "tri_e2", "sortedIndex", "mortonKey", "mx", "my", "mz"]:
        assert np.array_equal(O.get("mesh_" + f), g[f"{case}_{f}"]), f
    for f in ("minx", "miny", "minz", "maxx", "maxy", "maxz", "left", "right", "tri"):
        assert np.array_equal(O.get("bvh_" + f), g[f"{case}_bvh_{f}"]), f
    for (i, t), ref, hit in zip(g[f"{case}_pairs"], g[f"{case}_dist"], g[f"{case}_hitAt"]):
        out, h = O.dist_triangle(i, t)
        assert h == hit and np.array_equal(out, ref), (i, t)
    nw = O.get("numNeiWall")
    assert np.array_equal(nw, g[f"{case}_numNeiWall"])
    assert np.array_equal(compact_rows(O.get("neiListWall"), nw), g[f"{case}_neiListWall"])


@pytest.mark.parametrize("case", ["box_drop_100", "shaken_200", "tilted_2000"])
def test_trajectory_bit_exact(port, case):
    g = load_golden(case)
    O = port.OracleScene(scene_from_golden(g))
    done = 0
    for c in [0, *g["checkpoints"]]:
        O.step(int(c) - done)
        done = int(c)
        for nm in ("x", "v", "angv") + (("f", "mom") if c else ()):
            assert np.array_equal(O.get(nm), g[f"s{c}_{nm}"]), (c, nm)
        for nm in ("isActive", "numCont", "numContWall", "numNei", "numNeiWall"):
            assert np.array_equal(O.get(nm), g[f"s{c}_{nm}"]), (c, nm)
        nc, ncw = O.get("numCont"), O.get("numContWall")
        assert np.array_equal(compact_rows(O.get("indHis"), nc), g[f"s{c}_indHis"])
        assert np.array_equal(compact_rows(O.get("indHisWall"), ncw), g[f"s{c}_indHisWall"])
        dh = np.stack([compact_rows(O.get("deltHis" + a), nc) for a in "xyz"], 1)
        assert np.array_equal(dh, g[f"s{c}_deltHis"])
        dhw = np.stack([compact_rows(O.get("deltHis" + a + "Wall"), ncw) for a in "xyz"], 1)
        assert np.array_equal(dhw, g[f"s{c}_deltHisWall"])
        assert np.array_equal(compact_rows(O.get("neiList"), O.get("numNei")), g[f"s{c}_neiList"])
        assert np.array_equal(compact_rows(O.get("neiListWall"), O.get("numNeiWall")), g[f"s{c}_neiListWall"])
    assert O.counter("rebuilds") == int(np.sum(g["rebuilds"]))


def test_history_truncates_at_first_lost_contact(port):
    """update_history (cpu_dem.cu:587-609) drops every slot from the first
    lost contact on: two spheres in contact with a third, the first separates,
    the second contact's history is dropped too and restarts from zero."""
    from gpudem_gb300.scenes import Scene, eta_const, sphere_mass
    r = np.full(3, 0.01)
    x = np.array([[0.0, 0.0, 0.0], [0.0199, 0.0, 0.0], [0.0, 0.0199, 0.0]])
    v = np.array([[0.0, 0.0, 0.3], [2.0, 0.0, 0.0], [0.0, 0.0, -0.3]])
    k = np.full(3, 1e5)
    sc = Scene(x=x, r=r, m=sphere_mass(2500.0, r), k=k, eta=eta_const(k, 0.5), mu=0.5, dt=1e-5,
               tris=np.zeros((0, 3, 3)), inlet_lo=np.full(3, -0.2), inlet_hi=np.full(3, 0.2),
               g=np.zeros(3), v=v)
    O = port.OracleScene(sc)
    O.step(1)
    assert O.get("numCont")[0] == 2
    assert list(O.get("indHis")[:2]) == [1, 2]
    held = 0.0
    for _ in range(200):
        prev = O.get("deltHisz")[1]
        O.step(1)
        if O.get("numCont")[0] < 2:
            held = prev
            break
    nc0 = O.get("numCont")[0]
    # particle 1 flew off: slot 0 lost -> the row is cut to length 0, although
    # particle 2 still touches particle 0 ...
    assert nc0 == 0
    O.step(1)
    # ... and it comes back at the next step with a fresh (zero-started) spring
    assert O.get("numCont")[0] == 1 and O.get("indHis")[0] == 2
    fresh = O.get("deltHisz")[0]
    assert abs(held) > 2.0 * abs(fresh) > 0.0
