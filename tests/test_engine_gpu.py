"""Parity of the CUDA engine (through the C ABI) with the reference CPU path's
golden vectors (tests/golden, made by tests/golden/make_golden.py from the
unmodified reference).  Integer results (keys, permutations, cell lists,
neighbour and wall lists, contact histories' keys) must be identical;
FP64 results must agree to 1e-12 relative (array-wise) — they are expected
to be bit-identical, and the trajectory tests say so when they are."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import MAX_NEI, assert_rel, compact_rows, load_golden, scene_from_golden

pytestmark = pytest.mark.gpu

FP_RTOL = 1e-12


@pytest.fixture(scope="module")
def eng_mod():
    from gpudem_gb300 import engine
    return engine


def test_sort_keys_matches_reference(eng_mod):
    g = load_golden("components")
    names = sorted({k.split("_")[1] for k in g if k.startswith("sort_")})
    assert names
    for nm in names:
        keys = g[f"sort_{nm}_keys"]
        ks, pm = eng_mod.sort_keys(keys)
        assert np.array_equal(ks, g[f"sort_{nm}_sorted"]), nm
        assert np.array_equal(pm, g[f"sort_{nm}_perm"]), nm
    ks, pm = eng_mod.sort_keys(np.zeros(0, np.uint32))
    assert ks.size == 0 and pm.size == 0


def test_morton_sort_and_cells_withsort(eng_mod):
    """update_pList_withSort (BoundingBox.cu:664): keys, permutation, pNum,
    pStart, pList and the reordered pId."""
    g = load_golden("components")
    sc = scene_from_golden(g)
    E = eng_mod.Engine(sc, reorder=True)
    keys, order, pNum, pStart, pList = E.cells()
    assert np.array_equal(keys, g["wsort_keys"])
    assert np.array_equal(order, g["wsort_order"])
    assert np.array_equal(order, g["wsort_pId"])
    assert np.array_equal(pNum, g["wsort_pNum"])
    assert np.array_equal(pStart, g["wsort_pStart"])
    assert np.array_equal(pList, g["wsort_pList"])
    # unsorted keys in pId order
    k_orig = np.zeros_like(g["wsort_keys"])
    k_orig[g["wsort_order"]] = g["wsort_keys"]
    assert np.array_equal(E.morton_keys(), k_orig)
    E.close()


def test_cells_canonical(eng_mod):
    """update_pList (BoundingBox.cu:839): cell-id order, ascending index."""
    g = load_golden("components")
    sc = scene_from_golden(g)
    E = eng_mod.Engine(sc, reorder=False)
    keys, order, pNum, pStart, pList = E.cells()
    assert np.array_equal(pNum, g["plist_pNum"])
    assert np.array_equal(pStart, g["plist_pStart"])
    assert np.array_equal(pList, g["plist_pList"])
    E.close()


MESH_FIELDS = ["nx", "ny", "nz", "d", None, None, None, None, None, None, None, None, None,
               "e01x", "e01y", "e01z", "e02x", "e02y", "e02z", "e12x", "e12y", "e12z",
               "d00", "d01", "d11", "denom", "d00inv", "d11inv", "d22inv"]


@pytest.mark.parametrize("ingest", ["corners", "indexed"])
@pytest.mark.parametrize("case", ["tilted", "chute", "box"])
def test_mesh_precompute_and_wall_lists(eng_mod, case, ingest):
    """load_ascii_stl_double precompute (TriangleMesh.cu:560-722), dist_triangle
    (cpu_dem.cu:12) and the wall lists (BVH.cu:576) of probe spheres, with the
    mesh given as STL corners (welded by the engine) or as the reference
    loader's own welded arrays (gdem_set_mesh_indexed)."""
    from gpudem_gb300.scenes import Scene, eta_const, sphere_mass
    g = load_golden("meshes")
    tris = g[f"{case}_tris"]
    x = g[f"{case}_probe_x"]
    r = g[f"{case}_probe_r"]
    n = r.size
    lo_in = 0.5 * (tris.reshape(-1, 3).min(0) + tris.reshape(-1, 3).max(0)) - 0.01
    sc = Scene(x=x, r=r, m=sphere_mass(2500.0, r), k=np.full(n, 1e5), eta=eta_const(np.full(n, 1e5), 0.5),
               mu=0.5, dt=1e-5, tris=tris, inlet_lo=lo_in, inlet_hi=lo_in + 0.02)
    box_d = g[f"{case}_box_d"]
    E = eng_mod.Engine(sc, box=(box_d[0:3], box_d[3:6]))
    if ingest == "indexed":
        E.set_mesh_indexed(g[f"{case}_mx"], g[f"{case}_my"], g[f"{case}_mz"],
                           np.stack([g[f"{case}_tri_i{c}"] for c in range(3)], 1),
                           np.stack([g[f"{case}_tri_e{c}"] for c in range(3)], 1), g[f"{case}_d"])
    rec, irec, aabb, mort, idx = E.mesh()
    for c, f in enumerate(MESH_FIELDS):
        if f is not None:
            assert np.array_equal(rec[:, c], g[f"{case}_{f}"]), f
    mx, my, mz = g[f"{case}_mx"], g[f"{case}_my"], g[f"{case}_mz"]
    for c, nm in enumerate(["tri_i0", "tri_i1", "tri_i2"]):
        ids = g[f"{case}_{nm}"]
        assert np.array_equal(irec[:, c], ids), nm
        assert np.array_equal(rec[:, 4 + 3 * c], mx[ids])
        assert np.array_equal(rec[:, 5 + 3 * c], my[ids])
        assert np.array_equal(rec[:, 6 + 3 * c], mz[ids])
    for c, nm in enumerate(["tri_e0", "tri_e1", "tri_e2"]):
        assert np.array_equal(irec[:, 3 + c], g[f"{case}_{nm}"]), nm
    for c, nm in enumerate(["minx", "miny", "minz", "maxx", "maxy", "maxz"]):
        assert np.array_equal(aabb[:, c], g[f"{case}_{nm}"]), nm
    assert np.array_equal(mort, g[f"{case}_mortonKey"])
    assert np.array_equal(idx, g[f"{case}_sortedIndex"])
    # closest features
    pairs = g[f"{case}_pairs"]
    if pairs.size:
        out, hit = E.dist_triangle(x[pairs[:, 0]], r[pairs[:, 0]], pairs[:, 1])
        assert np.array_equal(hit, g[f"{case}_hitAt"])
        assert np.array_equal(out, g[f"{case}_dist"])
    # wall lists (skin = r_max, the reference default)
    nn, nl, nw, wl = E.lists()
    assert np.array_equal(nw, g[f"{case}_numNeiWall"])
    assert np.array_equal(compact_rows(wl, nw), g[f"{case}_neiListWall"])
    E.close()


def _active_rows(flat, counts, act):
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    return np.concatenate([flat[starts[i]:starts[i] + counts[i]] for i in np.nonzero(act)[0]] or [flat[:0]])


def _compare_state(E, g, tag, exact_log):
    st = E.export(history=True, forces=True)
    nn, nl, nw, wl = E.lists()
    for nm in ("isActive", "numCont", "numContWall"):
        assert np.array_equal(st[nm], g[f"{tag}_{nm}"]), f"{tag} {nm}"
    # lists of inactive particles are stale in the reference (never cleared); compare active rows
    act = st["isActive"] == 1
    gn, gw = g[f"{tag}_numNei"], g[f"{tag}_numNeiWall"]
    assert np.array_equal(nn[act], gn[act]), f"{tag} numNei"
    assert np.array_equal(nw[act], gw[act]), f"{tag} numNeiWall"
    assert np.array_equal(_active_rows(compact_rows(nl, nn), nn, act),
                          _active_rows(g[f"{tag}_neiList"], gn, act)), f"{tag} neiList"
    assert np.array_equal(_active_rows(compact_rows(wl, nw), nw, act),
                          _active_rows(g[f"{tag}_neiListWall"], gw, act)), f"{tag} neiListWall"
    nc, ncw = st["numCont"], st["numContWall"]
    assert np.array_equal(compact_rows(st["indHis"], nc), g[f"{tag}_indHis"]), f"{tag} indHis"
    assert np.array_equal(compact_rows(st["indHisWall"], ncw), g[f"{tag}_indHisWall"]), f"{tag} indHisWall"
    dh = np.stack([compact_rows(st["deltHis" + c], nc) for c in "xyz"], 1)
    dhw = np.stack([compact_rows(st["deltHis" + c + "Wall"], ncw) for c in "xyz"], 1)
    pairs = [("x", st["x"]), ("v", st["v"]), ("angv", st["angv"]), ("deltHis", dh), ("deltHisWall", dhw)]
    if tag != "s0":
        pairs += [("f", st["f"]), ("mom", st["mom"])]
    for nm, a in pairs:
        b = g[f"{tag}_{nm}"]
        assert_rel(a, b, FP_RTOL, f"{tag} {nm}")
        exact_log.append((tag, nm, bool(np.array_equal(a, b))))


@pytest.mark.parametrize("case", ["box_drop_100", "shaken_200", "tilted_2000"])
@pytest.mark.parametrize("reorder", [True, False])
def test_trajectory_matches_reference(eng_mod, case, reorder):
    """device_dem_verlet_verlet stepped against cpu_dem_verlet_verlet + checkOoB
    (main.cu:302-316): states, forces, torques, histories and lists at every
    checkpoint."""
    g = load_golden(case)
    sc = scene_from_golden(g)
    E = eng_mod.Engine(sc, reorder=reorder, store_forces=True)
    exact = []
    _compare_state(E, g, "s0", exact)
    done = 0
    for c in g["checkpoints"]:
        E.step(int(c) - done)
        done = int(c)
        _compare_state(E, g, f"s{c}", exact)
    st = E.stats()
    assert st["error_word"] == 0
    assert st["steps"] == done
    assert st["rebuilds"] == 1 + int(np.sum(g["rebuilds"]))
    not_exact = [e for e in exact if not e[2]]
    print(f"{case}: {len(exact) - len(not_exact)}/{len(exact)} FP64 arrays bit-identical; "
          f"not: {not_exact[:6]}")
    E.close()
