"""Generate the golden vectors in tests/golden/*.npz from the UNMODIFIED
reference CPU path (oracle/_ref/librefharness.so, built by oracle/build_ref.sh
from the reference sources).  Run from the repository root:

    python tests/golden/make_golden.py          # every fixture
    python tests/golden/make_golden.py init     # init_particles.npz only

Every fixture records the exact inputs next to the outputs, so the tests can
rebuild the same scene for the oracle port and the CUDA engine without the
reference being present.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from gpudem_gb300 import scenes  # noqa: E402
from oracle import refharness as rh  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
K = rh.MAX_NEI


def compact(rows, counts):
    rows = rows.reshape(-1, K)
    return np.concatenate([rows[i, :counts[i]] for i in range(counts.size)]) if counts.size else rows[:0, 0]


def scene_inputs(sc):
    d = dict(x=sc.x, r=sc.r, m=sc.m, k=sc.k, eta=sc.eta, mu=np.float64(sc.mu), dt=np.float64(sc.dt),
             g=sc.g, tris=sc.tris, inlet_lo=sc.inlet_lo, inlet_hi=sc.inlet_hi,
             skin=np.float64(sc.skin), refresh=np.float64(sc.refresh))
    if sc.v is not None:
        d["v"] = sc.v
    if sc.w is not None:
        d["w"] = sc.w
    return {"in_" + k: v for k, v in d.items()}


def state(R, tag):
    s = {}
    for nm in ("x", "v", "angv", "f", "mom"):
        s[nm] = R.get(nm)
    for nm in ("isActive", "numCont", "numContWall", "numNei", "numNeiWall"):
        s[nm] = R.get(nm)
    nc, ncw = s["numCont"], s["numContWall"]
    s["indHis"] = compact(R.get("indHis"), nc)
    s["deltHis"] = np.stack([compact(R.get("deltHis" + c), nc) for c in "xyz"], 1)
    s["indHisWall"] = compact(R.get("indHisWall"), ncw)
    s["deltHisWall"] = np.stack([compact(R.get("deltHis" + c + "Wall"), ncw) for c in "xyz"], 1)
    s["neiList"] = compact(R.get("neiList"), s["numNei"])
    s["neiListWall"] = compact(R.get("neiListWall"), s["numNeiWall"])
    s["ref"] = np.stack([R.get("refx"), R.get("refy"), R.get("refz")], 1)
    return {f"{tag}_{k}": v for k, v in s.items()}


def run_case(name, sc, checkpoints):
    R = rh.RefScene(sc)
    out = scene_inputs(sc)
    out.update(state(R, "s0"))
    done = 0
    reb = []
    for c in checkpoints:
        reb.append(R.step(c - done))
        done = c
        out.update(state(R, f"s{c}"))
    out["checkpoints"] = np.asarray(checkpoints, np.int64)
    out["rebuilds"] = np.asarray(reb, np.int64)
    d, iv = R.box()
    out["box_d"], out["box_i"] = d, iv
    R.close()
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB, rebuilds {reb}")


def shaken_box(n=200, seed=7):
    rng = np.random.default_rng(seed)
    r = rng.uniform(0.008, 0.012, n)
    half = 0.1
    x = scenes.random_packing(n, r, [-half, -half, -half], [half, half, half], rng)
    m = scenes.sphere_mass(2500.0, r)
    k = np.full(n, 1e5)
    v = rng.normal(0.0, 1.0, (n, 3))
    w = rng.normal(0.0, 50.0, (n, 3))
    return scenes.Scene(x=x, r=r, m=m, k=k, eta=scenes.eta_const(k, 0.5), mu=0.5, dt=1e-5,
                        tris=scenes.tilted_box_mesh(half, 20.0, levels=1),
                        inlet_lo=np.array([-half] * 3), inlet_hi=np.array([half] * 3), v=v, w=w,
                        name="shaken")


def tilted_twin(n=2000, seed=2):
    sc = scenes.config2_tilted_box(n=n, seed=seed, half=0.06, levels=1)
    rng = np.random.default_rng(seed + 100)
    sc.v = rng.normal(0.0, 0.3, (n, 3))
    sc.w = rng.normal(0.0, 20.0, (n, 3))
    return sc


def components():
    out = {}
    rng = np.random.default_rng(11)
    cases = {
        "one": np.array([5], np.uint32),
        "equal": np.full(257, 0x2AAAAAAA, np.uint32),
        "max30": np.concatenate([np.full(64, 0x3FFFFFFF, np.uint32), np.zeros(64, np.uint32)]),
        "max32": rng.choice(np.array([0, 0xFFFFFFFF, 0x80000000, 1], np.uint32), 999).astype(np.uint32),
        "dups": rng.integers(0, 50, 5000).astype(np.uint32),
        "rand30": rng.integers(0, 1 << 30, 20000).astype(np.uint32),
        "sorted": np.arange(3000, dtype=np.uint32),
        "reversed": np.arange(3000, dtype=np.uint32)[::-1].copy(),
    }
    for nm, keys in cases.items():
        ko, po = rh.radix_sort(keys)
        out[f"sort_{nm}_keys"] = keys
        out[f"sort_{nm}_sorted"] = ko
        out[f"sort_{nm}_perm"] = po
    # Morton encoding of boundary coordinates
    coords = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1023, 1023, 1023], [1024, 5, 7],
                       [513, 2, 1000], [77, 900, 300]], np.uint32)
    out["morton_coords"] = coords
    out["morton_keys"] = np.array([rh.morton3d(*c) for c in coords], np.uint32)

    # cell lists with and without the Morton reorder, on a polydisperse bed
    sc = tilted_twin(n=2000, seed=5)
    out.update(scene_inputs(sc))
    R = rh.RefScene(sc)
    pNum, pStart, pList, cellId, cellx = R.plist()
    out["plist_pNum"], out["plist_pStart"], out["plist_pList"] = pNum, pStart, pList
    out["plist_cellId"], out["plist_cellx"] = cellId, cellx
    R.close()
    R = rh.RefScene(sc)
    keys, order, pNum, pStart, pList, pId = R.plist_withsort()
    out["wsort_keys"], out["wsort_order"], out["wsort_pNum"] = keys, order, pNum
    out["wsort_pStart"], out["wsort_pList"], out["wsort_pId"] = pStart, pList, pId
    d, iv = R.box()
    out["box_d"], out["box_i"] = d, iv
    R.close()
    np.savez_compressed(os.path.join(OUT, "components.npz"), **out)
    print("components.npz", os.path.getsize(os.path.join(OUT, "components.npz")) // 1024, "KiB")


def meshes():
    out = {}
    mesh_cases = {
        "tilted": scenes.tilted_box_mesh(0.1, 30.0, levels=2),
        "chute": scenes.helical_chute_mesh(n_target=2000, seed=3),
        "box": scenes.box_mesh(0.1),
    }
    fields_d = ["nx", "ny", "nz", "d", "e01x", "e01y", "e01z", "e02x", "e02y", "e02z", "e12x", "e12y",
                "e12z", "d00", "d00inv", "d01", "d11", "d11inv", "d22", "d22inv", "denom", "minx",
                "maxx", "miny", "maxy", "minz", "maxz", "cx", "cy", "cz"]
    fields_i = ["tri_i0", "tri_i1", "tri_i2", "tri_e0", "tri_e1", "tri_e2", "sortedIndex", "mortonKey"]
    rng = np.random.default_rng(12)
    for nm, tris in mesh_cases.items():
        lo = tris.reshape(-1, 3).min(0)
        hi = tris.reshape(-1, 3).max(0)
        ctr = 0.5 * (lo + hi)
        # a few probe particles near the surface to exercise dist_triangle
        n = 400
        picks = rng.integers(0, tris.shape[0], n)
        bary = rng.dirichlet([0.3, 0.3, 0.3], n)
        surf = np.einsum("nc,ncd->nd", bary, tris[picks])
        r = np.full(n, 0.004)
        x = surf + rng.normal(0, 0.003, (n, 3))
        sc = scenes.Scene(x=x, r=r, m=scenes.sphere_mass(2500.0, r), k=np.full(n, 1e5),
                          eta=scenes.eta_const(np.full(n, 1e5), 0.5), mu=0.5, dt=1e-5, tris=tris,
                          inlet_lo=ctr - 0.01, inlet_hi=ctr + 0.01)
        R = rh.RefScene(sc)
        out[f"{nm}_tris"] = tris
        for f in fields_d + fields_i:
            out[f"{nm}_{f}"] = R.mesh(f)
        out[f"{nm}_nShift"] = R.mesh("nShift")
        out[f"{nm}_gbox"] = R.mesh("gbox")
        nv = int(max(R.mesh("tri_i0").max(), R.mesh("tri_i1").max(), R.mesh("tri_i2").max())) + 1
        out[f"{nm}_mx"] = R.mesh("mx")[:nv]
        out[f"{nm}_my"] = R.mesh("my")[:nv]
        out[f"{nm}_mz"] = R.mesh("mz")[:nv]
        for f in ("minx", "miny", "minz", "maxx", "maxy", "maxz", "left", "right", "tri"):
            out[f"{nm}_bvh_{f}"] = R.bvh(f)
        # dist_triangle over every (probe, triangle) pair close enough to matter
        pairs = []
        res = []
        hits = []
        for i in range(n):
            for t in range(tris.shape[0]):
                if np.min(np.linalg.norm(tris[t] - x[i], axis=1)) < 0.05 or tris.shape[0] <= 200:
                    o, h = R.dist_triangle(i, t)
                    if h != -2:
                        pairs.append((i, t))
                        res.append(o)
                        hits.append(h)
        out[f"{nm}_probe_x"] = x
        out[f"{nm}_probe_r"] = r
        out[f"{nm}_pairs"] = np.asarray(pairs, np.int32).reshape(-1, 2)
        out[f"{nm}_dist"] = np.asarray(res).reshape(-1, 4)
        out[f"{nm}_hitAt"] = np.asarray(hits, np.int32)
        # wall neighbour lists of the probes (BVH.cu:576), skin = r_max
        out[f"{nm}_numNeiWall"] = R.get("numNeiWall")
        out[f"{nm}_neiListWall"] = compact(R.get("neiListWall"), R.get("numNeiWall"))
        out[f"{nm}_box_d"], out[f"{nm}_box_i"] = R.box()
        R.close()
    np.savez_compressed(os.path.join(OUT, "meshes.npz"), **out)
    print("meshes.npz", os.path.getsize(os.path.join(OUT, "meshes.npz")) // 1024, "KiB")


# (radius, density, Young's modulus, restitution) of the particle-constant
# fixture: the three workloads' materials (linear twins) and two of the
# shipped cases' particles with a Young's modulus given
INIT_CASES = [(0.01, 2500.0, 9.487e7, 0.5), (2e-3, 2500.0, 5e6, 0.6), (1e-3, 2500.0, 5e6, 0.5),
              (0.01, 1000.0, 1e7, 0.3), (0.1, 1000.0, 1e9, 0.3)]


def init_particles():
    """The reference's initializeParticles (ParticleSystem.cu:189-340) on a
    40-particle shuffle inlet per material: mass, stiffness, damping constant,
    moment of inertia and the derived inverses it stores."""
    out = {"cases": np.array(INIT_CASES)}
    for c, (r, rho, E, e) in enumerate(INIT_CASES):
        o = rh.init_particles(40, r, rho, E, e, [-20 * r, 0.0, -20 * r], [20 * r, 20 * r, 20 * r])
        for k in ("m", "k", "etaconst", "moi", "invmoi", "sqrtm", "invm"):
            assert np.all(o[k] == o[k][0]), k
            out[f"c{c}_{k}"] = np.float64(o[k][0])
    np.savez_compressed(os.path.join(OUT, "init_particles.npz"), **out)
    print("init_particles.npz", os.path.getsize(os.path.join(OUT, "init_particles.npz")), "B")


def main():
    if not rh.available():
        rh.build()
    if sys.argv[1:] == ["init"]:
        init_particles()
        return
    init_particles()
    components()
    meshes()
    run_case("box_drop_100", scenes.config1_box_drop(), [1, 2, 10, 100, 1000, 5000, 10000, 20000])
    run_case("shaken_200", shaken_box(), [1, 10, 100, 500, 1000, 3000])
    run_case("tilted_2000", tilted_twin(), [1, 100, 1000, 2000])


if __name__ == "__main__":
    main()
