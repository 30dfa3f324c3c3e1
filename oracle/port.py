"""ctypes wrapper of the CPU restatement (oracle/gdem_oracle.cpp, built in-tree
as gpudem_gb300/_build/liboracle.so).  TEST INFRASTRUCTURE: used by the tests
as the checker, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg
— never by the product path."""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

K = 100
_lib = None


def lib():
    global _lib
    if _lib is None:
        from gpudem_gb300 import _build
        path = _build.ORACLE_LIB
        if not os.path.exists(path):
            _build.build_oracle()
        L = C.CDLL(path)
        vp = C.c_void_p
        dp = C.POINTER(C.c_double)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, vp, C.c_double, C.c_double, vp, C.c_int, vp,
                                 vp, C.c_int, vp, vp, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double,
                                 C.c_double, C.c_double, C.c_int]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_materials.argtypes = [vp, vp, vp]
        L.orc_set_materials.restype = C.c_int
        L.orc_step.argtypes = [vp, C.c_int]
        L.orc_step.restype = C.c_int
        L.orc_rebuild.argtypes = [vp]
        L.orc_rebuild.restype = C.c_int
        L.orc_get.argtypes = [vp, C.c_char_p, vp]
        L.orc_get.restype = C.c_long
        L.orc_plist_withsort.argtypes = [vp, vp, vp]
        L.orc_plist.argtypes = [vp]
        L.orc_radix_sort.argtypes = [C.c_int, vp, vp, vp]
        L.orc_morton3d.restype = C.c_uint
        L.orc_morton3d.argtypes = [C.c_uint, C.c_uint, C.c_uint]
        L.orc_dist_triangle.argtypes = [vp, C.c_int, C.c_int, vp, vp]
        L.orc_box.argtypes = [vp, vp, vp]
        L.orc_counter.argtypes = [vp, C.c_char_p]
        L.orc_counter.restype = C.c_long
        L.orc_threads.restype = C.c_int
        _lib = L
    return _lib


def _vp(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


_INT = {"isActive", "numCont", "numContWall", "indHis", "indHisWall", "numNei", "neiList", "numNeiWall",
        "neiListWall", "pNum", "pStart", "pList", "cellId", "cellx"}


class OracleScene:
    """One scene in the CPU restatement of the reference (reference layout)."""

    def __init__(self, sc, box=None, files=None, model="linear"):
        from gpudem_gb300.engine import box_limits
        L = lib()
        self.sc = sc
        self.N = sc.n
        if box is None and sc.box is not None:
            box = sc.box
        lo, hi = box if box is not None else box_limits(sc.tris, sc.inlet_lo, sc.inlet_hi)
        self._keep = [np.ascontiguousarray(a, np.float64) for a in (
            np.asarray(sc.x).ravel(), None if sc.v is None else np.asarray(sc.v).ravel(),
            None if sc.w is None else np.asarray(sc.w).ravel(), sc.r, sc.m, sc.k, sc.eta, sc.g,
            np.asarray(sc.tris).ravel(), lo, hi) if a is not None]
        x = np.ascontiguousarray(np.asarray(sc.x).ravel(), np.float64)
        v = None if sc.v is None else np.ascontiguousarray(np.asarray(sc.v).ravel(), np.float64)
        w = None if sc.w is None else np.ascontiguousarray(np.asarray(sc.w).ravel(), np.float64)
        arrs = [np.ascontiguousarray(a, np.float64) for a in (sc.r, sc.m, sc.k, sc.eta, sc.g)]
        tris = np.ascontiguousarray(np.asarray(sc.tris).ravel(), np.float64)
        lo = np.ascontiguousarray(lo, np.float64)
        hi = np.ascontiguousarray(hi, np.float64)
        fl = None if files is None else np.ascontiguousarray(files, np.int32)
        self._keep = [x, v, w, *arrs, tris, lo, hi, fl]
        self.nTri = int(np.asarray(sc.tris).shape[0]) if sc.tris is not None else 0
        self.h = L.orc_create(self.N, _vp(x), _vp(v), _vp(w), _vp(arrs[0]), _vp(arrs[1]), _vp(arrs[2]),
                              _vp(arrs[3]), float(sc.mu), float(sc.dt), _vp(arrs[4]), self.nTri, _vp(tris),
                              _vp(fl), 0 if fl is None else fl.size, _vp(lo), _vp(hi), float(sc.skin),
                              float(sc.refresh), {"linear": 0, "hertz_mindlin": 1}[model], float(sc.E),
                              float(sc.nu), float(sc.e), float(sc.mu_roll), 1 if sc.periodic_x else 0)
        if not self.h:
            raise ValueError("oracle: bad scene (a periodic x needs at least 3 cells across the period)")
        if sc.mu_p is not None:
            # per-particle friction and restitution (packed scenes), as the
            # engine takes them through gdem_set_particle_materials
            mu_p = np.ascontiguousarray(sc.mu_p, np.float64)
            e_p = np.ascontiguousarray(sc.e_p, np.float64)
            self._keep += [mu_p, e_p]
            if L.orc_set_materials(self.h, _vp(mu_p), _vp(e_p)) != 0:
                raise ValueError("oracle: per-particle materials need the Hertz-Mindlin law")

    def step(self, n=1):
        rc = lib().orc_step(self.h, int(n))
        if rc < 0:
            raise RuntimeError("oracle list overflow (more than 100 neighbours)")
        return rc

    def rebuild(self):
        return lib().orc_rebuild(self.h)

    def get(self, name, count=None):
        N = self.N
        if count is None:
            if name in ("x", "v", "angv", "f", "mom", "cellx"):
                count = 3 * N
            elif name in ("indHis", "indHisWall", "neiList", "neiListWall") or name.startswith("deltHis"):
                count = N * K
            elif name in ("pNum", "pStart"):
                count = self.box()[1][3]
            elif name in ("mesh_mx", "mesh_my", "mesh_mz"):
                count = self.box()[1][6]
            elif name.startswith("mesh_"):
                count = self.nTri
            elif name.startswith("bvh_"):
                count = self.box()[1][5]
            else:
                count = N
        if name == "mesh_mortonKey":
            out = np.zeros(count, np.uint32)
        elif name in _INT or name.startswith(("mesh_tri", "mesh_sorted", "bvh_left", "bvh_right", "bvh_tri")):
            out = np.zeros(count, np.int32)
        else:
            out = np.zeros(count, np.float64)
        need = lib().orc_get(self.h, (name + "#len").encode(), None)
        if need < 0:
            raise KeyError(name)
        if need > out.size:
            out = np.zeros(need, out.dtype)
        n = lib().orc_get(self.h, name.encode(), _vp(out))
        return out[:n]

    def box(self):
        d = np.zeros(11)
        iv = np.zeros(7, np.int32)
        lib().orc_box(self.h, _vp(d), _vp(iv))
        return d, iv

    def plist(self):
        lib().orc_plist(self.h)
        return self.get("pNum"), self.get("pStart"), self.get("pList")

    def plist_withsort(self):
        keys = np.zeros(self.N, np.uint32)
        order = np.zeros(self.N, np.int32)
        lib().orc_plist_withsort(self.h, _vp(keys), _vp(order))
        return keys, order, self.get("pNum"), self.get("pStart"), self.get("pList")

    def dist_triangle(self, i, t):
        out = np.zeros(4)
        hit = np.zeros(1, np.int32)
        lib().orc_dist_triangle(self.h, int(i), int(t), _vp(out), _vp(hit))
        return out, int(hit[0])

    def counter(self, name):
        return lib().orc_counter(self.h, name.encode())

    def close(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def radix_sort(keys):
    keys = np.ascontiguousarray(keys, np.uint32)
    n = keys.size
    ko = np.zeros(max(n, 1), np.uint32)
    po = np.zeros(max(n, 1), np.int32)
    if n:
        lib().orc_radix_sort(n, _vp(keys), _vp(ko), _vp(po))
    return ko[:n], po[:n]


def morton3d(x, y, z):
    return lib().orc_morton3d(int(x), int(y), int(z))


def threads():
    return lib().orc_threads()


def time_steps(sc, steps=400, warmup=3, budget_s=20.0):
    """Time the restated reference step on the host cores: setup (lists) is not
    timed; `warmup` steps untimed; then steps until `steps` or the budget."""
    O = OracleScene(sc)
    O.step(max(1, min(warmup, 3)))
    done = 0
    t0 = time.perf_counter()
    while done < steps:
        O.step(1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    act = int(np.sum(O.get("isActive") == 1))
    O.close()
    return {"value": act * done / dt, "steps": done, "ms_per_step": 1e3 * dt / done, "cores": threads(),
            "sample": f"{done} timed steps (after {max(1, min(warmup, 3))} untimed) of the full "
                      f"{sc.n}-sphere workload, {threads()} OpenMP threads"}


def time_sample(sc, budget_s=20.0):
    r = time_steps(sc, steps=10_000, warmup=1, budget_s=budget_s)
    return {"value": r["value"], "unit": "particle-steps/s", "cores": r["cores"], "kind": "port",
            "sample": r["sample"]}
