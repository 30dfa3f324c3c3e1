"""ctypes wrapper of oracle/_ref/librefharness.so (the unmodified reference CPU
path plus oracle/ref_harness.cu).  Test infrastructure: only the golden-vector
generator and the oracle-pinning tests use it, and only in a checkout where
the reference sources were available to build it (oracle/build_ref.sh)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "librefharness.so")
MAX_NEI = 100

_lib = None


def reference_dir():
    """The reference checkout oracle/build_ref.sh builds from (its
    GDEM_REFERENCE_DIR or default), or None where it is absent."""
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), "--where"], capture_output=True, text=True)
    where = r.stdout.strip()
    return where or None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def build() -> bool:
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True)
    return available()


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("reference harness not built (oracle/build_ref.sh)")
        L = C.CDLL(LIB_PATH)
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        up = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
        L.rh_create.restype = C.c_void_p
        L.rh_create.argtypes = [C.c_int, dp, dp, dp, dp, dp, dp, dp, C.c_double, C.c_double, dp,
                                C.c_int, dp, dp, dp, C.c_double, C.c_double]
        L.rh_step.restype = C.c_int
        L.rh_step.argtypes = [C.c_void_p, C.c_int]
        L.rh_set_active.argtypes = [C.c_void_p, ip]
        L.rh_get_particle.restype = C.c_long
        L.rh_get_particle.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
        L.rh_get_box.argtypes = [C.c_void_p, dp, ip]
        L.rh_get_mesh.restype = C.c_long
        L.rh_get_mesh.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
        L.rh_get_bvh.restype = C.c_long
        L.rh_get_bvh.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
        L.rh_rebuild_lists.argtypes = [C.c_void_p]
        L.rh_update_plist.argtypes = [C.c_void_p, ip, ip, ip, ip, ip]
        L.rh_update_plist_withsort.argtypes = [C.c_void_p, up, ip, ip, ip, ip, ip]
        L.rh_radix_sort.argtypes = [C.c_int, up, up, ip]
        L.rh_morton3d.restype = C.c_uint
        L.rh_morton3d.argtypes = [C.c_uint, C.c_uint, C.c_uint]
        L.rh_dist_triangle.argtypes = [C.c_void_p, C.c_int, C.c_int, dp, ip]
        L.rh_num_tri.restype = C.c_int
        L.rh_num_tri.argtypes = [C.c_void_p]
        L.rh_node_count.restype = C.c_int
        L.rh_node_count.argtypes = [C.c_void_p]
        L.rh_destroy.argtypes = [C.c_void_p]
        L.rh_init_particles.restype = C.c_int
        L.rh_init_particles.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, dp, dp] + [dp] * 8
        _lib = L
    return _lib


_PARTICLE_DTYPES = {
    "isActive": np.int32, "indHis": np.int32, "indHisWall": np.int32, "indHisWallNow": np.int32,
    "indHisVorENow": np.int32, "isContact": np.int32, "isContactWall": np.int32,
    "numCont": np.int32, "numContWall": np.int32, "cellId": np.int32, "cellx": np.int32,
    "pId": np.int32, "mortonKey": np.uint32, "mortonOrder": np.int32, "tmpMortonKey": np.uint32,
    "tmpMortonOrder": np.int32, "neiList": np.int32, "numNei": np.int32, "neiListWall": np.int32,
    "numNeiWall": np.int32,
}
_PARTICLE_SIZES = {"x": 3, "v": 3, "a": 3, "f": 3, "angv": 3, "anga": 3, "mom": 3, "cellx": 3,
                   "g": None}


class RefScene:
    """One reference scene (ParticleSys + BoundingBox + TriangleMesh + BVH)."""

    def __init__(self, sc):
        L = lib()
        N = sc.n
        z3 = np.zeros(3 * N)
        v = z3 if sc.v is None else np.ascontiguousarray(sc.v, np.float64).ravel()
        w = z3 if sc.w is None else np.ascontiguousarray(sc.w, np.float64).ravel()
        self.N = N
        self.h = L.rh_create(N, np.ascontiguousarray(sc.x, np.float64).ravel(), v, w,
                             np.ascontiguousarray(sc.r, np.float64), np.ascontiguousarray(sc.m, np.float64),
                             np.ascontiguousarray(sc.k, np.float64), np.ascontiguousarray(sc.eta, np.float64),
                             float(sc.mu), float(sc.dt), np.ascontiguousarray(sc.g, np.float64),
                             int(sc.tris.shape[0]), np.ascontiguousarray(sc.tris, np.float64).ravel(),
                             np.ascontiguousarray(sc.inlet_lo, np.float64),
                             np.ascontiguousarray(sc.inlet_hi, np.float64),
                             float(sc.skin), float(sc.refresh))
        if not self.h:
            raise RuntimeError("rh_create failed")
        self.nTri = L.rh_num_tri(self.h)

    def step(self, n=1) -> int:
        return lib().rh_step(self.h, int(n))

    def get(self, name):
        N = self.N
        if name in ("g",):
            cnt = 3
        elif name in ("neiList", "neiListWall", "indHis", "indHisWall", "indHisWallNow", "indHisVorENow",
                      "isContact", "isContactWall", "deltHisx", "deltHisy", "deltHisz",
                      "deltHisxWall", "deltHisyWall", "deltHiszWall"):
            cnt = N * MAX_NEI
        elif name in _PARTICLE_SIZES:
            cnt = 3 * N
        else:
            cnt = N
        dt = _PARTICLE_DTYPES.get(name, np.float64)
        out = np.zeros(cnt, dtype=dt)
        n = lib().rh_get_particle(self.h, name.encode(), out.ctypes.data)
        if n < 0:
            raise KeyError(name)
        return out[:n]

    def box(self):
        d = np.zeros(18)
        iv = np.zeros(4, np.int32)
        lib().rh_get_box(self.h, d, iv)
        return d, iv

    def mesh(self, name):
        T = self.nTri
        if name in ("mx", "my", "mz"):
            out = np.zeros(3 * T)
        elif name == "gbox":
            out = np.zeros(6)
        elif name == "nShift":
            out = np.zeros(1, np.int32)
        elif name == "mortonKey":
            out = np.zeros(T, np.uint32)
        elif name.startswith("tri_") or name == "sortedIndex":
            out = np.zeros(T, np.int32)
        else:
            out = np.zeros(T)
        n = lib().rh_get_mesh(self.h, name.encode(), out.ctypes.data)
        if n < 0:
            raise KeyError(name)
        return out[:n]

    def bvh(self, name):
        n = lib().rh_node_count(self.h)
        out = np.zeros(n, np.int32 if name in ("left", "right", "tri") else np.float64)
        lib().rh_get_bvh(self.h, name.encode(), out.ctypes.data)
        return out

    def rebuild_lists(self):
        lib().rh_rebuild_lists(self.h)

    def plist(self):
        _, iv = self.box()
        C_ = int(iv[3])
        pNum = np.zeros(C_, np.int32)
        pStart = np.zeros(C_, np.int32)
        pList = np.zeros(self.N, np.int32)
        cellId = np.zeros(self.N, np.int32)
        cellx = np.zeros(3 * self.N, np.int32)
        lib().rh_update_plist(self.h, pNum, pStart, pList, cellId, cellx)
        return pNum, pStart, pList, cellId, cellx

    def plist_withsort(self):
        _, iv = self.box()
        C_ = int(iv[3])
        keys = np.zeros(self.N, np.uint32)
        order = np.zeros(self.N, np.int32)
        pNum = np.zeros(C_, np.int32)
        pStart = np.zeros(C_, np.int32)
        pList = np.zeros(self.N, np.int32)
        pId = np.zeros(self.N, np.int32)
        lib().rh_update_plist_withsort(self.h, keys, order, pNum, pStart, pList, pId)
        return keys, order, pNum, pStart, pList, pId

    def dist_triangle(self, i, t):
        out = np.zeros(4)
        hit = np.zeros(1, np.int32)
        lib().rh_dist_triangle(self.h, int(i), int(t), out, hit)
        return out, int(hit[0])

    def close(self):
        if self.h:
            lib().rh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def radix_sort(keys):
    keys = np.ascontiguousarray(keys, np.uint32)
    N = keys.size
    ko = np.zeros(max(N, 1), np.uint32)
    po = np.zeros(max(N, 1), np.int32)
    if N:
        lib().rh_radix_sort(N, keys, ko, po)
    return ko[:N], po[:N]


def morton3d(x, y, z):
    return lib().rh_morton3d(int(x), int(y), int(z))


def init_particles(n, r, density, E, res, lo, hi):
    """initializeParticles (ParticleSystem.cu:189-340) of the reference on a
    shuffle inlet: positions and the per-particle constants it sets."""
    out = {k: np.zeros(3 * n if k == "x" else n) for k in ("x", "m", "k", "etaconst", "moi", "invmoi", "sqrtm", "invm")}
    lib().rh_init_particles(int(n), float(r), float(density), float(E), float(res),
                            np.ascontiguousarray(lo, np.float64), np.ascontiguousarray(hi, np.float64),
                            *[out[k] for k in ("x", "m", "k", "etaconst", "moi", "invmoi", "sqrtm", "invm")])
    return out
