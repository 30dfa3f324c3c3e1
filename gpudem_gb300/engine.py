"""Host-side mirror of gpudem's step-path interface over the C ABI.

The reference host program owns a ``ParticleSys<HostMemory>`` (reference
layout: xyz-interleaved vectors, MAX_NEI-strided history rows), a
``BoundingBox`` built by ``initialize_BoundingBox`` (BoundingBox.cu:364), a
``TriangleMesh`` from ``load_ascii_stl_double`` (TriangleMesh.cu:363) and a
``BVH`` (BVH.cu:741), and calls ``device_dem_verlet_verlet`` once per step
(main.cu:270).  :class:`Engine` holds the same scene on the GPU through
libgdem.so and keeps the reference's index space (pId) at its boundary.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from .scenes import Scene

MAX_NEI = 100  # row stride of the reference's list and history arrays (hardCodedParameters.h:3)


def _ptr(a, ctype=C.c_double):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


def _vp(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def box_limits(tris: np.ndarray, inlet_lo, inlet_hi):
    """calc_BoundingBoxLimits (BoundingBox.cu:448-478): the union of the mesh
    AABB and the inlet box, each bound multiplied by 1.1."""
    lo = np.array(inlet_lo, dtype=np.float64)
    hi = np.array(inlet_hi, dtype=np.float64)
    if tris is not None and len(tris):
        v = np.asarray(tris, np.float64).reshape(-1, 3)
        gmin, gmax = v.min(0), v.max(0)
        lo = np.where(gmin < lo, gmin, lo)
        hi = np.where(gmax > hi, gmax, hi)
    return lo * 1.1, hi * 1.1


class Engine:
    """One scene on the GPU.  ``precision`` is "fp64" (bit-compatible with the
    reference CPU path) or "mixed"; ``model`` is "linear" or "hertz_mindlin".
    ``inner_skin`` (mixed): skin of the inner rows the step scans (0: 0.1 r_max,
    negative: none, the step scans the list rows); results do not depend on it."""

    def __init__(self, scene: Scene, precision="fp64", model="linear", reorder=True,
                 store_forces=False, nei_capacity=64, wall_capacity=32, hist_capacity=32,
                 hist_wall_capacity=16, steps_per_graph=8, cell_size=-1.0, skin=None,
                 refresh=None, box=None, bvh_every_step=False, mixed_kernel=0, occupancy=0, inner_skin=0.0,
                 import_scene=True):
        self.L = _lib.load()
        self.scene = scene
        self.n = scene.n
        d = _lib.Desc()
        d.n_particles = scene.n
        d.precision = {"fp64": _lib.FP64, "mixed": _lib.MIXED}[precision]
        d.model = {"linear": _lib.LINEAR, "hertz_mindlin": _lib.HERTZ_MINDLIN}[model]
        d.nei_capacity = nei_capacity
        d.wall_capacity = wall_capacity
        d.hist_capacity = hist_capacity
        d.hist_wall_capacity = hist_wall_capacity
        d.reorder = 1 if reorder else 0
        d.store_forces = 1 if store_forces else 0
        d.steps_per_graph = steps_per_graph
        d.dt = scene.dt
        d.mu = scene.mu
        for k in range(3):
            d.g[k] = float(scene.g[k])
        if box is None and scene.box is not None:
            box = scene.box
        lo, hi = box if box is not None else box_limits(scene.tris, scene.inlet_lo, scene.inlet_hi)
        self.box_lo, self.box_hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
        for k in range(3):
            d.box_min[k] = float(self.box_lo[k])
            d.box_max[k] = float(self.box_hi[k])
        d.cell_size = cell_size
        d.skin = scene.skin if skin is None else skin
        d.refresh_thresh = scene.refresh if refresh is None else refresh
        d.youngs_modulus = scene.E
        d.poisson_ratio = scene.nu
        d.restitution = scene.e
        d.rolling_friction = scene.mu_roll
        d.bvh_every_step = 1 if bvh_every_step else 0
        d.mixed_kernel = int(mixed_kernel)
        d.occupancy = int(occupancy)
        d.periodic_x = 1 if scene.periodic_x else 0
        d.inner_skin = float(inner_skin)
        self.desc = d
        h = C.c_void_p()
        _lib.check(self.L.gdem_create(C.byref(d), C.byref(h)), None, "gdem_create")
        self.h = h
        self.store_forces = store_forces
        self.ntri = 0
        if scene.tris is not None and len(scene.tris):
            self.set_mesh(scene.tris)
        if import_scene:
            self.import_particles(scene, history=scene.history, hist_stride=scene.hist_stride)
            if scene.mu_p is not None:
                self.set_particle_materials(scene.mu_p, scene.e_p)

    # ------------------------------------------------------------------ setup
    def _check(self, rc, what):
        _lib.check(rc, self.h, what)

    def set_mesh(self, tris, file_tri_counts=None):
        t = np.ascontiguousarray(tris, np.float64).reshape(-1, 9)
        self.ntri = t.shape[0]
        fc = None if file_tri_counts is None else np.ascontiguousarray(file_tri_counts, np.int32)
        self._check(self.L.gdem_set_mesh(self.h, _vp(t), self.ntri, _vp(fc), 0 if fc is None else fc.size),
                    "gdem_set_mesh")

    def set_mesh_indexed(self, mx, my, mz, tri_i, tri_e, d):
        """Mesh from a loader's welded arrays (gdem_set_mesh_indexed): vertex
        coordinates, per-triangle vertex ids [T,3] (ascending), edge ids + nShift
        [T,3] and plane offsets d [T]."""
        keep = [np.ascontiguousarray(a, np.float64) for a in (mx, my, mz, d)]
        ti = np.ascontiguousarray(np.asarray(tri_i, np.int32).reshape(-1, 3).T)
        te = np.ascontiguousarray(np.asarray(tri_e, np.int32).reshape(-1, 3).T)
        m = _lib.MeshArrays()
        m.nVert, m.nTri = keep[0].size, ti.shape[1]
        m.mx, m.my, m.mz, m.d = (_vp(a) for a in keep)
        m.tri_i0, m.tri_i1, m.tri_i2 = (_vp(ti[c]) for c in range(3))
        m.tri_e0, m.tri_e1, m.tri_e2 = (_vp(te[c]) for c in range(3))
        self.ntri = m.nTri
        self._check(self.L.gdem_set_mesh_indexed(self.h, C.byref(m)), "gdem_set_mesh_indexed")

    def import_particles(self, sc: Scene, history=None, hist_stride=MAX_NEI):
        n = sc.n
        self._keep = []
        arr = lambda a: self._keep.append(np.ascontiguousarray(a, np.float64)) or self._keep[-1]
        p = _lib.Particles()
        p.n = n
        p.x = _ptr(arr(np.asarray(sc.x).reshape(-1)))
        p.v = _ptr(arr(np.asarray(sc.v).reshape(-1))) if sc.v is not None else None
        p.angv = _ptr(arr(np.asarray(sc.w).reshape(-1))) if sc.w is not None else None
        p.r = _ptr(arr(sc.r))
        p.m = _ptr(arr(sc.m))
        p.k = _ptr(arr(sc.k))
        p.etaconst = _ptr(arr(sc.eta))
        if sc.active is not None:
            act = np.ascontiguousarray(sc.active, np.int32)
            self._keep.append(act)
            p.isActive = _ptr(act, C.c_int)
        p.hist_stride = 0
        if history is not None:
            p.hist_stride = hist_stride
            for nm, v in history.items():
                a = np.ascontiguousarray(v, np.int32 if nm.startswith(("num", "ind")) else np.float64)
                self._keep.append(a)
                setattr(p, nm, _ptr(a, C.c_int if a.dtype == np.int32 else C.c_double))
        self._check(self.L.gdem_import_particles(self.h, C.byref(p)), "gdem_import_particles")

    def set_particle_materials(self, mu, restitution):
        """Hertz-Mindlin friction and restitution per particle (pId order)."""
        mu = np.ascontiguousarray(mu, np.float64)
        e = np.ascontiguousarray(restitution, np.float64)
        assert mu.size == self.n and e.size == self.n
        self._check(self.L.gdem_set_particle_materials(self.h, _vp(mu), _vp(e)), "gdem_set_particle_materials")

    # ------------------------------------------------------------------ stepping
    def step(self, nsteps=1):
        """device_dem_verlet_verlet, nsteps times (asynchronous)."""
        self._check(self.L.gdem_step(self.h, int(nsteps)), "gdem_step")

    def sync(self):
        self._check(self.L.gdem_synchronize(self.h), "gdem_synchronize")

    def rebuild(self):
        self._check(self.L.gdem_rebuild(self.h), "gdem_rebuild")

    # ------------------------------------------------------------------ export
    def export(self, history=True, forces=None, hist_stride=MAX_NEI):
        """copyFromDevice (ParticleSystem.cu:97): state in pId order, reference
        layout (history rows of `hist_stride` slots, MAX_NEI by default)."""
        n = self.n
        out = {k: np.zeros(3 * n) for k in ("x", "v", "angv")}
        out["isActive"] = np.zeros(n, np.int32)
        for k in ("r", "m", "k", "etaconst"):
            out[k] = np.zeros(n)
        p = _lib.Particles()
        p.n = n
        p.x, p.v, p.angv = _ptr(out["x"]), _ptr(out["v"]), _ptr(out["angv"])
        p.r, p.m, p.k, p.etaconst = _ptr(out["r"]), _ptr(out["m"]), _ptr(out["k"]), _ptr(out["etaconst"])
        p.isActive = _ptr(out["isActive"], C.c_int)
        forces = self.store_forces if forces is None else forces
        if forces:
            out["f"] = np.zeros(3 * n)
            out["mom"] = np.zeros(3 * n)
            p.f, p.mom = _ptr(out["f"]), _ptr(out["mom"])
        if history:
            p.hist_stride = hist_stride
            for nm in ("numCont", "numContWall"):
                out[nm] = np.zeros(n, np.int32)
                setattr(p, nm, _ptr(out[nm], C.c_int))
            for nm in ("indHis", "indHisWall"):
                out[nm] = np.full(n * hist_stride, -1, np.int32)
                setattr(p, nm, _ptr(out[nm], C.c_int))
            for nm in ("deltHisx", "deltHisy", "deltHisz", "deltHisxWall", "deltHisyWall", "deltHiszWall"):
                out[nm] = np.zeros(n * hist_stride)
                setattr(p, nm, _ptr(out[nm]))
        self._check(self.L.gdem_export_particles(self.h, C.byref(p)), "gdem_export_particles")
        return out

    def export_positions(self, out=None):
        """Positions in pId order (x[3n], reference layout) with one device
        gather and one transfer; `out` may be a pinned host array."""
        x = np.empty(3 * self.n) if out is None else out
        assert x.dtype == np.float64 and x.size == 3 * self.n and x.flags.c_contiguous
        self._check(self.L.gdem_export_positions(self.h, _vp(x)), "gdem_export_positions")
        return x

    def export_positions_async(self, out):
        """Positions in pId order into `out` (a pinned float64 array of 3n)
        without waiting; `out` is valid after sync()."""
        assert out.dtype == np.float64 and out.size == 3 * self.n and out.flags.c_contiguous
        self._check(self.L.gdem_export_positions_async(self.h, _vp(out)), "gdem_export_positions_async")

    def lists(self, stride=MAX_NEI):
        n = self.n
        nn = np.zeros(n, np.int32)
        nl = np.full(n * stride, -1, np.int32)
        nw = np.zeros(n, np.int32)
        wl = np.full(n * stride, -1, np.int32)
        self._check(self.L.gdem_export_lists(self.h, stride, _vp(nn), _vp(nl), _vp(nw), _vp(wl)),
                    "gdem_export_lists")
        return nn, nl, nw, wl

    def morton_keys(self):
        k = np.zeros(self.n, np.uint32)
        self._check(self.L.gdem_morton_keys(self.h, _vp(k)), "gdem_morton_keys")
        return k

    def cells(self):
        nc = C.c_int()
        self._check(self.L.gdem_export_cells(self.h, None, None, None, None, None, C.byref(nc)),
                    "gdem_export_cells")
        n = self.n
        keys = np.zeros(n, np.uint32)
        order = np.zeros(n, np.int32)
        pNum = np.zeros(nc.value, np.int32)
        pStart = np.zeros(nc.value, np.int32)
        pList = np.zeros(n, np.int32)
        self._check(self.L.gdem_export_cells(self.h, _vp(keys), _vp(order), _vp(pNum), _vp(pStart),
                                             _vp(pList), C.byref(nc)), "gdem_export_cells")
        return keys, order, pNum, pStart, pList

    def mesh(self):
        T = self.ntri
        rec = np.zeros((T, 29))
        irec = np.zeros((T, 6), np.int32)
        aabb = np.zeros((T, 6))
        mort = np.zeros(T, np.uint32)
        idx = np.zeros(T, np.int32)
        self._check(self.L.gdem_export_mesh(self.h, _vp(rec), _vp(irec), _vp(aabb), _vp(mort), _vp(idx)),
                    "gdem_export_mesh")
        return rec, irec, aabb, mort, idx

    def dist_triangle(self, pos, r, tri):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(r, np.float64)
        tri = np.ascontiguousarray(tri, np.int32)
        m = tri.size
        out = np.zeros((m, 4))
        hit = np.zeros(m, np.int32)
        self._check(self.L.gdem_dist_triangle(self.h, _vp(pos), _vp(r), _vp(tri), m, _vp(out), _vp(hit)),
                    "gdem_dist_triangle")
        return out, hit

    def stream(self) -> int:
        """cudaStream_t of this engine (as an integer handle)."""
        s = C.c_void_p()
        self._check(self.L.gdem_get_stream(self.h, C.byref(s)), "gdem_get_stream")
        return int(s.value or 0)

    def init_particles(self, box_min, box_max, placement="random", radius=("mono", 1e-3), density=2500.0,
                       youngs_modulus=5e6, restitution=0.5, velocity=(0.0, 0.0, 0.0), velocity_sigma=0.0,
                       gap=0.1, seed=1):
        """Place and import the engine's particles on the device (the
        reference's shuffle inlet with polydisperse radii; gdem_init_particles).
        `radius`: ("mono", r), ("uniform", lo, hi), ("lognormal", median,
        sigma, lo, hi) or ("bidisperse", r1, r2, fraction of r1)."""
        inl = _lib.Inlet()
        for a in range(3):
            inl.box_min[a] = float(box_min[a])
            inl.box_max[a] = float(box_max[a])
            inl.velocity[a] = float(velocity[a])
        inl.placement = _lib.PLACE[placement]
        inl.radius_dist = _lib.RADIUS[radius[0]]
        vals = [float(x) for x in radius[1:]] + [0.0] * 4
        if radius[0] == "bidisperse":
            inl.r_a, inl.r_b, inl.r_c = vals[0], vals[1], vals[2]
        else:
            inl.r_a, inl.r_b, inl.r_c, inl.r_d = vals[:4]
        inl.density = float(density)
        inl.youngs_modulus = float(youngs_modulus)
        inl.restitution = float(restitution)
        inl.velocity_sigma = float(velocity_sigma)
        inl.gap = float(gap)
        inl.seed = int(seed)
        self._check(self.L.gdem_init_particles(self.h, C.byref(inl)), "gdem_init_particles")

    def frame_write_async(self, directory, step, length_factor=1.0):
        """Queue write_frame_bin's file <directory>/result_%012d.bin of the
        current state (built on the device, written by a host thread); returns
        at once.  `frames_flush` waits for the files."""
        self._check(self.L.gdem_frame_write_async(self.h, os.fsencode(directory), int(step), float(length_factor)),
                    "gdem_frame_write_async")

    def frames_flush(self):
        self._check(self.L.gdem_frames_flush(self.h), "gdem_frames_flush")

    def save_snapshot(self, path):
        """Checkpoint the exact state (see gdem_save_snapshot)."""
        self._check(self.L.gdem_save_snapshot(self.h, os.fsencode(path)), "gdem_save_snapshot")

    def load_snapshot(self, path):
        """Restart from a snapshot of an engine of the same size, precision and
        model; the run continues bit for bit."""
        self._check(self.L.gdem_load_snapshot(self.h, os.fsencode(path)), "gdem_load_snapshot")

    def profile_step(self, iters=10) -> float:
        """Mean duration (ms) of the step kernel alone over `iters` launches."""
        ms = C.c_float()
        self._check(self.L.gdem_profile_step(self.h, int(iters), C.byref(ms)), "gdem_profile_step")
        return float(ms.value)

    def stats(self):
        s = _lib.Stats()
        self._check(self.L.gdem_stats_get(self.h, C.byref(s)), "gdem_stats_get")
        return {f: getattr(s, f) for f, _ in s._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.L.gdem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sort_keys(keys):
    """Stable radix sort on the device: (sorted keys, permutation)."""
    L = _lib.load()
    keys = np.ascontiguousarray(keys, np.uint32)
    n = keys.size
    ks = np.zeros(max(n, 1), np.uint32)
    pm = np.zeros(max(n, 1), np.int32)
    _lib.check(L.gdem_sort_keys(_vp(keys), n, _vp(ks), _vp(pm)), None, "gdem_sort_keys")
    return ks[:n], pm[:n]


def device_dem_verlet_verlet(engine: Engine, nsteps: int = 1):
    """The reference's per-step entry point (device_dem.cu:1195) by name."""
    engine.step(nsteps)
