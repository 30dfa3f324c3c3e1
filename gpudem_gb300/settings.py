"""demSettings.json to a scene: the host side of the reference's main program
(main.cu:44-140) over the engine's C ABI.

``load(path)`` reads the settings (gdem_settings_load: the reference's keys,
with YoungModulus and bruteOn optional and the "file" inlet taking its file
name as a string or as {"name": ...}).  ``scene(path)`` builds what main.cu
sets up before its step loop: the walls from the ASCII STL files
(gdem_read_stl, welded per file by gdem_set_mesh as load_ascii_stl_double
does), the particles from the particle file (file inlet) or at seeded random
non-overlapping positions in the shuffle box (shuffle inlet), with the mass,
stiffness and damping constant the reference derives, the time step snapped
to the output interval, gravity and friction.  Paths in the settings are
taken relative to the settings file's directory (the reference runs in the
case directory and opens them relative to it).
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import _lib
from .scenes import Scene, random_packing

_FIELDS_STR = ("particle_file",)


def _as_dict(s: "_lib.Settings") -> dict:
    out = {}
    for name, _ in s._fields_:
        val = getattr(s, name)
        if name == "walls":
            out[name] = [val[i].value.decode() for i in range(s.n_walls)]
        elif name in _FIELDS_STR:
            out[name] = val.decode()
        elif isinstance(val, C.Array):
            out[name] = list(val)
        else:
            out[name] = val
    out["input_mode"] = "file" if s.input_mode == _lib.INLET_FILE else "shuffle"
    return out


def _call(fn, arg) -> dict:
    s = _lib.Settings()
    msg = C.create_string_buffer(512)
    rc = fn(arg, C.byref(s), msg, len(msg))
    if rc != _lib.GDEM_OK:
        raise _lib.GdemError(f"settings: {_lib.ERRORS.get(rc, rc)} {msg.value.decode()}")
    return _as_dict(s)


def parse(text: str) -> dict:
    """Settings from the JSON text (gdem_settings_parse)."""
    return _call(_lib.load().gdem_settings_parse, text.encode())


def load(path: str) -> dict:
    """Settings from a demSettings.json file (gdem_settings_load)."""
    return _call(_lib.load().gdem_settings_load, os.fsencode(path))


def read_stl(path: str) -> np.ndarray:
    """(T, 3, 3) triangle corners of an ASCII STL file in file order."""
    L = _lib.load()
    n = L.gdem_read_stl(os.fsencode(path), None, 0)
    if n < 0:
        raise _lib.GdemError(f"cannot read the STL file {path}")
    tris = np.zeros((max(n, 1), 3, 3))
    L.gdem_read_stl(os.fsencode(path), C.c_void_p(tris.ctypes.data), n)
    return tris[:n]


def read_particle_file(path: str, n: int):
    """Positions, velocities and their bounding box from the file inlet's CSV."""
    L = _lib.load()
    x = np.zeros(3 * n)
    v = np.zeros(3 * n)
    lo = np.zeros(3)
    hi = np.zeros(3)
    rc = L.gdem_read_particle_file(os.fsencode(path), n, *[C.c_void_p(a.ctypes.data) for a in (x, v, lo, hi)])
    if rc != _lib.GDEM_OK:
        raise _lib.GdemError(f"particle file {path}: needs a header with x,y,z,vx,vy,vz and {n} rows")
    return x.reshape(-1, 3), v.reshape(-1, 3), lo, hi


def scene(path: str, seed: int | None = None) -> tuple[Scene, np.ndarray, dict]:
    """(scene, file_tri_counts, settings) of a demSettings.json: the scene is
    ready for Engine(...); pass file_tri_counts to Engine.set_mesh to weld the
    walls per file as the reference's loader does."""
    st = load(path)
    base = os.path.dirname(os.path.abspath(path))
    here = lambda p: p if os.path.isabs(p) else os.path.join(base, p)
    meshes = [read_stl(here(f)) for f in st["walls"]]
    tris = np.concatenate(meshes) if meshes else np.zeros((0, 3, 3))
    counts = np.array([m.shape[0] for m in meshes], np.int32)
    n = st["n_particles"]
    r = np.full(n, st["radius"])
    v = None
    if st["input_mode"] == "file":
        x, v, lo, hi = read_particle_file(here(st["particle_file"]), n)
    else:
        lo, hi = np.array(st["inlet_min"]), np.array(st["inlet_max"])
        rng = np.random.default_rng(st["seed"] if seed is None else seed)
        x = random_packing(n, r, lo, hi, rng)
    sc = Scene(x=x, r=r, m=np.full(n, st["mass"]), k=np.full(n, st["stiffness"]), eta=np.full(n, st["etaconst"]),
               mu=st["mu"], dt=st["dt"], tris=tris, inlet_lo=np.asarray(lo, np.float64),
               inlet_hi=np.asarray(hi, np.float64), g=np.array(st["g"]), v=v,
               e=st["restitution"], name=os.path.basename(base))
    return sc, counts, st

