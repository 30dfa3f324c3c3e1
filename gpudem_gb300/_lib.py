"""ctypes binding of the engine's C ABI (include/gdem.h).

The library is the in-tree build gpudem_gb300/_build/libgdem.so.  There is no
fallback: if it is missing or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

GDEM_OK = 0
ERRORS = {1: "GDEM_ERR_ARG", 2: "GDEM_ERR_CUDA", 3: "GDEM_ERR_CAPACITY", 4: "GDEM_ERR_STATE",
          5: "GDEM_ERR_RANGE", 6: "GDEM_ERR_DEVICE"}
FP64, MIXED = 0, 1
LINEAR, HERTZ_MINDLIN = 0, 1

EXPORTED = [
    "gdem_create", "gdem_destroy", "gdem_last_error", "gdem_set_mesh", "gdem_import_particles",
    "gdem_step", "gdem_synchronize", "gdem_export_particles", "gdem_stats_get", "gdem_rebuild",
    "gdem_export_lists", "gdem_morton_keys", "gdem_export_cells", "gdem_sort_keys",
    "gdem_sort_keys_noalloc", "gdem_set_mesh_indexed", "gdem_set_particle_materials",
    "gdem_dist_triangle", "gdem_export_mesh", "gdem_get_stream", "gdem_profile_step",
    "gdem_export_positions", "gdem_frame_write_async", "gdem_frames_flush", "gdem_save_snapshot",
    "gdem_load_snapshot", "gdem_init_particles", "gdem_export_positions_async", "gdem_check_snapshot",
    "gdem_settings_load", "gdem_settings_parse", "gdem_read_particle_file", "gdem_read_stl",
]
PLACE = {"random": 0, "lattice": 1}
RADIUS = {"mono": 0, "uniform": 1, "lognormal": 2, "bidisperse": 3}


class Inlet(C.Structure):
    """gdem_inlet: device-side particle placement (the reference's shuffle inlet)."""
    _fields_ = [("box_min", C.c_double * 3), ("box_max", C.c_double * 3), ("placement", C.c_int),
                ("radius_dist", C.c_int), ("r_a", C.c_double), ("r_b", C.c_double), ("r_c", C.c_double),
                ("r_d", C.c_double), ("density", C.c_double), ("youngs_modulus", C.c_double),
                ("restitution", C.c_double), ("velocity", C.c_double * 3), ("velocity_sigma", C.c_double),
                ("gap", C.c_double), ("seed", C.c_ulonglong)]


SETTINGS_MAX_WALLS, SETTINGS_PATH = 16, 1024
INLET_SHUFFLE, INLET_FILE = 0, 1


class Settings(C.Structure):
    """gdem_settings: demSettings.json as main.cu reads it."""
    _fields_ = [("radius", C.c_double), ("restitution", C.c_double), ("density", C.c_double), ("mu", C.c_double),
                ("youngs_modulus", C.c_double), ("k_given", C.c_double), ("mass", C.c_double),
                ("stiffness", C.c_double), ("etaconst", C.c_double), ("dt", C.c_double), ("out_step", C.c_int),
                ("n_particles", C.c_int), ("input_mode", C.c_int), ("inlet_min", C.c_double * 3),
                ("inlet_max", C.c_double * 3), ("particle_file", C.c_char * SETTINGS_PATH), ("n_walls", C.c_int),
                ("walls", (C.c_char * SETTINGS_PATH) * SETTINGS_MAX_WALLS), ("g", C.c_double * 3),
                ("gpu_on", C.c_int), ("brute_on", C.c_int), ("seed", C.c_int), ("dt_factor", C.c_double),
                ("start_time", C.c_double), ("end_time", C.c_double), ("output_timing", C.c_double)]


class MeshArrays(C.Structure):
    """gdem_mesh_arrays: a welded mesh in the reference loader's arrays."""
    _fields_ = [("nVert", C.c_int), ("nTri", C.c_int)] + [
        (nm, C.c_void_p) for nm in ("mx", "my", "mz", "tri_i0", "tri_i1", "tri_i2",
                                    "tri_e0", "tri_e1", "tri_e2", "d")]


class Desc(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int), ("precision", C.c_int), ("model", C.c_int),
        ("nei_capacity", C.c_int), ("wall_capacity", C.c_int), ("hist_capacity", C.c_int),
        ("hist_wall_capacity", C.c_int), ("reorder", C.c_int), ("store_forces", C.c_int),
        ("steps_per_graph", C.c_int),
        ("dt", C.c_double), ("mu", C.c_double), ("g", C.c_double * 3),
        ("box_min", C.c_double * 3), ("box_max", C.c_double * 3),
        ("cell_size", C.c_double), ("skin", C.c_double), ("refresh_thresh", C.c_double),
        ("youngs_modulus", C.c_double), ("poisson_ratio", C.c_double),
        ("restitution", C.c_double), ("rolling_friction", C.c_double),
        ("bvh_every_step", C.c_int), ("mixed_kernel", C.c_int), ("occupancy", C.c_int),
        ("periodic_x", C.c_int), ("inner_skin", C.c_double),
    ]


_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)


class Particles(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("x", _DP), ("v", _DP), ("angv", _DP), ("r", _DP), ("m", _DP), ("k", _DP),
        ("etaconst", _DP), ("isActive", _IP), ("hist_stride", C.c_int), ("numCont", _IP),
        ("indHis", _IP), ("deltHisx", _DP), ("deltHisy", _DP), ("deltHisz", _DP),
        ("numContWall", _IP), ("indHisWall", _IP), ("deltHisxWall", _DP), ("deltHisyWall", _DP),
        ("deltHiszWall", _DP), ("f", _DP), ("mom", _DP),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("steps", C.c_longlong), ("rebuilds", C.c_longlong), ("n_active", C.c_longlong),
        ("n_nei", C.c_longlong), ("n_wall", C.c_longlong), ("n_contacts", C.c_longlong),
        ("n_wall_contacts", C.c_longlong), ("kinetic_energy", C.c_double),
        ("coordination", C.c_double), ("packing_fraction", C.c_double),
        ("max_overlap", C.c_double), ("error_word", C.c_uint), ("max_nei", C.c_int),
        ("max_wall", C.c_int), ("n_inner", C.c_longlong), ("inner_builds", C.c_longlong),
        ("n_inner_wall", C.c_longlong),
    ]


_lib = None


class GdemError(RuntimeError):
    pass


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libgdem.so; raise if it is absent (no CPU fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build_engine()
        else:
            raise GdemError(f"{path} not built: run __graft_entry__.build() (nvcc, sm_103a)")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.gdem_create.argtypes = [C.POINTER(Desc), C.POINTER(vp)]
    L.gdem_destroy.argtypes = [vp]
    L.gdem_last_error.argtypes = [vp]
    L.gdem_last_error.restype = C.c_char_p
    L.gdem_set_mesh.argtypes = [vp, vp, C.c_int, vp, C.c_int]
    L.gdem_import_particles.argtypes = [vp, C.POINTER(Particles)]
    L.gdem_step.argtypes = [vp, C.c_int]
    L.gdem_synchronize.argtypes = [vp]
    L.gdem_export_particles.argtypes = [vp, C.POINTER(Particles)]
    L.gdem_stats_get.argtypes = [vp, C.POINTER(Stats)]
    L.gdem_rebuild.argtypes = [vp]
    L.gdem_export_lists.argtypes = [vp, C.c_int, vp, vp, vp, vp]
    L.gdem_morton_keys.argtypes = [vp, vp]
    L.gdem_export_cells.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.gdem_sort_keys.argtypes = [vp, C.c_int, vp, vp]
    L.gdem_sort_keys_noalloc.argtypes = [vp, C.c_int, vp, vp, vp]
    L.gdem_set_mesh_indexed.argtypes = [vp, C.POINTER(MeshArrays)]
    L.gdem_set_particle_materials.argtypes = [vp, vp, vp]
    L.gdem_dist_triangle.argtypes = [vp, vp, vp, vp, C.c_int, vp, vp]
    L.gdem_export_mesh.argtypes = [vp, vp, vp, vp, vp, vp]
    L.gdem_get_stream.argtypes = [vp, C.POINTER(vp)]
    L.gdem_export_positions.argtypes = [vp, vp]
    L.gdem_profile_step.argtypes = [vp, C.c_int, C.POINTER(C.c_float)]
    L.gdem_frame_write_async.argtypes = [vp, C.c_char_p, C.c_int, C.c_double]
    L.gdem_frames_flush.argtypes = [vp]
    L.gdem_save_snapshot.argtypes = [vp, C.c_char_p]
    L.gdem_load_snapshot.argtypes = [vp, C.c_char_p]
    L.gdem_check_snapshot.argtypes = [C.c_char_p, C.c_int]
    L.gdem_settings_load.argtypes = [C.c_char_p, C.POINTER(Settings), C.c_char_p, C.c_int]
    L.gdem_settings_parse.argtypes = [C.c_char_p, C.POINTER(Settings), C.c_char_p, C.c_int]
    L.gdem_read_particle_file.argtypes = [C.c_char_p, C.c_int, vp, vp, vp, vp]
    L.gdem_read_stl.argtypes = [C.c_char_p, vp, C.c_int]
    L.gdem_init_particles.argtypes = [vp, C.POINTER(Inlet)]
    L.gdem_export_positions_async.argtypes = [vp, vp]
    for nm in EXPORTED:
        if nm != "gdem_last_error":
            getattr(L, nm).restype = C.c_int
    _lib = L
    return L


def check(rc: int, h=None, what: str = ""):
    if rc != GDEM_OK:
        msg = ""
        if h is not None and _lib is not None:
            m = _lib.gdem_last_error(h)
            msg = m.decode() if m else ""
        raise GdemError(f"{what}: {ERRORS.get(rc, rc)} {msg}".strip())
