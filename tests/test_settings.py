"""The host side of the reference's main program: demSettings.json, the
"file" inlet's particle file and ASCII STL walls (gdem_settings_load /
_parse, gdem_read_particle_file, gdem_read_stl; gpudem_gb300/settings.py).

* Every demSettings.json the reference ships (tests/golden/settings_cases.json)
  is read: none has YoungModulus or bruteOn, which the reference's main.cu
  requires (main.cu:64, :72), so the reference itself stops on all of them.
* The derived constants against the reference's own initializeParticles
  (tests/golden/init_particles.npz, made by the reference harness), bit for
  bit: mass, stiffness, damping constant, moment of inertia.
* The file inlet, which the reference cannot start (its string getter takes
  only objects, cJSON_d.c:3226-3232), with the file name as a string and as
  an object.
* Errors name the missing key instead of aborting.  CPU only."""
from __future__ import annotations

import json
import math
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN

CASES = json.load(open(os.path.join(GOLDEN, "settings_cases.json")))
INIT = dict(np.load(os.path.join(GOLDEN, "init_particles.npz")))
PI_REF = 3.14159265359  # hardCodedParameters.h:6


def _json(text):
    """The shipped files write numbers such as "1000." (accepted by cJSON's
    strtod, not by strict JSON): read them the same way here."""
    return json.loads(re.sub(r"(\d)\.(?=\s*[,}\]])", r"\1.0", text))


def _dt(mass, k, dt_factor, output_timing):
    """main.cu:123-129: contact-time step snapped to the output interval."""
    dt = 2.0 * PI_REF * math.sqrt(mass / k) / dt_factor
    out_step = int(math.floor(output_timing / dt))
    return output_timing / out_step, out_step


@pytest.mark.parametrize("name", sorted(CASES))
def test_every_shipped_settings_file_reads(name):
    from gpudem_gb300 import scenes, settings
    raw = _json(CASES[name])
    st = settings.parse(CASES[name])
    p0 = raw["particleTypes"]["particle0"]
    assert (st["radius"], st["restitution"], st["density"], st["mu"]) == (p0["radius"], p0["CoR"], p0["density"],
                                                                          p0["mu"])
    assert "YoungModulus" not in p0 and math.isnan(st["youngs_modulus"])
    assert st["stiffness"] == p0["k"] == st["k_given"]
    assert st["brute_on"] == 0 and "bruteOn" not in raw["others"]
    assert st["gpu_on"] == raw["others"]["gpuOn"]
    assert st["n_particles"] == raw["inlet"]["numParticle"] and st["input_mode"] == raw["inlet"]["inputMode"]
    sh = raw["inlet"]["shuffle"]
    assert st["inlet_min"] == [sh["minx"], sh["miny"], sh["minz"]]
    assert st["inlet_max"] == [sh["maxx"], sh["maxy"], sh["maxz"]]
    assert st["walls"] == raw["walls"]["filepaths"]
    assert st["g"] == [raw["gravity"][a] for a in "xyz"]
    assert st["mass"] == float(scenes.sphere_mass(p0["density"], p0["radius"]))
    assert st["etaconst"] == float(scenes.eta_const(p0["k"], p0["CoR"]))
    dt, out_step = _dt(st["mass"], st["stiffness"], raw["others"]["dtFactor"], raw["others"]["outputTiming"])
    assert (st["dt"], st["out_step"]) == (dt, out_step)


@pytest.mark.parametrize("c", range(len(INIT["cases"])))
def test_derived_constants_match_the_reference_initialiser(c):
    """Mass (main.cu:67), stiffness (ParticleSystem.cu:202), damping constant
    (:301) from the settings reader and from scenes.py, and the moment of
    inertia and inverses the engine derives at import (2/5 m r^2, 1/m,
    sqrt(m)), against the reference's initializeParticles."""
    from gpudem_gb300 import scenes, settings
    r, rho, E, e = (float(a) for a in INIT["cases"][c])
    ref = {k: float(INIT[f"c{c}_{k}"]) for k in ("m", "k", "etaconst", "moi", "invmoi", "sqrtm", "invm")}
    text = json.dumps({
        "walls": {"filepaths": ["box.stl"]},
        "inlet": {"inputMode": "shuffle", "numParticle": 10,
                  "shuffle": {"minx": 0, "maxx": 1, "miny": 0, "maxy": 1, "minz": 0, "maxz": 1}},
        "particleTypes": {"particle0": {"density": rho, "radius": r, "CoR": e, "YoungModulus": E, "mu": 0.3}},
        "others": {"dtFactor": 15, "endTime": 1.0, "outputTiming": 0.01, "gpuOn": 1},
        "gravity": {"x": 0.0, "y": -9.81, "z": 0.0}})
    st = settings.parse(text)
    assert (st["mass"], st["stiffness"], st["etaconst"]) == (ref["m"], ref["k"], ref["etaconst"])
    assert float(scenes.sphere_mass(rho, r)) == ref["m"]
    assert scenes.stiffness_from_E(E, r) == ref["k"]
    assert float(scenes.eta_const(ref["k"], e)) == ref["etaconst"]
    m = ref["m"]
    moi = 2.0 / 5.0 * m * (r * r)
    assert moi == ref["moi"] and 1.0 / moi == ref["invmoi"]
    assert 1.0 / m == ref["invm"] and math.sqrt(m) == ref["sqrtm"]


def _box_stl(path, tris):
    with open(path, "w") as f:
        f.write("solid box\n")
        for t in tris:
            f.write("  facet normal 0 0 0\n    outer loop\n")
            for c in t:
                f.write("      vertex %.17g %.17g %.17g\n" % tuple(c))
            f.write("    endloop\n  endfacet\n")
        f.write("endsolid box\n")


@pytest.mark.parametrize("form", ["string", "object"])
def test_file_inlet_and_walls_make_a_scene(tmp_path, form):
    from gpudem_gb300 import scenes, settings
    tris = scenes.box_mesh(0.1)
    _box_stl(tmp_path / "box.stl", tris)
    rng = np.random.default_rng(5)
    n = 50
    x = scenes.random_packing(n, np.full(n, 0.005), [-0.05, 0.0, -0.05], [0.05, 0.05, 0.05], rng)
    v = rng.normal(0, 0.1, (n, 3))
    with open(tmp_path / "parts.csv", "w") as f:
        f.write("vx,vy,vz,x,y,z\n")       # columns in any order, by name
        for i in range(n):
            f.write(",".join("%.17g" % a for a in (*v[i], *x[i])) + "\n")
    raw = _json(CASES["demSettings.json"])
    raw["walls"]["filepaths"] = ["box.stl"]
    raw["inlet"].update({"inputMode": "file", "numParticle": n,
                         "file": "parts.csv" if form == "string" else {"name": "parts.csv"}})
    (tmp_path / "demSettings.json").write_text(json.dumps(raw))
    sc, counts, st = settings.scene(str(tmp_path / "demSettings.json"))
    assert st["input_mode"] == "file" and st["particle_file"] == "parts.csv"
    assert np.array_equal(sc.x, x) and np.array_equal(sc.v, v)
    assert np.array_equal(sc.inlet_lo, x.min(0)) and np.array_equal(sc.inlet_hi, x.max(0))
    assert np.array_equal(sc.tris, tris) and list(counts) == [12]
    assert np.all(sc.k == st["stiffness"]) and np.all(sc.m == st["mass"]) and sc.dt == st["dt"]


def test_shuffle_inlet_scene(tmp_path):
    from gpudem_gb300 import scenes, settings
    _box_stl(tmp_path / "simpleBox.stl", scenes.box_mesh(0.5))
    raw = _json(CASES["cases/10000Particles_spiral/demSettings.json"])
    raw["walls"]["filepaths"] = ["simpleBox.stl"]
    (tmp_path / "demSettings.json").write_text(json.dumps(raw))
    sc, counts, st = settings.scene(str(tmp_path / "demSettings.json"))
    r = raw["particleTypes"]["particle0"]["radius"]
    assert sc.n == raw["inlet"]["numParticle"]
    spatial = pytest.importorskip("scipy.spatial")
    d, _ = spatial.cKDTree(sc.x).query(sc.x, k=2)
    assert d[:, 1].min() >= 2 * r                         # no two closer than 2 r (ParticleSystem.cu:262)
    assert np.all(sc.x >= sc.inlet_lo) and np.all(sc.x <= sc.inlet_hi)


@pytest.mark.parametrize("edit,key", [
    (lambda d: d["particleTypes"]["particle0"].pop("radius"), "particleTypes.particle0.radius"),
    (lambda d: d["particleTypes"]["particle0"].pop("k"), "YoungModulus or k"),
    (lambda d: d["others"].pop("dtFactor"), "others.dtFactor"),
    (lambda d: d["others"].__setitem__("gpuOn", "yes"), "others.gpuOn"),
    (lambda d: d.pop("gravity"), "gravity"),
    (lambda d: d["walls"].__setitem__("filepaths", "box.stl"), "walls.filepaths"),
    (lambda d: d["inlet"].__setitem__("inputMode", "files"), "inlet.inputMode"),
    (lambda d: d["inlet"].pop("shuffle"), "inlet.shuffle"),
    (lambda d: (d["inlet"].__setitem__("inputMode", "file"), d["inlet"].pop("file")), "inlet.file"),
])
def test_errors_name_the_key(edit, key):
    from gpudem_gb300 import _lib, settings
    raw = _json(CASES["demSettings.json"])
    edit(raw)
    with pytest.raises(_lib.GdemError, match=key.replace(".", r"\.")):
        settings.parse(json.dumps(raw))


@pytest.mark.parametrize("text", ["", "{", "{\"a\": }", "[1, 2]", "{\"a\": 1} x", "{\"a\": 01x}"])
def test_malformed_json_is_refused(text):
    from gpudem_gb300 import _lib, settings
    with pytest.raises(_lib.GdemError, match="GDEM_ERR_ARG"):
        settings.parse(text)


def test_particle_file_with_the_wrong_row_count_is_refused(tmp_path):
    from gpudem_gb300 import _lib, settings
    (tmp_path / "p.csv").write_text("x,y,z,vx,vy,vz\n0,0,0,0,0,0\n1,1,1,0,0,0\n")
    with pytest.raises(_lib.GdemError):
        settings.read_particle_file(str(tmp_path / "p.csv"), 3)
    x, v, lo, hi = settings.read_particle_file(str(tmp_path / "p.csv"), 2)
    assert np.array_equal(lo, [0, 0, 0]) and np.array_equal(hi, [1, 1, 1])
