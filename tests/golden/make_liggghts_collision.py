"""Extract the LIGGGHTS 3.8.0 two-sphere collision that the reference keeps as
a physics check (liggghtsCases/testCases/in.collision and its dump.txt) into
tests/golden/liggghts_collision.json.  Run from the repository root where the
reference checkout exists:

    python tests/golden/make_liggghts_collision.py [reference root]

The fixture holds the input deck's parameters and, for a few dump frames, the
id, position, velocity and angular velocity of each sphere, as LIGGGHTS
printed them (6 significant digits).
"""
from __future__ import annotations

import json
import os
import re
import sys

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "liggghts_collision.json")
FRAMES = (0, 18000, 19000, 20000, 22000, 50000, 100000)


def parse_deck(text: str) -> dict:
    def num(pattern):
        return float(re.search(pattern, text, re.M).group(1))

    atoms = re.findall(r"^create_atoms 1 single (\S+) (\S+) (\S+)", text, re.M)
    vel = {int(i): [float(a), float(b), float(c)]
           for i, a, b, c in re.findall(r"^set atom (\d) vx (\S+) vy (\S+) vz (\S+)", text, re.M)}
    diam = {int(i): float(d) for i, d in re.findall(r"^set atom (\d) diameter (\S+)", text, re.M)}
    rho = {int(i): float(d) for i, d in re.findall(r"^set atom (\d) diameter \S+ density (\S+)", text, re.M)}
    return {
        "pair_style": re.search(r"^pair_style (.*)$", text, re.M).group(1).strip(),
        "x0": [[float(c) for c in a] for a in atoms],
        "v0": [vel[1], vel[2]],
        "diameter": [diam[1], diam[2]],
        "density": [rho[1], rho[2]],
        "characteristic_velocity": num(r"characteristicVelocity scalar (\S+)"),
        "youngs_modulus": num(r"youngsModulus peratomtype (\S+)"),
        "poisson_ratio": num(r"poissonsRatio peratomtype (\S+)"),
        "restitution": num(r"coefficientRestitution peratomtypepair 1 (\S+)"),
        "friction": num(r"coefficientFriction peratomtypepair 1 (\S+)"),
        "timestep": num(r"^timestep (\S+)"),
    }


def parse_dump(text: str) -> dict:
    frames = {}
    blocks = text.split("ITEM: TIMESTEP")[1:]
    for b in blocks:
        lines = b.strip().splitlines()
        step = int(lines[0])
        i = lines.index(next(l for l in lines if l.startswith("ITEM: ATOMS")))
        rows = [l.split() for l in lines[i + 1:] if l.strip()]
        frames[step] = {int(r[0]): [float(c) for c in r[1:10]] for r in rows}
    return frames


def main(ref_root: str) -> None:
    base = os.path.join(ref_root, "liggghtsCases", "testCases")
    with open(os.path.join(base, "in.collision")) as f:
        deck = parse_deck(f.read())
    with open(os.path.join(base, "dump.txt")) as f:
        frames = parse_dump(f.read())
    out = {
        "source": "liggghtsCases/testCases/in.collision, dump.txt (LIGGGHTS-PUBLIC 3.8.0)",
        "columns": ["x", "y", "z", "vx", "vy", "vz", "omegax", "omegay", "omegaz"],
        "deck": deck,
        "frames": {str(s): {str(i): frames[s][i] for i in sorted(frames[s])} for s in FRAMES},
    }
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    if len(sys.argv) > 1:
        root = sys.argv[1]
    else:
        sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
        from oracle.refharness import reference_dir
        root = reference_dir()
        if root is None:
            sys.exit("no reference checkout (set GDEM_REFERENCE_DIR or pass its root)")
    main(root)
