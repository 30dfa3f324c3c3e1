"""Collect the demSettings.json files the reference ships (its top-level
file and cases/*/demSettings.json) into tests/golden/settings_cases.json, as
inputs for the settings reader's tests.  Run from the repository root where
the reference checkout exists:

    python tests/golden/make_settings_cases.py [reference root]
"""
from __future__ import annotations

import glob
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "settings_cases.json")


def main(ref):
    files = [os.path.join(ref, "demSettings.json")] + sorted(glob.glob(os.path.join(ref, "cases", "*",
                                                                                     "demSettings.json")))
    out = {}
    for f in files:
        name = os.path.relpath(f, ref)
        with open(f) as fh:
            out[name] = fh.read()
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=1)
    print(f"wrote {OUT}: {len(out)} files")


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main(sys.argv[1])
    else:
        sys.path.insert(0, ROOT)
        from oracle.refharness import reference_dir
        ref = reference_dir()
        if ref is None:
            sys.exit("no reference checkout (set GDEM_REFERENCE_DIR or pass its root)")
        main(ref)
