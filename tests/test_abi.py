"""The C-ABI library builds, loads without a GPU and exports every entry
point include/gdem.h declares (no compute calls here)."""
from __future__ import annotations

import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "gdem.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(gdem_[a-z_0-9]+)\s*\(", hdr)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "gdem_step" in syms and "gdem_create" in syms and len(syms) >= 15


def test_library_exports_every_declared_symbol():
    from gpudem_gb300 import _build, _lib
    path = _build.build_engine()
    L = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    assert set(_lib.EXPORTED) <= set(declared_symbols())


def test_binding_fails_loudly_without_library(tmp_path, monkeypatch):
    from gpudem_gb300 import _build, _lib
    monkeypatch.setattr(_build, "LIB", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    try:
        _lib.load()
    except _lib.GdemError as e:
        assert "not built" in str(e)
    else:
        raise AssertionError("load() must raise when libgdem.so is missing")
