"""Snapshot files are checked on the host before a restart uploads anything
(gdem_check_snapshot, also the first step of gdem_load_snapshot).  The files
here are written in the snapshot layout by hand, so no GPU is needed: a sound
file passes, and a history key outside the particles or the mesh, a count
above the capacity, a truncated file and trailing bytes are refused."""
from __future__ import annotations

import struct

import numpy as np
import pytest

GDEM_OK, GDEM_ERR_ARG = 0, 1


def _snapshot_bytes(n=5, mixed=False, hist_cap=4, histw_cap=3, hist=None, histw=None):
    """Header (magic, version, n, precision, model, caps, per-particle flag,
    real size, steps, error word) then the state arrays and two histories."""
    rs = 4 if mixed else 8
    hd = b"GDEMSNAP" + struct.pack("<8iQ2I", 1, n, 1 if mixed else 0, 0, hist_cap, histw_cap, 0, rs, 7, 0, 0)
    assert len(hd) == 56
    state = bytes(n * (7 * 16 if mixed else 4 * 32))
    nterms = 6 if mixed else 3
    out = [hd, state]
    for h in (hist or {}, histw or {}):
        cnt = np.zeros(n, np.int32)
        ids = []
        for i, keys in sorted(h.items()):
            cnt[i] = len(keys)
            ids += keys
        out.append(cnt.tobytes())
        out.append(np.asarray(ids, np.int32).tobytes())
        out.append(bytes(len(ids) * nterms * rs))
    return b"".join(out)


@pytest.fixture(scope="module")
def L():
    from gpudem_gb300 import _lib
    return _lib.load()


@pytest.mark.parametrize("mixed", [False, True])
def test_sound_snapshot_passes(L, tmp_path, mixed):
    p = tmp_path / "s.snap"
    p.write_bytes(_snapshot_bytes(mixed=mixed, hist={0: [1, 4], 3: [2]}, histw={1: [0, 11]}))
    assert L.gdem_check_snapshot(str(p).encode(), 12) == GDEM_OK


@pytest.mark.parametrize("case", ["partner_high", "partner_negative", "triangle_outside", "count_over_cap",
                                  "truncated", "trailing", "bad_magic"])
def test_broken_snapshot_is_refused(L, tmp_path, case):
    kw = dict(hist={0: [1, 4], 3: [2]}, histw={1: [0, 11]})
    ntri = 12
    if case == "partner_high":
        kw["hist"] = {0: [1, 5]}           # n = 5: partner ids are 0..4
    elif case == "partner_negative":
        kw["hist"] = {2: [-1]}
    elif case == "triangle_outside":
        ntri = 11                           # triangle 11 is not in an 11-triangle mesh
    elif case == "count_over_cap":
        kw["hist"] = {0: [1, 2, 3, 4, 0]}  # 5 entries, capacity 4
    b = _snapshot_bytes(**kw)
    if case == "truncated":
        b = b[:-3]
    elif case == "trailing":
        b = b + b"\0"
    elif case == "bad_magic":
        b = b"GDEMSNAQ" + b[8:]
    p = tmp_path / "s.snap"
    p.write_bytes(b)
    assert L.gdem_check_snapshot(str(p).encode(), ntri) == GDEM_ERR_ARG


def test_missing_file_and_bad_arguments(L, tmp_path):
    assert L.gdem_check_snapshot(str(tmp_path / "absent").encode(), 0) == GDEM_ERR_ARG
    assert L.gdem_check_snapshot(None, 0) == GDEM_ERR_ARG
    p = tmp_path / "s.snap"
    p.write_bytes(_snapshot_bytes())
    assert L.gdem_check_snapshot(str(p).encode(), -1) == GDEM_ERR_ARG
