"""gdem_sort_keys_noalloc (device pointers, fixed device scratch, nothing
allocated) against gdem_sort_keys through the C ABI.

Two calls in a row with different key sets and sizes (the second smaller, so
scratch left over from the first would show), an in-place call, the size
limit and n = 0.  This file is collected last so that it runs both alone and
after every other GPU test in one process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 20  # GDEM_SORT_NOALLOC_MAX_KEYS in include/gdem.h


def _vp(a):
    return a.ctypes.data_as(C.c_void_p)


def _sort_host(L, keys):
    n = keys.size
    ks = np.zeros(n, np.uint32)
    pm = np.zeros(n, np.int32)
    assert L.gdem_sort_keys(_vp(keys), n, _vp(ks), _vp(pm)) == 0
    return ks, pm


def _sort_noalloc(L, torch, keys, in_place=False):
    n = keys.size
    d_keys = torch.from_numpy(keys.view(np.int32)).cuda()
    d_sorted = d_keys if in_place else torch.empty(n, dtype=torch.int32, device="cuda")
    d_perm = torch.empty(n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.gdem_sort_keys_noalloc(C.c_void_p(d_keys.data_ptr()), n, C.c_void_p(d_sorted.data_ptr()),
                                  C.c_void_p(d_perm.data_ptr()), C.c_void_p(stream))
    assert rc == 0, rc
    torch.cuda.synchronize()
    return d_sorted.cpu().numpy().view(np.uint32), d_perm.cpu().numpy()


def _key_sets():
    rng = np.random.default_rng(2024)
    # Morton-like keys with many duplicates and the all-ones "inactive" key,
    # at the maximum size
    a = rng.integers(0, 1 << 12, MAX_KEYS, dtype=np.uint32) * np.uint32(977)
    a[rng.random(MAX_KEYS) < 0.01] = np.uint32(0xFFFFFFFF)
    # full-range 32-bit keys, smaller than the first call
    b = rng.integers(0, 1 << 32, 300_001, dtype=np.uint64).astype(np.uint32)
    return a, b


def test_noalloc_sort_matches_allocating_sort_twice_in_a_row():
    torch = pytest.importorskip("torch")
    from gpudem_gb300 import _lib
    L = _lib.load()
    a, b = _key_sets()
    for keys in (a, b):
        ks_ref, pm_ref = _sort_host(L, keys)
        ks, pm = _sort_noalloc(L, torch, keys)
        assert np.array_equal(ks, ks_ref)
        assert np.array_equal(pm, pm_ref)
        assert np.array_equal(pm, np.argsort(keys, kind="stable"))


def test_noalloc_sort_in_place_and_limits():
    torch = pytest.importorskip("torch")
    from gpudem_gb300 import _lib
    L = _lib.load()
    _, b = _key_sets()
    keys = b[:12_345].copy()
    ks_ref, pm_ref = _sort_host(L, keys)
    ks, pm = _sort_noalloc(L, torch, keys, in_place=True)
    assert np.array_equal(ks, ks_ref) and np.array_equal(pm, pm_ref)
    # n = 0 is a no-op; more keys than the scratch holds is refused before any launch
    assert L.gdem_sort_keys_noalloc(None, 0, None, None, None) == 0
    d = torch.empty(1, dtype=torch.int32, device="cuda")
    p = C.c_void_p(d.data_ptr())
    assert L.gdem_sort_keys_noalloc(p, MAX_KEYS + 1, p, p, None) == 3  # GDEM_ERR_CAPACITY
    assert L.gdem_sort_keys_noalloc(p, -1, p, p, None) == 1  # GDEM_ERR_ARG
