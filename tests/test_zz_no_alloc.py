"""SortUsingThrustNoAlloc through the C-ABI: the same stable order as SortUsingThrust,
from its static device scratch, on two calls in a row (the second reuses the array the
first left behind), and a clear rejection above its 262,144-key limit.  Collected
last so that a failure here cannot stop the other GPU tests."""
import ctypes as C

import numpy as np
import pytest

from simulation_project_gb300 import lib
from simulation_project_gb300.lib import DeviceArray

pytestmark = pytest.mark.gpu
LIMIT = 262144


def _fn():
    f = lib.load().SortUsingThrustNoAlloc
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    return f


def _sorted_pair(fn, keys):
    n = len(keys)
    dk = DeviceArray.from_host(keys)
    dv = DeviceArray.from_host(np.arange(n, dtype=np.int32))
    rc = fn(n, dk.ptr, dv.ptr)
    return rc, dk.download(), dv.download()


def test_no_alloc_sort_matches_sort_using_thrust_on_consecutive_calls():
    noalloc = _fn()
    reference = lib.load().SortUsingThrust
    rng = np.random.default_rng(11)
    cases = [rng.integers(0, 1 << 17, size=LIMIT, dtype=np.int64).astype(np.int32),
             rng.integers(-(1 << 30), 1 << 30, size=70001, dtype=np.int64).astype(np.int32)]
    for keys in cases:
        rc0, k0, v0 = _sorted_pair(reference, keys)
        rc1, k1, v1 = _sorted_pair(noalloc, keys)
        assert rc0 == 0 and rc1 == 0
        assert np.array_equal(k0, k1) and np.array_equal(v0, v1)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(v1, order)


def test_no_alloc_sort_rejects_more_keys_than_its_scratch_holds():
    noalloc = _fn()
    keys = np.arange(16, dtype=np.int32)[::-1].copy()
    dk = DeviceArray.from_host(keys)
    dv = DeviceArray.from_host(np.arange(16, dtype=np.int32))
    assert noalloc(LIMIT + 1, dk.ptr, dv.ptr) == 2          # CCT_PARAMERR, nothing launched
    assert b"262144" in lib.load().mps_last_error()
    assert np.array_equal(dk.download(), keys)
