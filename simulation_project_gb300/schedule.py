"""The dt schedule of the reference (DtFrame.cpp, CheckAndUpdateDt in
MultiGPUHandler.cpp) through the library: read_dt_file() and schedule_next()."""
import ctypes as C

import numpy as np

from . import lib
from .types import MpsError

ROW = np.dtype([("step", "<i4"), ("dt", "<f4"), ("courant", "<f4"), ("inflow_step", "<f4"), ("output_step", "<f4")])

_bound = False


def _L():
    global _bound
    L = lib.load()
    if not _bound:
        P = C.c_void_p
        L.mps_read_dt_file.restype = C.c_int
        L.mps_read_dt_file.argtypes = [C.c_char_p, C.POINTER(C.c_int), P, C.c_int]
        L.mps_dt_schedule_next.restype = C.c_int
        L.mps_dt_schedule_next.argtypes = [P, C.c_int, C.POINTER(C.c_int), C.c_int, P, C.POINTER(C.c_int)]
        _bound = True
    return L


def read_dt_file(path) -> np.ndarray:
    L = _L()
    n = C.c_int()
    st = L.mps_read_dt_file(str(path).encode(), C.byref(n), None, 0)
    if st:
        raise MpsError(st, "mps_read_dt_file")
    rows = np.zeros(max(n.value, 1), ROW)
    st = L.mps_read_dt_file(str(path).encode(), C.byref(n), rows.ctypes.data, len(rows))
    if st:
        raise MpsError(st, "mps_read_dt_file")
    return rows[:n.value]


def schedule_next(rows: np.ndarray, nxt: int, current_step: int, param) -> tuple:
    """Applies the next due row to param (a CParameter); returns (next, applied)."""
    L = _L()
    rows = np.ascontiguousarray(rows, ROW)
    k, a = C.c_int(nxt), C.c_int()
    st = L.mps_dt_schedule_next(rows.ctypes.data if len(rows) else None, len(rows), C.byref(k), int(current_step),
                                C.addressof(param), C.byref(a))
    if st:
        raise MpsError(st, "mps_dt_schedule_next")
    return k.value, bool(a.value)
