"""ctypes binding of libmps_gb300.so (the GB300 CUDA library).

The library is built in-tree by simulation_project_gb300.build (or
__graft_entry__.build()).  There is no CPU fallback: load() raises if the library is
missing, and every wrapped entry point raises MpsError on a non-zero status.
"""
import ctypes as C
import os

import numpy as np

from .types import (CParameter, CGridBox, MpsError, check)

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libmps_gb300.so")
P = C.c_void_p
I = C.c_int

_SIGS = {
    # runtime helpers (include/mps_runtime.h)
    "mps_device_count": (I, [C.POINTER(I)]),
    "mps_device_sm_count": (I, [C.POINTER(I)]),
    "mps_set_device": (I, [I]),
    "mps_malloc": (I, [C.POINTER(P), C.c_size_t]),
    "mps_free": (I, [P]),
    "mps_memset": (I, [P, I, C.c_size_t]),
    "mps_memcpy_htod": (I, [P, P, C.c_size_t]),
    "mps_memcpy_dtoh": (I, [P, P, C.c_size_t]),
    "mps_memcpy_dtod": (I, [P, P, C.c_size_t]),
    "mps_host_alloc_pinned": (I, [C.POINTER(P), C.c_size_t]),
    "mps_host_free_pinned": (I, [P]),
    "mps_stream_create": (I, [C.POINTER(P)]),
    "mps_stream_destroy": (I, [P]),
    "mps_stream_sync": (I, [P]),
    "mps_device_sync": (I, []),
    "mps_event_create": (I, [C.POINTER(P)]),
    "mps_event_destroy": (I, [P]),
    "mps_event_record": (I, [P, P]),
    "mps_event_elapsed_ms": (I, [P, P, C.POINTER(C.c_float)]),
    "mps_last_error": (C.c_char_p, []),
    "mps_clear_error": (None, []),
    "mps_scratch_bytes": (C.c_size_t, []),
    "mps_build_info": (C.c_char_p, []),
    "mps_kernel_launches": (C.c_ulonglong, []),
    # reference-named launcher API (include/mps_device_process.h)
    "CalcTurbulenceViscosity": (I, [C.POINTER(P), I]),
    "CheckParticleOutsideComputeZone": (I, [C.POINTER(P), C.POINTER(I)]),
    "CalcDragEffect": (I, [C.POINTER(P), I]),
    "CalcExplicitly": (I, [C.POINTER(P), I]),
    "CalcExplicitPressure": (I, [C.POINTER(P), I]),
    "CalcExplicitPressureGradient": (I, [C.POINTER(P), I]),
    "CalcTemperatureFactor": (I, [C.POINTER(P), I]),
    "RegisterTriangleTopology": (I, [C.POINTER(P), P, I, P, I]),
    "ResetTriangleTopology": (I, [C.POINTER(P), I, P]),
    "ResetWallPosition": (I, [C.POINTER(P), I, I, P]),
    "UpdateTrianglePosition": (I, [C.POINTER(P), I, P]),
    "RotateTrianglePosition": (I, [C.POINTER(P), I, P, I]),
    "CalcSTLDistance": (I, [C.POINTER(P), I]),
    "CaculateCellIDandInitializeHash": (I, [C.POINTER(P), I, I, P, P, P]),
    "reorderDataAndFindCellStart": (I, [C.POINTER(P), I, I, P, P, P, P]),
    "SortUsingThrust": (I, [I, P, P]),
    "StableSortUsingThrust": (I, [I, P, P]),
    "InitializeDeviceMemConst": (I, [CParameter, I, P, I, P, I, P, P, P, I, P, P, P, CGridBox]),
    "InitializeDeviceConstOutPutParticles": (I, [P] * 9),
    "InitializeDeviceConstInputParticles": (I, [P] * 11),
    "ParticleNumberToConst": (I, [I]),
    "DragParametersToConst": (I, [P, P, P, I, P, P]),
}

_lib = None


def exported_symbols():
    """Names this binding expects the library to export."""
    return list(_SIGS.keys())


def load(path: str = LIB_PATH):
    """Loads the library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m simulation_project_gb300.build` "
                           "(no CPU fallback exists)")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def call(name: str, *args):
    st = getattr(load(), name)(*args)
    if st != 0:
        raise MpsError(st, f"{name} ({load().mps_last_error().decode()})")
    return st


def kernel_launches() -> int:
    """Kernels the library has launched since it was loaded."""
    return int(load().mps_kernel_launches())


class DeviceArray:
    """A device allocation mirrored by a numpy dtype/shape (test and bench helper)."""

    def __init__(self, shape, dtype):
        self.shape = tuple(shape) if isinstance(shape, (tuple, list)) else (int(shape),)
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        p = P()
        call("mps_malloc", C.byref(p), max(self.nbytes, 1))
        self.ptr = p.value

    @classmethod
    def from_host(cls, a: np.ndarray):
        a = np.ascontiguousarray(a)
        d = cls(a.shape, a.dtype)
        d.upload(a)
        return d

    def upload(self, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=self.dtype)
        assert a.nbytes <= self.nbytes
        if a.nbytes:
            call("mps_memcpy_htod", self.ptr, a.ctypes.data, a.nbytes)

    def download(self) -> np.ndarray:
        out = np.empty(self.shape, self.dtype)
        if self.nbytes:
            call("mps_memcpy_dtoh", out.ctypes.data, self.ptr, self.nbytes)
        return out

    def fill_bytes(self, value: int):
        call("mps_memset", self.ptr, value, self.nbytes)

    def free(self):
        if self.ptr:
            load().mps_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Stream:
    def __init__(self):
        p = P()
        call("mps_stream_create", C.byref(p))
        self.handle = P(p.value)

    def ref(self):
        return C.byref(self.handle)

    def sync(self):
        call("mps_stream_sync", self.handle)

    def __del__(self):
        try:
            if self.handle:
                load().mps_stream_destroy(self.handle)
        except Exception:
            pass


class Event:
    def __init__(self):
        p = P()
        call("mps_event_create", C.byref(p))
        self.handle = p.value

    def record(self, stream=None):
        call("mps_event_record", self.handle, stream.handle if stream is not None else None)

    def elapsed_ms(self, later) -> float:
        ms = C.c_float()
        call("mps_event_elapsed_ms", self.handle, later.handle, C.byref(ms))
        return float(ms.value)


def gpu_available() -> bool:
    try:
        n = I()
        return load().mps_device_count(C.byref(n)) == 0 and n.value > 0
    except Exception:
        return False
