"""Output frames of the reference's format (IO::Save, radix/SPVSOLVER/MultiGPUSolver/
IO.cpp:649-756) through the library: write_frame() for host arrays, read_frame() to
load one back, and Solver.save_frame() (solver.py) for the device state."""
import ctypes as C

import numpy as np

from . import lib
from .types import MpsError

# binary per-particle record: position, velocity, pressure, density, temperature,
# viscosity, solid rate, type
RECORD = np.dtype([("pos", "<f4", 3), ("vel", "<f4", 3), ("pressure", "<f4"), ("density", "<f4"),
                   ("temperature", "<f4"), ("viscosity", "<f4"), ("solid", "<f4"), ("type", "<i4")])

_bound = False


def _fn():
    global _bound
    L = lib.load()
    f = L.mps_write_frame
    if not _bound:
        P = C.c_void_p
        f.restype = C.c_int
        f.argtypes = [C.c_char_p, C.c_int, C.c_int, P, P, P, P, P, P, P, P, C.c_float, C.c_int, P, P]
        _bound = True
    return f


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(shape) if shape is not None else a


def write_frame(path, ascii, pos, vel, pressure, density, viscosity, ptype, time=0.0, model_pos=None,
                model_angle=None, temperature=None, solid=None):
    """Writes one frame (arrays in output order); temperature / solid None: zeros."""
    n = len(pressure)
    pos, vel = _f32(pos, (n, 3)), _f32(vel, (n, 3))
    pressure, density, viscosity = _f32(pressure), _f32(density), _f32(viscosity)
    ptype = np.ascontiguousarray(ptype, dtype=np.int32)
    temperature = None if temperature is None else _f32(temperature)
    solid = None if solid is None else _f32(solid)
    mp = _f32(np.zeros((0, 3)) if model_pos is None else model_pos, (-1, 3))
    ma = _f32(np.zeros(0) if model_angle is None else model_angle)
    p = lambda a: None if a is None else a.ctypes.data
    st = _fn()(str(path).encode(), int(bool(ascii)), n, p(pos), p(vel), p(pressure), p(density), p(temperature),
               p(viscosity), p(solid), p(ptype), float(time), len(ma), p(mp), p(ma))
    if st != 0:
        raise MpsError(st, "mps_write_frame")


def read_frame(path, ascii):
    """Loads a frame: (records (RECORD dtype), time, model positions (m, 3), angles (m,))."""
    if ascii:
        lines = open(path).read().split("\n")
        n = int(lines[0])
        rec = np.zeros(n, RECORD)
        for i in range(n):
            v = lines[1 + i].split(" ")
            rec[i] = ((float(v[0]), float(v[1]), float(v[2])), (float(v[3]), float(v[4]), float(v[5])),
                      float(v[6]), float(v[7]), float(v[8]), float(v[9]), float(v[10]), int(v[11]))
        time = float(lines[1 + n])
        m = int(lines[2 + n])
        mv = np.array([[float(x) for x in lines[3 + n + k].split("\t")] for k in range(m)], np.float32).reshape(m, 4)
        return rec, time, mv[:, :3], mv[:, 3]
    raw = open(path, "rb").read()
    n = int(np.frombuffer(raw, "<i4", 1)[0])
    rec = np.frombuffer(raw, RECORD, n, 4).copy()
    o = 4 + n * RECORD.itemsize
    time = float(np.frombuffer(raw, "<f4", 1, o)[0])
    m = int(np.frombuffer(raw, "<i4", 1, o + 4)[0])
    mv = np.frombuffer(raw, "<f4", 4 * m, o + 8).reshape(m, 4)
    return rec, time, mv[:, :3].copy(), mv[:, 3].copy()
