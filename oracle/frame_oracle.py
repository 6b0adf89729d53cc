"""CPU oracle of the reference's output frames (test infrastructure only).

A restatement of IO::SaveAscii and IO::SaveBinary,
radix/SPVSOLVER/MultiGPUSolver/IO.cpp:670-756, used by tests/test_frames.py to check
the library's writer byte for byte:

* ASCII (:674-709): the particle count; per particle the twelve values
  "x y z vx vy vz P n T nu solidRate type" separated by single spaces, written by a
  std::ostream with default flags (each float printed like printf's %g, six
  significant digits; the ParticleType enum as its integer); the current time; the
  model count; per model "x<TAB>y<TAB>z<TAB>angle".  Every line ends with a newline.
* Binary (:717-753): int32 count; per particle the float32 position (3), velocity (3),
  pressure, density, temperature, viscosity, solid rate and the int32 type; the
  float32 time; int32 model count; per model the float32 position (3) and angle.
"""
import struct

import numpy as np


def _g(v) -> str:
    return "%g" % float(v)


def frame_bytes(ascii: bool, pos, vel, pressure, density, temperature, viscosity, solid, ptype, time,
                model_pos, model_angle) -> bytes:
    n = len(pressure)
    f32 = lambda a: np.asarray(a, dtype=np.float32)
    pos, vel = f32(pos).reshape(n, 3), f32(vel).reshape(n, 3)
    pressure, density, temperature, viscosity, solid = map(f32, (pressure, density, temperature, viscosity, solid))
    ptype = np.asarray(ptype, dtype=np.int32)
    model_pos = f32(model_pos).reshape(-1, 3)
    model_angle = f32(model_angle)
    time = np.float32(time)
    if ascii:
        out = [f"{n}\n"]
        for i in range(n):
            vals = [*pos[i], *vel[i], pressure[i], density[i], temperature[i], viscosity[i], solid[i]]
            out.append(" ".join(_g(v) for v in vals) + f" {int(ptype[i])}\n")
        out.append(_g(time) + "\n")
        out.append(f"{len(model_angle)}\n")
        for m in range(len(model_angle)):
            out.append("\t".join(_g(v) for v in (*model_pos[m], model_angle[m])) + "\n")
        return "".join(out).encode()
    b = [struct.pack("<i", n)]
    for i in range(n):
        b.append(struct.pack("<3f3f5fi", *pos[i], *vel[i], pressure[i], density[i], temperature[i],
                             viscosity[i], solid[i], int(ptype[i])))
    b.append(struct.pack("<f", time))
    b.append(struct.pack("<i", len(model_angle)))
    for m in range(len(model_angle)):
        b.append(struct.pack("<4f", *model_pos[m], model_angle[m]))
    return b"".join(b)
