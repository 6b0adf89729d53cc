"""CPU restatement of the reference's configuration-file and drag-file readers (test
infrastructure only: the checker of include/mps_io.h's mps_read_configuration and
mps_read_drag_file, never the product).

  read_configuration  CConfiguration::ReadConfigurationFileWithDrag,
                      radix/SPVSOLVER/MultiGPUSolver/Configuration.cpp:21-452
  read_drag_records   IO::Load(drag file), radix/SPVSOLVER/MultiGPUSolver/IO.cpp:524-564
  model_parameters    the per-model CTriangleParameters, MultiGPUHandler.cpp:466-555

The reference reads each field with `stream >> value`; IStream below restates those
extraction rules (skip whitespace; an integer is [sign]digits, a float
[sign]digits[.digits][(e|E)[sign]digits]; a field that does not parse stores 0 and puts
the stream in a failed state in which later reads leave their variables unchanged; a
bool is read as an integer, 0 or 1, anything else stores true and fails).  Lines end at
LF and a CR before it is dropped (the reference runs on Windows, in text mode).
Where the reference leaves a value uninitialised (a wall line without a temperature,
a DF drag line without a V token) this restatement uses 0, as the library does.
"""
import ctypes

import numpy as np

_libc = ctypes.CDLL(None)
_libc.strtof.restype = ctypes.c_float
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]

WS = " \t\n\r\v\f"


class IStream:
    def __init__(self, text: str):
        self.s = text
        self.i = 0
        self.fail = False
        self.eof = False

    def _sentry(self):
        if self.fail or self.eof:
            self.fail = True
            return False
        while self.i < len(self.s) and self.s[self.i] in WS:
            self.i += 1
        if self.i >= len(self.s):
            self.eof = True
            self.fail = True
            return False
        return True

    def _end(self):
        if self.i >= len(self.s):
            self.eof = True

    def word(self, default=""):
        if not self._sentry():
            return default
        j = self.i
        while j < len(self.s) and self.s[j] not in WS:
            j += 1
        tok = self.s[self.i:j]
        self.i = j
        self._end()
        return tok

    def _digits(self, j):
        k = j
        while k < len(self.s) and self.s[k].isdigit():
            k += 1
        return k

    def int(self, default=0):
        if not self._sentry():
            return default
        j = self.i
        if j < len(self.s) and self.s[j] in "+-":
            j += 1
        k = self._digits(j)
        if k == j:
            self.i = k
            self.fail = True
            self._end()
            return 0
        v = int(self.s[self.i:k])
        self.i = k
        self._end()
        if not -2 ** 31 <= v < 2 ** 31:
            self.fail = True
            return 2 ** 31 - 1 if v > 0 else -2 ** 31
        return v

    def float(self, default=0.0):
        if not self._sentry():
            return default
        j = self.i
        if j < len(self.s) and self.s[j] in "+-":
            j += 1
        k = self._digits(j)
        nd = k - j
        if k < len(self.s) and self.s[k] == ".":
            k2 = self._digits(k + 1)
            nd += k2 - (k + 1)
            k = k2
        if nd > 0 and k < len(self.s) and self.s[k] in "eE":
            e = k + 1
            if e < len(self.s) and self.s[e] in "+-":
                e += 1
            e2 = self._digits(e)
            k = e2 if e2 > e else e
        tok = self.s[self.i:k]
        self.i = k
        self._end()
        if nd == 0:
            self.fail = True
            return 0.0
        end = ctypes.c_char_p()
        v = _libc.strtof(tok.encode(), ctypes.byref(end))
        return float(np.float32(v))

    def bool(self, default=False):
        if not self._sentry():
            return default
        save_fail = self.fail
        v = self.int(None)
        if v is None:
            return default
        if self.fail and not save_fail:
            return True if v != 0 else False
        if v in (0, 1):
            return bool(v)
        self.fail = True
        return True


def _lines(text: str):
    out = []
    for ln in text.split("\n"):
        out.append(ln[:-1] if ln.endswith("\r") else ln)
    return out


def _f32(x):
    return float(np.float32(x))


def _wall_model(name, first, st):
    m = _model_defaults(name)
    m["velocity"] = [_f32(float(first)), 0.0, 0.0]   # boost::lexical_cast<float>
    m["velocity"][1] = st.float(0.0)
    m["velocity"][2] = st.float(0.0)
    m["temperature"] = st.float(0.0)
    m["position"] = tuple(st.float(0.0) for _ in range(3))
    m["linear_movable"] = int(st.bool(False))
    m["reset_interval"] = st.int(0)
    m["rotating"] = int(st.bool(False))
    m["rpm"] = st.int(0)
    m["rotation_start"] = st.float(0.0)
    m["time_to_reach_rpm"] = st.float(0.0)
    m["center_of_rotation"] = tuple(st.float(0.0) for _ in range(3))
    m["second_point_of_rotation"] = tuple(st.float(0.0) for _ in range(3))
    m["wall_friction"] = st.float(0.0)
    m["wall_thermal_resistivity"] = st.float(0.0)
    m["wall_thermal_conductivity"] = st.float(0.0)
    m["negative_pressure_check"] = int(st.bool(False))
    m["influence_region"] = st.float(0.0)
    m["direction"] = tuple(st.float(0.0) for _ in range(3))
    m["pressure_gas"] = st.float(0.0)
    m["velocity"] = tuple(m["velocity"])
    return m


DRAG_FIELDS = ["DragID", "DragToken", "InputVelocityToken1", "OutputVelocityToken2", "CoefficientofInflueneRegion",
               "VelocityIndex", "VelocityExponential", "VelocityDragPermiabilityConstant", "TempIndex",
               "TempExponential", "TempDragPermiabilityConstant", "ConstantVx", "ConstantVy", "ConstantVz",
               "VelocityMagnitueFactor"]


def _model_defaults(name):
    z3 = (0.0, 0.0, 0.0)
    return {"file": name, "is_drag": 0, "drag_id": -1, "velocity": z3, "temperature": 0.0, "position": z3,
            "linear_movable": 0, "reset_interval": 0, "rotating": 0, "rpm": 0, "rotation_start": 0.0,
            "time_to_reach_rpm": 0.0, "center_of_rotation": z3, "second_point_of_rotation": z3,
            "wall_friction": 0.0, "wall_thermal_resistivity": 0.0, "wall_thermal_conductivity": 0.0,
            "negative_pressure_check": 0, "influence_region": 0.0, "direction": z3, "pressure_gas": 0.0,
            "drag": {k: (0 if k == "DragID" else "" if "Token" in k else 0.0) for k in DRAG_FIELDS}}


def _drag_model(name, mode, drag_id, st):
    """Configuration.cpp:86-274."""
    m = _model_defaults(name)
    d = m["drag"]
    m["is_drag"], m["drag_id"], d["DragID"] = 1, drag_id, drag_id
    tin = st.word("").upper()
    st.word("")   # output token, read and not used
    d["CoefficientofInflueneRegion"] = st.float(0.0)
    if mode in ("D", "DE"):
        d["DragToken"] = "E"
        if tin == "V":
            d["InputVelocityToken1"] = d["OutputVelocityToken2"] = "V"
            for k in ("VelocityIndex", "VelocityExponential", "VelocityDragPermiabilityConstant"):
                d[k] = st.float(0.0)
        elif tin == "T":
            d["InputVelocityToken1"] = d["OutputVelocityToken2"] = "T"
            for k in ("TempIndex", "TempExponential", "TempDragPermiabilityConstant"):
                d[k] = st.float(0.0)
        else:   # `inputToken == "VT" || "TV"` (Configuration.cpp:143) is always true
            d["InputVelocityToken1"] = d["OutputVelocityToken2"] = "B"
            for k in ("VelocityIndex", "VelocityExponential", "VelocityDragPermiabilityConstant", "TempIndex",
                      "TempExponential", "TempDragPermiabilityConstant"):
                d[k] = st.float(0.0)
    if mode == "DF":
        d["DragToken"] = "F"
        if tin == "V":
            d["InputVelocityToken1"] = d["OutputVelocityToken2"] = "V"
            d["VelocityMagnitueFactor"] = st.float(0.0)
    elif mode == "DC":
        d["InputVelocityToken1"] = d["OutputVelocityToken2"] = "V"
        d["DragToken"] = "C"
        for k in ("ConstantVx", "ConstantVy", "ConstantVz"):
            d[k] = st.float(0.0)
    m["temperature"] = 533.0
    return m


def read_configuration(text: str) -> dict:
    """Configuration.cpp:21-452 on the file's text (latin-1 decoded)."""
    lines = _lines(text)
    pos = [0]

    def getline():
        if pos[0] < len(lines) and not (pos[0] == len(lines) - 1 and lines[pos[0]] == "" and text.endswith("\n")):
            ln = lines[pos[0]]
            pos[0] += 1
            return ln
        pos[0] = len(lines)
        return ""

    cfg = {"input_path": getline(), "parameter_file": getline(), "particle_file": getline()}
    buckets = []
    line = getline()
    while line:
        st = IStream(line)
        name = st.word("")
        buckets.append({"file": name, "interval": st.int(0), "total_steps": st.int(0)})
        line = getline()
    models = []
    drags = 0
    line = getline()
    while line:
        st = IStream(line)
        name = st.word("")
        mode = st.word("").upper()
        if mode in ("D", "DE", "DC", "DF"):
            models.append(_drag_model(name, mode, drags, st))
            drags += 1
        else:
            try:
                float(mode)
            except ValueError:
                raise ValueError(f"model line of {name}: {mode!r} is not a number")
            models.append(_wall_model(name, mode, st))
        line = getline()
    cfg["output_path"] = getline()
    cfg["output_name"] = getline()
    cfg["output_interval"] = IStream(getline()).int(0)
    st = IStream(getline())
    lo = tuple(st.float(0.0) for _ in range(3))
    hi = tuple(st.float(0.0) for _ in range(3))
    ok = all(abs(_f32(h - l)) != 0.0 for l, h in zip(lo, hi))
    cfg["compute_zone"] = (lo, hi) if ok else None
    st = IStream(getline())
    cfg["section"] = tuple(st.int(0) for _ in range(3))
    cfg["start_step"] = IStream(getline()).int(0)
    cfg["output_ascii"] = 0 if IStream(getline()).word("").upper() == "BINARY" else 1
    cfg.update({"buckets": buckets, "models": models, "bucket_count": len(buckets), "model_count": len(models),
                "drag_count": drags, "has_compute_zone": 1 if ok else 0})
    return cfg


def model_parameters(models, dt: float):
    """MultiGPUHandler.cpp:466-555: AngleOfRotationInDegree = RPM * Dt * 6 in float."""
    out = []
    for m in models:
        rpm_dt = np.float32(np.float32(m["rpm"]) * np.float32(dt))
        out.append({"AngleOfRotationInDegree": float(np.float32(rpm_dt * np.float32(6))),
                    "RotationInRPM": float(np.float32(m["rpm"])), "isDrag": bool(m["is_drag"]),
                    "DragTriangleID": m["drag_id"], "LinearMovableOrNot": bool(m["linear_movable"]),
                    "LinearResetInterval": m["reset_interval"], "RotatingOrNot": bool(m["rotating"]),
                    "Temperature": m["temperature"], "WallFrictionCoefficient": m["wall_friction"]})
    return out


def join(directory: str, name: str) -> str:
    """Configuration.cpp:646-825: '\\\\' appended unless the path ends with '/' or '\\\\'."""
    if not directory:
        return name
    return directory + ("" if directory[-1] in "/\\" else "\\") + name


def read_drag_records(text: str):
    """IO.cpp:524-564: (root, inner-pressure name, [(file, DragLength, StartStep01,
    StartStep02, EndStep, InitialAcc, GradAcc)]).  A record counts only if the stream is
    good after its last field; a field that does not parse ends the records (the
    reference would loop forever there)."""
    st = IStream(text)
    root = st.word("")
    inner = st.word("")
    recs = []
    while not st.eof:
        name = st.word("")
        length = st.float(0.0)
        s1, s2, e = st.int(0), st.int(0), st.int(0)
        acc = tuple(st.float(0.0) for _ in range(3))
        grad = tuple(st.float(0.0) for _ in range(3))
        if not st.fail and not st.eof:
            recs.append((name, length, s1, s2, e, acc, grad))
        elif st.fail:
            break
    return root, inner, recs
