"""Python front end of the configuration-file and drag-file readers (include/mps_io.h).

    cfg = read_configuration("configurationDragTemp.txt")
    cfg["models"][0]["file"], cfg["drag_count"], cfg["compute_zone"] ...
    tris, inner = read_drag_file("drag.txt")     # CDragTriangle records (numpy)

The parsing runs in libmps_gb300.so (host code; no GPU needed).
"""
import ctypes as C

import numpy as np

from . import lib
from .types import CBox, CParameter, CTriangleParameters, DragParameter, Integer3, MpsError, Scalar3

PATH_MAX = 512


class MpsConfigBucket(C.Structure):
    _fields_ = [("file", C.c_char * PATH_MAX), ("interval", C.c_int), ("total_steps", C.c_int)]


class MpsConfigModel(C.Structure):
    _fields_ = [("file", C.c_char * PATH_MAX), ("is_drag", C.c_int), ("drag_id", C.c_int), ("velocity", Scalar3),
                ("temperature", C.c_float), ("position", Scalar3), ("linear_movable", C.c_int),
                ("reset_interval", C.c_int), ("rotating", C.c_int), ("rpm", C.c_int), ("rotation_start", C.c_float),
                ("time_to_reach_rpm", C.c_float), ("center_of_rotation", Scalar3),
                ("second_point_of_rotation", Scalar3), ("wall_friction", C.c_float),
                ("wall_thermal_resistivity", C.c_float), ("wall_thermal_conductivity", C.c_float),
                ("negative_pressure_check", C.c_int), ("influence_region", C.c_float), ("direction", Scalar3),
                ("pressure_gas", C.c_float), ("drag", DragParameter)]


class MpsConfiguration(C.Structure):
    _fields_ = [("input_path", C.c_char * PATH_MAX), ("parameter_file", C.c_char * PATH_MAX),
                ("particle_file", C.c_char * PATH_MAX), ("output_path", C.c_char * PATH_MAX),
                ("output_name", C.c_char * PATH_MAX), ("bucket_count", C.c_int), ("model_count", C.c_int),
                ("drag_count", C.c_int), ("output_interval", C.c_int), ("has_compute_zone", C.c_int),
                ("compute_zone", CBox), ("section", Integer3), ("start_step", C.c_int), ("output_ascii", C.c_int)]


# numpy view of the reference's CDragTriangle record (DataType.h:205-218)
DRAG_TRIANGLE_DTYPE = np.dtype([("Normal", "<f4", 3), ("Vertex", "<f4", (3, 3)), ("DragLength", "<f4"),
                                ("StartStep01", "<i4"), ("StartStep02", "<i4"), ("EndStep", "<i4"),
                                ("InitialAcc", "<f4", 3), ("GradAcc", "<f4", 3), ("ID", "<i4")])

_bound = False


def _lib():
    global _bound
    L = lib.load()
    if not _bound:
        L.mps_read_configuration.argtypes = [C.c_char_p, C.POINTER(MpsConfiguration), C.c_void_p, C.c_int,
                                             C.c_void_p, C.c_int]
        L.mps_configuration_path.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]
        L.mps_configuration_triangle_parameters.argtypes = [C.c_void_p, C.c_int, C.POINTER(CParameter), C.c_void_p]
        L.mps_read_drag_file.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.c_void_p, C.c_int, C.c_char_p, C.c_int]
        _bound = True
    return L


def _s3(v):
    return (v.x, v.y, v.z)


def _value(x):
    if isinstance(x, bytes):
        return x.decode("latin-1")
    if isinstance(x, Scalar3):
        return _s3(x)
    if isinstance(x, (DragParameter,)):
        out = {}
        for k, _ in x._fields_:
            v = getattr(x, k)
            out[k] = v.decode("latin-1").rstrip("\0") if isinstance(v, bytes) else v
        return out
    return x


def _check(rc, what):
    if rc != 0:
        raise MpsError(rc, what)


def read_configuration_raw(path):
    """(MpsConfiguration, [MpsConfigBucket], [MpsConfigModel]) as the library returns them."""
    L = _lib()
    cfg = MpsConfiguration()
    p = str(path).encode()
    _check(L.mps_read_configuration(p, C.byref(cfg), None, 0, None, 0), f"mps_read_configuration({path})")
    buckets = (MpsConfigBucket * max(cfg.bucket_count, 1))()
    models = (MpsConfigModel * max(cfg.model_count, 1))()
    _check(L.mps_read_configuration(p, C.byref(cfg), buckets, cfg.bucket_count, models, cfg.model_count),
           f"mps_read_configuration({path})")
    return cfg, list(buckets)[:cfg.bucket_count], list(models)[:cfg.model_count]


def read_configuration(path) -> dict:
    """The configuration file as a dict (models and buckets as lists of dicts)."""
    cfg, buckets, models = read_configuration_raw(path)
    out = {k: _value(getattr(cfg, k)) for k, _ in MpsConfiguration._fields_ if k not in ("compute_zone", "section")}
    z = cfg.compute_zone
    out["compute_zone"] = (_s3(z.m_MinBound), _s3(z.m_MaxBound)) if cfg.has_compute_zone else None
    out["section"] = (cfg.section.x, cfg.section.y, cfg.section.z)
    out["buckets"] = [{k: _value(getattr(b, k)) for k, _ in MpsConfigBucket._fields_} for b in buckets]
    out["models"] = [{k: _value(getattr(m, k)) for k, _ in MpsConfigModel._fields_} for m in models]
    return out


def configuration_path(directory: str, name: str) -> str:
    buf = C.create_string_buffer(4 * PATH_MAX)
    _check(_lib().mps_configuration_path(directory.encode(), name.encode(), buf, len(buf)), "mps_configuration_path")
    return buf.value.decode("latin-1")


def triangle_parameters(models, param: CParameter):
    """CTriangleParameters per model (models: the MpsConfigModel list of read_configuration_raw)."""
    arr = (MpsConfigModel * max(len(models), 1))(*models)
    out = (CTriangleParameters * max(len(models), 1))()
    _check(_lib().mps_configuration_triangle_parameters(arr, len(models), C.byref(param), out),
           "mps_configuration_triangle_parameters")
    return list(out)[:len(models)]


def read_drag_file(path):
    """(CDragTriangle records as a numpy structured array, inner-pressure file name)."""
    L = _lib()
    n = C.c_int()
    p = str(path).encode()
    name = C.create_string_buffer(4 * PATH_MAX)
    _check(L.mps_read_drag_file(p, C.byref(n), None, 0, name, len(name)), f"mps_read_drag_file({path})")
    out = np.zeros(n.value, DRAG_TRIANGLE_DTYPE)
    _check(L.mps_read_drag_file(p, C.byref(n), out.ctypes.data, n.value, name, len(name)),
           f"mps_read_drag_file({path})")
    return out, name.value.decode("latin-1")
