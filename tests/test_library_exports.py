"""The C-ABI library builds, loads without a GPU, and exports every function the
public headers declare (no compute call is made here)."""
import ctypes as C
import os
import re

import pytest

from simulation_project_gb300 import build, lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h") or h == "mps_types.h":
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", text, re.M):
            name = m.group(1)
            if name in ("if", "defined", "extern"):
                continue
            names.append(name)
    return sorted(set(names))


@pytest.fixture(scope="module")
def so():
    path = build.build()
    return C.CDLL(path)


def test_every_declared_function_is_exported(so):
    names = declared_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, missing


def test_binding_signatures_cover_exports(so):
    for name in lib.exported_symbols():
        assert hasattr(so, name), name


def test_library_is_built_for_sm103a():
    path = build.build()
    blob = open(path, "rb").read()
    assert b"sm_103a" in blob


def test_default_options_through_the_python_mirror(so):
    """mps_solver_default_options (host code, no GPU) read through the ctypes mirror of
    MpsSolverOptions: every field lands where the header puts it, with the documented
    defaults (FP32 inner solve on FP16 weights streamed by bulk copies, multilevel
    preconditioner with smoothing weight 1.3, automatic warm start and inner floor)."""
    from simulation_project_gb300.solver import default_options, MpsSolverOptions
    o = default_options()
    # 18 ints and 10 doubles in header order, naturally aligned (four 4-byte pads)
    assert C.sizeof(MpsSolverOptions) == 168
    assert o.precision == 1 and o.pressure_mode == 0 and o.learned == 0
    assert o.compressibility == 1e-9 and o.cg_rtol == 1e-8 and o.cg_max_iter == 5000
    assert o.ir_inner_rtol == 0.0 and o.ir_max_outer == 12 and o.max_neighbours == 384
    assert o.check_every == 8 and o.source_relaxation == 0.05
    assert o.preconditioner == 1 and o.mg_omega == 1.3 and o.compress_rows == 1 and o.mg_sweeps == 1
    assert o.matrix_free == 0 and o.spmv_stream == 1 and o.inner_weights == 16 and o.spmv_wide == 0
    assert o.warm_start == -1 and o.flexible == 0 and o.learned_gate == 1
    assert o.fine_smoother == 0 and o.smoother_weight == 0.8 and o.rows_sell == 0


@pytest.mark.parametrize("bad", [{"matrix_free": 3}, {"spmv_stream": 2}, {"inner_weights": 8}, {"spmv_wide": 2},
                                 {"warm_start": 3}, {"warm_start": -2}, {"flexible": 2}, {"learned_gate": -1},
                                 {"fine_smoother": 2}, {"smoother_weight": -1.0}, {"rows_sell": 2}])
def test_invalid_solver_options_are_rejected_before_any_device_work(so, bad):
    """mps_solver_create checks its options before it touches the device: an invalid
    value returns CCT_PARAMERR (2) and no solver, with or without a GPU."""
    from simulation_project_gb300 import scenes
    from simulation_project_gb300.solver import default_options, _lib
    sc = scenes.random_block(4)
    o = default_options(**bad)
    h = C.c_void_p()
    rc = _lib().mps_solver_create(C.byref(sc.param), C.byref(sc.box), sc.n, C.byref(o), C.byref(h))
    assert rc == 2 and not h.value
