"""Pins the CPU oracle to the reference: the oracle's restatement and the reference's
own kernel header compiled for the CPU (oracle/_ref/libref.so) must agree bit for bit
on seeded inputs.  Skipped where the reference sources are unavailable; the committed
golden vectors (test_golden.py) carry the same pin there."""
import ctypes as C

import numpy as np
import pytest

import orc
from simulation_project_gb300 import scenes
from simulation_project_gb300.types import Scalar3, CTriangle, CParameter, TRIANGLE_DTYPE

ORC = orc.oracle()
REF = orc.reference()
pytestmark = pytest.mark.skipif(REF is None, reason="reference sources not available")


def bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


def test_fast_sqrt_and_weights():
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(0, 1, 2000), rng.uniform(0, 1e-6, 200), [0.0, 1e-30, 1.0, 4.0, 1e6]])
    for x in xs.astype(np.float32):
        assert np.float32(ORC.sqrt_utility(x)).tobytes() == np.float32(REF.sqrt_utility(x)).tobytes()
    for _ in range(2000):
        re = np.float32(rng.uniform(0.001, 0.1))
        r = np.float32(rng.uniform(0, 0.12))
        assert ORC.get_weight(re, r) == REF.get_weight(re, r)
    assert ORC.get_weight(np.float32(1.0), np.float32(0.0)) == REF.get_weight(np.float32(1.0), np.float32(0.0))


@pytest.mark.parametrize("fn", ["zgrad", "zlap", "zgrad2d", "zlap2d"])
def test_z_tables(fn):
    rng = np.random.default_rng(1)
    l0 = np.float32(0.004)
    rs = np.concatenate([rng.uniform(0, 4.5, 5000), np.arange(0, 4.2, 0.01), np.arange(0, 4.2, 0.1)]) * 0.004
    f_o, f_r = getattr(ORC, fn), getattr(REF, fn)
    for r in rs.astype(np.float32):
        assert np.float32(f_o(r, l0)).tobytes() == np.float32(f_r(r, l0)).tobytes(), (fn, r)


def _rand_tri(rng, scale=0.05):
    t = CTriangle()
    v = rng.normal(0, scale, (3, 3)).astype(np.float32)
    for q in range(3):
        t.Vertex[q] = Scalar3(*v[q])
    nrm = orc.triangle_normals_q(v[None])[0]
    t.Normal = Scalar3(*nrm)
    return t


def test_triangle_distance():
    rng = np.random.default_rng(2)
    for _ in range(3000):
        t = _rand_tri(rng)
        p = Scalar3(*rng.normal(0, 0.05, 3).astype(np.float32))
        d1, d2 = Scalar3(), Scalar3()
        m1 = ORC.triangle_distance(C.byref(t), C.byref(p), C.byref(d1))
        m2 = REF.triangle_distance(C.byref(t), C.byref(p), C.byref(d2))
        assert np.float32(m1).tobytes() == np.float32(m2).tobytes()
        assert (d1.x, d1.y, d1.z) == (d2.x, d2.y, d2.z)


def test_cell_id_include_courant():
    sc = scenes.random_block(6)
    rng = np.random.default_rng(3)
    for _ in range(2000):
        p = Scalar3(*rng.uniform(-0.05, 0.12, 3).astype(np.float32))
        a = [C.c_int(), C.c_int(), C.c_int()]
        b = [C.c_int(), C.c_int(), C.c_int()]
        k1 = ORC.cell_id(C.byref(sc.box), C.byref(p), *[C.byref(x) for x in a])
        k2 = REF.cell_id(C.byref(sc.box), C.byref(p), *[C.byref(x) for x in b])
        assert k1 == k2 and [x.value for x in a] == [x.value for x in b]
        assert ORC.is_include(C.byref(sc.box), C.byref(p), np.float32(0.001)) == \
            REF.is_include(C.byref(sc.box), C.byref(p), np.float32(0.001))
        v1 = Scalar3(*rng.normal(0, 3.0, 3).astype(np.float32))
        v2 = Scalar3(v1.x, v1.y, v1.z)
        ORC.correct_velocity(C.byref(sc.param), C.byref(v1))
        REF.correct_velocity(C.byref(sc.param), C.byref(v2))
        assert (v1.x, v1.y, v1.z) == (v2.x, v2.y, v2.z)


def _run_both(scene, fn_names, setup=None):
    so = orc.RefState(scene)
    if setup:
        setup(so)
    sr = so.copy()
    bo, br = so.bindings(), sr.bindings()
    orc.ref_topology(ORC, so, bo)
    orc.ref_topology(REF, sr, br)
    for lib, st, b in ((ORC, so, bo), (REF, sr, br)):
        lib.reset_triangle_topology(st.cells_n, orc.ptr(st.cells))
        lib.register_triangle_topology(C.byref(b), orc.ptr(st.triangles), st.t, orc.ptr(st.cells), st.cells_n)
        for name in fn_names:
            assert getattr(lib, name)(C.byref(b), st.n) == 0
    return so, sr


FIELDS = ["hash", "index", "cell_start", "cell_end", "id", "pos", "vel", "pressure", "density", "kin_visc", "type",
          "out_id", "out_pos", "out_vel", "out_pressure", "out_density", "out_solid_rate", "out_type", "cells",
          "stl_distance", "stl_id", "drag_acc", "magnifier_count"]


def _compare(so, sr):
    for f in FIELDS:
        assert bits_equal(getattr(so, f), getattr(sr, f)), f


@pytest.mark.parametrize("seed", [0, 1])
def test_topology_and_walls(seed):
    sc = scenes.random_block(9, seed=seed)
    so, sr = _run_both(sc, ["calc_stl_distance"])
    _compare(so, sr)
    assert (so.stl_id[:so.n] >= 0).any()


@pytest.mark.parametrize("seed", [0, 3])
def test_explicit_step_kernels(seed):
    sc = scenes.random_block(9, seed=seed)
    so, sr = _run_both(sc, ["calc_stl_distance", "calc_explicitly"])
    _compare(so, sr)
    # second half of the reference schedule on the predicted positions
    for lib, st in ((ORC, so), (REF, sr)):
        b = st.bindings()
        orc.ref_topology(lib, st, b)
        assert lib.calc_stl_distance(C.byref(b), st.n) == 0
        assert lib.calc_explicit_pressure(C.byref(b), st.n) == 0
        assert lib.calc_explicit_pressure_gradient(C.byref(b), st.n) == 0
    _compare(so, sr)
    assert np.abs(so.out_pressure[:so.n]).max() > 0


@pytest.mark.parametrize("seed", [0, 2])
def test_explicit_step_kernels_2d_branches(seed):
    """Dimension = 2 on the same block: the 2D Z tables (gradient and Laplacian), the
    2-dimensional coefficients of the Laplacian, PND, gradient and temperature terms."""
    sc = scenes.random_block(9, seed=seed)
    sc.param.Dimension = 2
    setup = orc.thermal_scene(sc, seed)
    so, sr = _run_both(sc, ["calc_stl_distance", "calc_explicitly", "calc_temperature_factor"], setup)
    _compare(so, sr)
    for f in FIELDS_HEAT:
        assert bits_equal(getattr(so, f), getattr(sr, f)), f
    for lib, st in ((ORC, so), (REF, sr)):
        b = st.bindings()
        orc.ref_topology(lib, st, b)
        assert lib.calc_stl_distance(C.byref(b), st.n) == 0
        assert lib.calc_explicit_pressure(C.byref(b), st.n) == 0
        assert lib.calc_explicit_pressure_gradient(C.byref(b), st.n) == 0
    _compare(so, sr)
    assert np.abs(so.out_pressure[:so.n]).max() > 0


def test_drag_kernel():
    sc = scenes.rotating_bucket(l0=0.02, n_drag=6, drag_index=5.0)
    sc.vel = np.random.default_rng(5).normal(0, 0.2, sc.pos.shape)

    def setup(st):
        st.magnifier_count[: st.n: 7] = 3
    so, sr = _run_both(sc, ["calc_stl_distance", "calc_drag_effect", "calc_explicitly"], setup)
    _compare(so, sr)
    assert (np.abs(so.drag_acc[:so.n]).sum(1) > 0).any()


def test_triangle_motion():
    sc = scenes.rotating_bucket(l0=0.02, n_drag=0)
    sc.tri_params[0].TimeToReachRPM = 0.01
    so = orc.RefState(sc)
    sr = so.copy()
    for lib, st in ((ORC, so), (REF, sr)):
        b = st.bindings()
        for step in range(0, 400, 7):
            lib.update_triangle_position(C.byref(b), st.t)
            lib.rotate_triangle_position(C.byref(b), st.t, step)
    # cosf/sinf vs the host math library differ in the last bits: tolerance
    np.testing.assert_allclose(so.triangles["Vertex"], sr.triangles["Vertex"], rtol=0, atol=2e-6)
    assert np.abs(so.triangles["Vertex"] - orc.RefState(sc).triangles["Vertex"]).max() > 1e-3


def test_linear_wall_reset():
    """UpdateTrianglePosition each step, then ResetWallPosition: movable models return
    to the original triangles at the steps with (step + 1) % interval == 0."""
    sc = orc.linear_walls_scene(seed=4)
    so = orc.RefState(sc)
    sr = so.copy()
    orig = so.triangles.copy()
    resets = 0
    for lib, st in ((ORC, so), (REF, sr)):
        b = st.bindings()
        for step in range(17):
            assert lib.update_triangle_position(C.byref(b), st.t) == 0
            assert lib.reset_wall_position(C.byref(b), st.t, step, orc.ptr(orig)) == 0
            if lib is ORC:
                resets += int(((step + 1) % 3 == 0) or ((step + 1) % 5 == 0))
    assert bits_equal(so.triangles, sr.triangles)
    # model 0 moved with velocity 0: unchanged; models 1 and 2 moved since their last reset
    m = so.triangles["ModelIDNumber"][:so.t]
    assert bits_equal(so.triangles[:so.t][m == 0], orig[:so.t][m == 0])
    assert (so.triangles["Vertex"][:so.t][m == 1] != orig["Vertex"][:so.t][m == 1]).any()
    assert resets > 0


FIELDS_HEAT = ["out_id", "out_temperature", "out_kin_visc", "temperature", "stl_distance", "stl_id", "drag_acc",
               "out_solid_rate"]
FIELDS_TURB = ["turb_visc", "strain", "out_id", "out_pos", "out_vel", "pressure"]


@pytest.mark.parametrize("seed", [0, 2])
def test_temperature_kernel(seed):
    sc = scenes.random_block(9, seed=seed)
    setup = orc.thermal_scene(sc, seed)
    so, sr = _run_both(sc, ["calc_stl_distance", "calc_temperature_factor"], setup)
    for f in FIELDS_HEAT:
        assert bits_equal(getattr(so, f), getattr(sr, f)), f
    t = so.out_temperature[:so.n]
    assert (t != np.float32(0)).all() and (t <= 330.0).all() and (t >= 290.0).all()


def test_temperature_with_drag_heating():
    sc = scenes.rotating_bucket(l0=0.02, n_drag=6, drag_index=5.0)
    sc.vel = np.random.default_rng(5).normal(0, 0.2, sc.pos.shape)
    for d in sc.drag:
        d.InputVelocityToken1 = b"T"
        d.TempIndex, d.TempExponential, d.TempDragPermiabilityConstant = 2.0, 1.5, 0.5
    sc.param.ThermalStep = 1
    setup = orc.thermal_scene(sc, 3)
    so, sr = _run_both(sc, ["calc_stl_distance", "calc_drag_effect", "calc_temperature_factor"], setup)
    for f in FIELDS_HEAT:
        assert bits_equal(getattr(so, f), getattr(sr, f)), f
    assert (so.drag_temperature[:so.n] != 0).any()


@pytest.mark.parametrize("seed", [0, 1])
def test_turbulence_kernels(seed):
    sc = scenes.random_block(9, seed=seed)
    orc.turbulent_scene(sc, seed)
    so, sr = _run_both(sc, ["calc_stl_distance", "calc_turbulence_viscosity", "calc_explicitly"])
    for f in FIELDS_TURB:
        assert bits_equal(getattr(so, f), getattr(sr, f)), f
    assert (so.turb_visc[:so.n] > 0).any() and (so.strain[:so.n] > 0).any()
    assert (so.turb_visc[:so.n] == np.float32(2e-5)).any()   # the cap is reached
