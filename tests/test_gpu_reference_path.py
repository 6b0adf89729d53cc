"""GPU parity of the reference-named launcher API against the oracle: hash keys,
sort permutation, cell tables, reorder, triangle binning, wall distance, drag, the
three explicit-schedule particle kernels and the temperature operator must be
bit-identical to the oracle (itself pinned to the reference's kernel code).  Wall
rotation uses cosf/sinf and the turbulence model's wall damping expf on both sides:
those are compared with tolerances stated in their tests."""
import ctypes as C

import numpy as np
import pytest

import orc
from simulation_project_gb300 import scenes, lib
from simulation_project_gb300.lib import DeviceArray, call

pytestmark = pytest.mark.gpu
ORC = orc.oracle()

COMPARE = ["hash", "index", "cell_start", "cell_end", "id", "pos", "vel", "pressure", "density", "kin_visc", "type",
           "out_id", "out_pos", "out_vel", "out_pressure", "out_density", "out_solid_rate", "out_type", "cells",
           "stl_distance", "stl_id", "drag_acc", "magnifier_count"]


def _gpu():
    import gpu_ref
    return gpu_ref


def assert_same(st, got, fields=COMPARE, n=None):
    for f in fields:
        a = getattr(st, f)
        b = got[f]
        assert a.tobytes() == b.tobytes(), f"{f} differs: {np.flatnonzero(a.view(np.uint8) != b.view(np.uint8))[:10]}"


def oracle_topology_walls(st, with_walls=True):
    b = st.bindings()
    orc.ref_topology(ORC, st, b)
    if with_walls:
        ORC.reset_triangle_topology(st.cells_n, orc.ptr(st.cells))
        ORC.register_triangle_topology(C.byref(b), orc.ptr(st.triangles), st.t, orc.ptr(st.cells), st.cells_n)
    return b


@pytest.mark.parametrize("n_side,seed", [(5, 0), (12, 1), (40, 2)])
def test_hash_sort_cells_reorder(n_side, seed):
    sc = scenes.random_block(n_side, seed=seed, with_box=False)
    st = orc.RefState(sc)
    g = _gpu().GpuRef(st)
    g.topology(st.n)
    oracle_topology_walls(st, with_walls=False)
    assert_same(st, g.download(), ["hash", "index", "cell_start", "cell_end", "id", "pos", "vel", "pressure",
                                   "kin_visc", "type"])


@pytest.mark.parametrize("entry", ["SortUsingThrust", "StableSortUsingThrust"])
@pytest.mark.parametrize("n,lo,hi", [(1, 0, 5), (2, 3, 3), (1000, -50, 50), (70000, 0, 1 << 17),
                                     (300000, -(1 << 30), 1 << 30), (65536, 7, 7), (4097, 0, 255),
                                     (5000, -1000, 40000)])
def test_radix_sort_is_stable_sort(n, lo, hi, entry):
    rng = np.random.default_rng(n)
    keys = rng.integers(lo, hi + 1, size=n, dtype=np.int64).astype(np.int32)
    vals = np.arange(n, dtype=np.int32)
    dk, dv = DeviceArray.from_host(keys), DeviceArray.from_host(vals)
    call(entry, n, dk.ptr, dv.ptr)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(dk.download(), keys[order])
    assert np.array_equal(dv.download(), vals[order])


def test_compaction_matches_reference_order():
    sc = scenes.random_block(10, seed=4, with_box=False)
    st = orc.RefState(sc)
    rng = np.random.default_rng(9)
    # push a scattered set of particles (including the last ones) out of the zone
    out = rng.choice(st.n, size=st.n // 5, replace=False)
    out = np.concatenate([out, [st.n - 1, st.n - 2, 0]])
    st.out_pos[out, 0] += 10.0
    g = _gpu().GpuRef(st)
    n = C.c_int(st.n)
    call("CheckParticleOutsideComputeZone", g.stream.ref(), C.byref(n))
    no = C.c_int(st.n)
    ORC.check_outside_compute_zone(C.byref(st.bindings()), C.byref(no))
    assert n.value == no.value < st.n
    got = g.download()
    for f in ["out_pos", "out_vel", "out_pressure", "out_id", "out_type", "out_kin_visc"]:
        assert getattr(st, f)[:no.value].tobytes() == got[f][:no.value].tobytes(), f


def _explicit_pipeline(sc, with_drag=False, setup=None):
    st = orc.RefState(sc)
    if setup:
        setup(st)
    g = _gpu().GpuRef(st)
    # oracle
    b = oracle_topology_walls(st)
    ORC.calc_stl_distance(C.byref(b), st.n)
    if with_drag:
        ORC.calc_drag_effect(C.byref(b), st.n)
    ORC.calc_explicitly(C.byref(b), st.n)
    # gpu
    g.topology(st.n)
    g.walls()
    g.run("CalcSTLDistance", st.n)
    if with_drag:
        g.run("CalcDragEffect", st.n)
    g.run("CalcExplicitly", st.n)
    assert_same(st, g.download())
    # second half of the reference step on the predicted positions
    b = st.bindings()
    orc.ref_topology(ORC, st, b)
    ORC.calc_stl_distance(C.byref(b), st.n)
    ORC.calc_explicit_pressure(C.byref(b), st.n)
    ORC.calc_explicit_pressure_gradient(C.byref(b), st.n)
    g.topology(st.n)
    g.run("CalcSTLDistance", st.n)
    g.run("CalcExplicitPressure", st.n)
    g.run("CalcExplicitPressureGradient", st.n)
    assert_same(st, g.download())
    return st


@pytest.mark.parametrize("n_side,seed", [(8, 0), (20, 3)])
def test_explicit_step_bit_exact(n_side, seed):
    st = _explicit_pipeline(scenes.random_block(n_side, seed=seed))
    assert np.abs(st.out_pressure[:st.n]).max() > 0
    assert (st.stl_id[:st.n] >= 0).any()


def test_drag_and_bucket_bit_exact():
    sc = scenes.rotating_bucket(l0=0.012, n_drag=10, drag_index=5.0)
    sc.vel = np.random.default_rng(5).normal(0, 0.2, sc.pos.shape)

    def setup(st):
        st.magnifier_count[: st.n: 7] = 3
    st = _explicit_pipeline(sc, with_drag=True, setup=setup)
    assert (np.abs(st.drag_acc[:st.n]).sum(1) > 0).any()


def test_triangle_motion_close():
    sc = scenes.rotating_bucket(l0=0.02, n_drag=0)
    sc.tri_params[0].TimeToReachRPM = 0.01
    st = orc.RefState(sc)
    g = _gpu().GpuRef(st)
    b = st.bindings()
    for step in range(0, 400, 7):
        ORC.update_triangle_position(C.byref(b), st.t)
        ORC.rotate_triangle_position(C.byref(b), st.t, step)
        call("UpdateTrianglePosition", g.stream.ref(), st.t, g.p("triangles"))
        call("RotateTrianglePosition", g.stream.ref(), st.t, g.p("triangles"), step)
    g.stream.sync()
    got = g.download()["triangles"]
    np.testing.assert_allclose(got["Vertex"], st.triangles["Vertex"], rtol=0, atol=2e-6)


def test_linear_wall_reset_bit_exact():
    """UpdateTrianglePosition + ResetWallPosition (DeviceProcess_Kernel.h:603-621,
    690-704) over 17 steps: the triangles equal the oracle's bit for bit."""
    sc = orc.linear_walls_scene(seed=4)
    st = orc.RefState(sc)
    orig = st.triangles.copy()
    g = _gpu().GpuRef(st)
    d_orig = DeviceArray.from_host(orig)
    b = st.bindings()
    for step in range(17):
        ORC.update_triangle_position(C.byref(b), st.t)
        ORC.reset_wall_position(C.byref(b), st.t, step, orc.ptr(orig))
        assert call("UpdateTrianglePosition", g.stream.ref(), st.t, g.p("triangles")) == 0
        assert call("ResetWallPosition", g.stream.ref(), st.t, step, d_orig.ptr) == 0
    g.stream.sync()
    got = g.download()["triangles"]
    assert got.tobytes() == st.triangles.tobytes()
    assert got.tobytes() != orig.tobytes()


def test_unsupported_features_report_paramerr():
    sc = scenes.random_block(4)
    sc.param.bNegativePressure = True
    st = orc.RefState(sc)
    g = _gpu().GpuRef(st)
    assert lib.load().CalcExplicitPressureGradient(g.stream.ref(), st.n) == 2


HEAT = ["out_id", "out_temperature", "out_kin_visc", "temperature", "stl_distance", "stl_id", "drag_acc",
        "drag_temperature", "out_solid_rate"]


POWF = ["drag_temperature", "out_solid_rate", "out_temperature", "out_kin_visc"]


def _heat_pipeline(sc, setup, with_drag):
    st = orc.RefState(sc)
    setup(st)
    g = _gpu().GpuRef(st)
    b = oracle_topology_walls(st)
    ORC.calc_stl_distance(C.byref(b), st.n)
    if with_drag:
        ORC.calc_drag_effect(C.byref(b), st.n)
    assert ORC.calc_temperature_factor(C.byref(b), st.n) == 0
    g.topology(st.n)
    g.walls()
    g.run("CalcSTLDistance", st.n)
    if with_drag:
        g.run("CalcDragEffect", st.n)
    assert call("CalcTemperatureFactor", g.stream.ref(), st.n) == 0
    g.stream.sync()
    got = g.download()
    if not with_drag:
        assert_same(st, got, HEAT)
        return st
    # the drag heating raises the slip speed to TempExponential with powf, CUDA's on the
    # GPU and the host library's on the CPU (last-bit differences): those fields and the
    # temperatures they heat are compared with tolerances, the rest bit for bit
    assert_same(st, got, [f for f in HEAT if f not in POWF])
    n = st.n
    np.testing.assert_allclose(got["drag_temperature"][:n], st.drag_temperature[:n], rtol=1e-6, atol=0)
    np.testing.assert_allclose(got["out_solid_rate"][:n], st.out_solid_rate[:n], rtol=1e-6, atol=0)
    np.testing.assert_allclose(got["out_temperature"][:n], st.out_temperature[:n], rtol=0, atol=1e-4)
    np.testing.assert_allclose(got["out_kin_visc"][:n], st.out_kin_visc[:n], rtol=1e-6, atol=0)
    return st


@pytest.mark.parametrize("n_side,seed", [(9, 0), (24, 2)])
def test_temperature_bit_exact(n_side, seed):
    sc = scenes.random_block(n_side, seed=seed)
    st = _heat_pipeline(sc, orc.thermal_scene(sc, seed), with_drag=False)
    t = st.out_temperature[:st.n]
    assert (t <= 330.0).all() and (t >= 290.0).all() and len(np.unique(t)) > st.n // 2


def test_temperature_with_drag_heating_bit_exact():
    sc = scenes.rotating_bucket(l0=0.02, n_drag=6, drag_index=5.0)
    sc.vel = np.random.default_rng(5).normal(0, 0.2, sc.pos.shape)
    for d in sc.drag:
        d.InputVelocityToken1 = b"T"
        d.TempIndex, d.TempExponential, d.TempDragPermiabilityConstant = 2.0, 1.5, 0.5
    sc.param.ThermalStep = 1
    st = _heat_pipeline(sc, orc.thermal_scene(sc, 3), with_drag=True)
    assert (st.drag_temperature[:st.n] != 0).any()


@pytest.mark.parametrize("n_side,seed", [(9, 0), (20, 1)])
def test_turbulence_and_explicit_step(n_side, seed):
    """Strain-rate products and everything that does not depend on the wall damping
    are bit-identical; the damping factor 1 - expf(-r/re) uses CUDA's expf (2 ulp) on the
    GPU and the host library's on the CPU.  An error of k ulp in e = expf(-r/re) moves
    damp by k ulp * e/(1-e) relative, and the viscosity carries damp squared: the
    viscosity is compared against that bound per particle (k = 4), the predicted
    velocities and positions to 1e-6 relative (the viscosity term is Dt-scaled)."""
    sc = scenes.random_block(n_side, seed=seed)
    orc.turbulent_scene(sc, seed)
    st = orc.RefState(sc)
    g = _gpu().GpuRef(st)
    b = oracle_topology_walls(st)
    ORC.calc_stl_distance(C.byref(b), st.n)
    assert ORC.calc_turbulence_viscosity(C.byref(b), st.n) == 0
    tv_o = st.turb_visc.copy()
    assert ORC.calc_explicitly(C.byref(b), st.n) == 0
    g.topology(st.n)
    g.walls()
    g.run("CalcSTLDistance", st.n)
    assert call("CalcTurbulenceViscosity", g.stream.ref(), st.n) == 0
    g.stream.sync()
    tv_g = g.download()["turb_visc"]
    assert call("CalcExplicitly", g.stream.ref(), st.n) == 0
    g.stream.sync()
    got = g.download()
    assert_same(st, got, ["strain", "out_id", "stl_distance", "stl_id", "pressure", "id", "hash", "index"])
    n = st.n
    re = np.float64(sc.param.GradientInfluenceRadiusCoefficient) * sc.param.InitialParticleDistance
    e = np.exp(-st.stl_distance["Magnitude"][:n].astype(np.float64) / re)
    bound = tv_o[:n].astype(np.float64) * (2 * 4 * 2.0 ** -24 * e / np.maximum(1 - e, 1e-30) + 4 * 2.0 ** -24)
    assert (np.abs(tv_g[:n].astype(np.float64) - tv_o[:n]) <= bound).all()
    assert (tv_o[:n] > 0).any() and (tv_o[:n] == np.float32(2e-5)).any()
    for f in ["out_vel", "out_pos", "vel", "pos"]:
        np.testing.assert_allclose(got[f][:n], getattr(st, f)[:n], rtol=1e-6, atol=1e-9, err_msg=f)
