"""GPU parity of the reference-named launcher API against the oracle: hash keys,
sort permutation, cell tables, reorder, triangle binning, wall distance, drag and the
three explicit-schedule particle kernels must be bit-identical to the oracle (itself
pinned to the reference's kernel code).  Wall rotation uses cosf/sinf on both sides
and is compared with an absolute tolerance of 2e-6 m."""
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


@pytest.mark.parametrize("n,lo,hi", [(1, 0, 5), (2, 3, 3), (1000, -50, 50), (70000, 0, 1 << 17),
                                     (300000, -(1 << 30), 1 << 30), (65536, 7, 7), (4097, 0, 255)])
def test_radix_sort_is_stable_sort(n, lo, hi):
    rng = np.random.default_rng(n)
    keys = rng.integers(lo, hi + 1, size=n, dtype=np.int64).astype(np.int32)
    vals = np.arange(n, dtype=np.int32)
    dk, dv = DeviceArray.from_host(keys), DeviceArray.from_host(vals)
    call("SortUsingThrust", n, dk.ptr, dv.ptr)
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


def test_unsupported_features_report_paramerr():
    sc = scenes.random_block(4)
    sc.param.bTurbulance = True
    st = orc.RefState(sc)
    g = _gpu().GpuRef(st)
    assert lib.load().CalcTurbulenceViscosity(g.stream.ref(), st.n) == 2
    assert lib.load().CalcExplicitly(g.stream.ref(), st.n) == 2
