"""The reference-schedule driver (simulation_project_gb300.refpath.RefStep: CCellSet's
device arrays bound once, one step of CMultiGPUHandler::Calculate through the
reference-named launchers) against the oracle's restatement of the same schedule:
bit-identical particle outputs over several steps (walls fixed: the rotation's cosf and
the host cos differ in the last bits, which later steps would carry), and on the
rotating bucket with drag for one step."""
import ctypes as C

import numpy as np
import pytest

import orc
from simulation_project_gb300 import scenes
from simulation_project_gb300.refpath import RefStep

pytestmark = pytest.mark.gpu
ORC = orc.oracle()
FIELDS = ["out_pos", "out_vel", "out_pressure", "out_density", "out_id", "out_type"]


def _oracle_step(st, i, rotate):
    b = st.bindings()
    n = C.c_int(st.n)
    ORC.check_outside_compute_zone(C.byref(b), C.byref(n))
    st.n = n.value
    b = st.bindings()
    orc.ref_topology(ORC, st, b)
    ORC.reset_triangle_topology(st.cells_n, orc.ptr(st.cells))
    ORC.register_triangle_topology(C.byref(b), orc.ptr(st.triangles), st.t, orc.ptr(st.cells), st.cells_n)
    ORC.calc_stl_distance(C.byref(b), st.n)
    if st.drag_num:
        ORC.calc_drag_effect(C.byref(b), st.n)
    ORC.calc_explicitly(C.byref(b), st.n)
    orc.ref_topology(ORC, st, b)
    ORC.calc_stl_distance(C.byref(b), st.n)
    ORC.calc_explicit_pressure(C.byref(b), st.n)
    ORC.calc_explicit_pressure_gradient(C.byref(b), st.n)
    ORC.update_triangle_position(C.byref(b), st.t)
    if rotate:
        ORC.rotate_triangle_position(C.byref(b), st.t, i)


@pytest.mark.parametrize("name,steps", [("block", 4), ("bucket", 1)])
def test_refstep_matches_oracle_schedule(name, steps):
    if name == "block":
        sc = scenes.random_block(12, seed=5)
    else:
        sc = scenes.rotating_bucket(l0=0.012, n_drag=10, drag_index=5.0)
        sc.vel = np.random.default_rng(5).normal(0, 0.2, sc.pos.shape)
    sc.param.bExplicitPressure = True
    sc.param.SonicVelocity = 20.0
    st = orc.RefState(sc)
    g = RefStep(sc)
    for i in range(steps):
        n = g.step(i)
        _oracle_step(st, i, rotate=name == "bucket")
        assert n == st.n
    for f in FIELDS:
        got = g.download(f)
        want = getattr(st, f)
        assert got[:n].tobytes() == want[:n].tobytes(), f
    assert np.abs(st.out_pressure[:n]).max() > 0
    g.close()


def test_launchers_without_particles_return_noerr_and_touch_nothing():
    """N <= 0: every per-step launcher returns CCT_NOERR at once and leaves the bound
    arrays as they were (the reference's launchers, radix/SPVSOLVER/MultiGPUSolver/
    DeviceProcess.cu:49-409, launch nothing for an empty particle range)."""
    from simulation_project_gb300.lib import call
    sc = scenes.rotating_bucket(l0=0.012, n_drag=10, drag_index=5.0)
    sc.param.bExplicitPressure = True
    sc.param.SonicVelocity = 20.0
    g = RefStep(sc)
    g.step(0)
    before = {k: g.download(k) for k in g.d}
    s, d = g.stream.ref(), g.p
    for n in (0, -3):
        for name in RefStep.PARTICLE_KERNELS:
            g._kernel(name, n)
        call("CaculateCellIDandInitializeHash", s, n, g.cells, d("hash"), d("index"), d("out_pos"))
        call("SortUsingThrust", n, d("hash"), d("index"))
        call("reorderDataAndFindCellStart", s, n, g.cells, d("hash"), d("index"), d("cell_start"), d("cell_end"))
        cnt = C.c_int(n)
        call("CheckParticleOutsideComputeZone", s, C.byref(cnt))
        assert cnt.value == n
    for k, a in before.items():
        assert g.download(k).tobytes() == a.tobytes(), k
    g.close()
