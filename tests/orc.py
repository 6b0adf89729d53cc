"""Loader and state helpers for the CPU oracle (oracle/liborc.so) and the reference
CPU harness (oracle/_ref/libref.so).  Test infrastructure only."""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from simulation_project_gb300.types import (CParameter, CGridBox, CTriangle, CTriangleParameters, CDistance,  # noqa: E402
                                            CCell, DragParameter, Scalar3, TRIANGLE_DTYPE, DISTANCE_DTYPE,
                                            CELL_DTYPE)

P = C.c_void_p


class OrcBindings(C.Structure):
    _fields_ = [
        ("param", CParameter), ("box", CGridBox), ("particle_num", C.c_int), ("max_particle_num", C.c_int),
        ("id", P), ("pos", P), ("vel", P), ("pressure", P), ("density", P), ("temperature", P), ("kin_visc", P),
        ("solid_rate", P), ("type", P),
        ("out_id", P), ("out_pos", P), ("out_vel", P), ("out_pressure", P), ("out_density", P),
        ("out_temperature", P), ("out_kin_visc", P), ("out_solid_rate", P), ("out_type", P),
        ("triangles", P), ("triangle_num", C.c_int), ("tri_params", P), ("stl_distance", P), ("stl_id", P),
        ("cells", P), ("cell_num", C.c_int), ("cell_start", P), ("cell_end", P),
        ("drag_params", P), ("drag_num", C.c_int), ("drag_acc", P), ("drag_temperature", P),
        ("magnifier_count", P), ("turb_visc", P), ("strain", P),
    ]


class OrcSimConfig(C.Structure):
    _fields_ = [("param", CParameter), ("box", CGridBox), ("quirks", C.c_int), ("n0_pnd", C.c_double),
                ("n0_lap", C.c_double), ("lambda_", C.c_double), ("compressibility", C.c_double),
                ("cg_rtol", C.c_double), ("cg_max_iter", C.c_int), ("threads", C.c_int),
                ("source_relaxation", C.c_double)]


class OrcStepStats(C.Structure):
    _fields_ = [("cg_iterations", C.c_int), ("cg_relres", C.c_double), ("b_norm", C.c_double),
                ("interior", C.c_int), ("particles", C.c_int)]


_FUNCS = {
    "orc_sqrt_utility": (C.c_float, [C.c_float]),
    "orc_calc_distance": (C.c_float, [P, P]),
    "orc_get_weight": (C.c_float, [C.c_float, C.c_float]),
    "orc_zgrad": (C.c_float, [C.c_float, C.c_float]),
    "orc_zlap": (C.c_float, [C.c_float, C.c_float]),
    "orc_zgrad2d": (C.c_float, [C.c_float, C.c_float]),
    "orc_zlap2d": (C.c_float, [C.c_float, C.c_float]),
    "orc_triangle_distance": (C.c_float, [P, P, P]),
    "orc_cell_id": (C.c_int, [P, P, P, P, P]),
    "orc_is_include": (C.c_int, [P, P, C.c_float]),
    "orc_correct_velocity": (None, [P, P]),
    "orc_lambda_table": (C.c_float, [C.c_float]),
    "orc_calc_hash": (C.c_int, [P, C.c_int, P, P, P]),
    "orc_sort": (C.c_int, [C.c_int, P, P]),
    "orc_reorder_find_cell_start": (C.c_int, [P, C.c_int, C.c_int, P, P, P, P]),
    "orc_check_outside_compute_zone": (C.c_int, [P, P]),
    "orc_reset_triangle_topology": (C.c_int, [C.c_int, P]),
    "orc_register_triangle_topology": (C.c_int, [P, P, C.c_int, P, C.c_int]),
    "orc_update_triangle_position": (C.c_int, [P, C.c_int]),
    "orc_rotate_triangle_position": (C.c_int, [P, C.c_int, C.c_int]),
    "orc_reset_wall_position": (C.c_int, [P, C.c_int, C.c_int, P]),
    "orc_calc_stl_distance": (C.c_int, [P, C.c_int]),
    "orc_calc_drag_effect": (C.c_int, [P, C.c_int]),
    "orc_calc_explicitly": (C.c_int, [P, C.c_int]),
    "orc_calc_temperature_factor": (C.c_int, [P, C.c_int]),
    "orc_calc_turbulence_viscosity": (C.c_int, [P, C.c_int]),
    "orc_calc_explicit_pressure": (C.c_int, [P, C.c_int]),
    "orc_calc_explicit_pressure_gradient": (C.c_int, [P, C.c_int]),
    "orc_sim_create": (P, [P, C.c_int]),
    "orc_sim_destroy": (None, [P]),
    "orc_sim_set_particles": (C.c_int, [P, C.c_int, P, P, P, P, P]),
    "orc_sim_set_triangles": (C.c_int, [P, C.c_int, P, P, C.c_int, P]),
    "orc_sim_set_drag": (C.c_int, [P, C.c_int, P]),
    "orc_sim_step": (C.c_int, [P, C.c_int, P]),
    "orc_sim_get": (C.c_int, [P, P, P, P, P, P]),
    "orc_sim_get_triangles": (C.c_int, [P, P]),
    "orc_sim_last_ppe": (C.c_int, [P, P, P, P, P, P]),
    "orc_sim_get_ids": (C.c_int, [P, P]),
    "orc_sim_last_nbr": (C.c_int, [P, P, P, P]),
    "orc_sim_last_matrix": (C.c_longlong, [P, P, P, P]),
}


class Lib:
    """Thin wrapper: attributes are the exported functions that exist in the .so."""

    def __init__(self, path):
        self.path = path
        self.dll = C.CDLL(path)
        for name, (res, args) in _FUNCS.items():
            try:
                f = getattr(self.dll, name)
            except AttributeError:
                continue
            f.restype = res
            f.argtypes = args
            setattr(self, name[4:] if name.startswith("orc_") else name, f)


_oracle = None
_ref = None


def oracle() -> Lib:
    global _oracle
    if _oracle is None:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import build_ref
        _oracle = Lib(build_ref.build_oracle())
    return _oracle


def reference():
    """The reference CPU harness, or None where its sources are unavailable."""
    global _ref
    if _ref is None:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import build_ref
        path = build_ref.build_ref()
        if path is None:
            return None
        _ref = Lib(path)
    return _ref


def ptr(a):
    return None if a is None else a.ctypes.data


class RefState:
    """Host arrays for one reference-schedule state (sorted + original order) of a
    scene, plus the OrcBindings that points at them."""

    def __init__(self, scene, max_n=None):
        n = scene.n
        m = max_n or n
        self.n = n
        self.cells_n = scene.box.cell_num
        f3 = lambda: np.zeros((m, 3), dtype=np.float32)  # noqa: E731
        self.id = np.zeros(m, np.int32)
        self.pos, self.vel = f3(), f3()
        self.pressure, self.density, self.temperature = (np.zeros(m, np.float32) for _ in range(3))
        self.kin_visc, self.solid_rate = np.zeros(m, np.float32), np.zeros(m, np.float32)
        self.type = np.zeros(m, np.int32)
        self.out_id = np.arange(m, dtype=np.int32)
        self.out_pos, self.out_vel = f3(), f3()
        self.out_pos[:n] = scene.pos.astype(np.float32)
        self.out_vel[:n] = scene.vel.astype(np.float32)
        self.out_pressure = np.zeros(m, np.float32)
        self.out_pressure[:n] = scene.press
        self.out_density = np.zeros(m, np.float32)
        self.out_temperature = np.zeros(m, np.float32)
        self.out_kin_visc = np.zeros(m, np.float32)
        self.out_kin_visc[:n] = scene.visc
        self.out_solid_rate = np.zeros(m, np.float32)
        self.out_type = np.zeros(m, np.int32)
        self.out_type[:n] = scene.ptype
        t = scene.t
        self.triangles = np.zeros(max(t, 1), dtype=TRIANGLE_DTYPE)
        self.triangles["ModelIDNumber"][:t] = scene.tri_model
        self.triangles["Vertex"][:t] = scene.tri_vertices.astype(np.float32)
        self.triangles["Normal"][:t] = triangle_normals_q(self.triangles["Vertex"][:t])
        self.t = t
        self.tri_params = (CTriangleParameters * max(len(scene.tri_params), 1))(*scene.tri_params)
        self.stl_distance = np.zeros(m, dtype=DISTANCE_DTYPE)
        self.stl_id = np.full(m, -1, np.int32)
        self.cells = np.zeros(self.cells_n, dtype=CELL_DTYPE)
        self.cell_start = np.full(self.cells_n, -1, np.int32)
        self.cell_end = np.full(self.cells_n, -1, np.int32)
        self.drag_params = (DragParameter * max(len(scene.drag), 1))(*scene.drag)
        self.drag_num = len(scene.drag)
        self.drag_acc = f3()
        self.drag_temperature = np.zeros(m, np.float32)
        self.magnifier_count = np.zeros(m, np.int32)
        self.turb_visc = np.zeros(m, np.float32)
        self.strain = np.zeros(m, np.float32)
        self.hash = np.zeros(m, np.int32)
        self.index = np.zeros(m, np.int32)
        self.param = scene.param
        self.box = scene.box
        self.max_n = m

    def bindings(self) -> OrcBindings:
        b = OrcBindings()
        b.param = self.param
        b.box = self.box
        b.particle_num = self.n
        b.max_particle_num = self.max_n
        for name in ["id", "pos", "vel", "pressure", "density", "temperature", "kin_visc", "solid_rate", "type",
                     "out_id", "out_pos", "out_vel", "out_pressure", "out_density", "out_temperature",
                     "out_kin_visc", "out_solid_rate", "out_type", "triangles", "stl_distance", "stl_id", "cells",
                     "cell_start", "cell_end", "drag_acc", "drag_temperature", "magnifier_count", "turb_visc",
                     "strain"]:
            setattr(b, name, getattr(self, name).ctypes.data)
        b.tri_params = C.addressof(self.tri_params)
        b.drag_params = C.addressof(self.drag_params)
        b.triangle_num = self.t
        b.cell_num = self.cells_n
        b.drag_num = self.drag_num
        return b

    def copy(self):
        import copy as _copy
        other = _copy.copy(self)
        for k, v in self.__dict__.items():
            if isinstance(v, np.ndarray):
                setattr(other, k, v.copy())
        other.tri_params = (CTriangleParameters * len(self.tri_params))(*self.tri_params)
        other.drag_params = (DragParameter * len(self.drag_params))(*self.drag_params)
        return other


def fast_sqrt_np(x: np.ndarray) -> np.ndarray:
    """The reference's sqrt_stl / sqrt_utility for float32 arrays."""
    x = np.asarray(x, dtype=np.float32)
    xhalf = np.float32(0.5) * x
    i = x.view(np.int32)
    i = np.int32(0x5f3759df) - (i >> 1)
    y = i.view(np.float32)
    y = y * (np.float32(1.5) - xhalf * y * y)
    return np.float32(1.0) / y


def triangle_normals_q(v: np.ndarray) -> np.ndarray:
    """CalcTriangleNormal (IO.cpp:449-467): cross product of the two edges from
    vertex 0, divided by sqrt_stl of its squared length (float)."""
    v = v.astype(np.float32)
    a = v[:, 1] - v[:, 0]
    b = v[:, 2] - v[:, 0]
    n = np.empty_like(a)
    n[:, 0] = a[:, 1] * b[:, 2] - b[:, 1] * a[:, 2]
    n[:, 1] = a[:, 2] * b[:, 0] - b[:, 2] * a[:, 0]
    n[:, 2] = a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1]
    ab = fast_sqrt_np(n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1] + n[:, 2] * n[:, 2])
    out = n / ab[:, None]
    out[ab == 0] = 0
    return out.astype(np.float32)


def ref_topology(lib: Lib, st: RefState, b: OrcBindings) -> None:
    """CCellSet::RegisterParticleTopology without the compaction (CGPUCellSet.cpp:980-1031)."""
    n = st.n
    lib.calc_hash(C.byref(b), n, ptr(st.hash), ptr(st.index), ptr(st.out_pos))
    if hasattr(lib, "sort"):
        lib.sort(n, ptr(st.hash), ptr(st.index))
    else:
        order = np.argsort(st.hash[:n], kind="stable")
        st.hash[:n] = st.hash[:n][order]
        st.index[:n] = st.index[:n][order]
    lib.reorder_find_cell_start(C.byref(b), n, st.cells_n, ptr(st.hash), ptr(st.index), ptr(st.cell_start),
                                ptr(st.cell_end))


class OracleSim:
    """The FP64 semi-implicit solver of the oracle (no reference counterpart)."""

    def __init__(self, scene, cg_rtol=1e-8, compressibility=1e-9, cg_max_iter=5000, threads=0,
                 source_relaxation=0.05):
        self.lib = oracle()
        cfg = OrcSimConfig()
        cfg.param = scene.param
        cfg.box = scene.box
        cfg.n0_pnd = scene.n0_pnd
        cfg.n0_lap = scene.n0_lap
        cfg.lambda_ = scene.lam
        cfg.compressibility = compressibility
        cfg.cg_rtol = cg_rtol
        cfg.cg_max_iter = cg_max_iter
        cfg.threads = threads
        cfg.source_relaxation = source_relaxation
        self.cfg = cfg
        self.scene = scene
        self.h = self.lib.sim_create(C.byref(cfg), scene.n)
        pos = np.ascontiguousarray(scene.pos, np.float64)
        vel = np.ascontiguousarray(scene.vel, np.float64)
        pr = np.ascontiguousarray(scene.press, np.float64)
        vi = np.ascontiguousarray(scene.visc, np.float64)
        ty = np.ascontiguousarray(scene.ptype, np.int32)
        self.lib.sim_set_particles(self.h, scene.n, ptr(pos), ptr(vel), ptr(pr), ptr(vi), ptr(ty))
        if scene.t:
            v = np.ascontiguousarray(scene.tri_vertices.reshape(-1, 9), np.float64)
            m = np.ascontiguousarray(scene.tri_model, np.int32)
            tp = (CTriangleParameters * len(scene.tri_params))(*scene.tri_params)
            self.lib.sim_set_triangles(self.h, scene.t, ptr(v), ptr(m), len(scene.tri_params), C.addressof(tp))
        if scene.drag:
            dp = (DragParameter * len(scene.drag))(*scene.drag)
            self.lib.sim_set_drag(self.h, len(scene.drag), C.addressof(dp))

    def step(self, i):
        st = OrcStepStats()
        rc = self.lib.sim_step(self.h, i, C.byref(st))
        return rc, {k: getattr(st, k) for k, _ in st._fields_}

    def state(self):
        n0 = self.scene.n
        n = C.c_int()
        pos, vel = np.zeros((n0, 3)), np.zeros((n0, 3))
        press, pnd = np.zeros(n0), np.zeros(n0)
        ids = np.zeros(n0, np.int32)
        self.lib.sim_get(self.h, C.byref(n), ptr(pos), ptr(vel), ptr(press), ptr(pnd))
        self.lib.sim_get_ids(self.h, ptr(ids))
        k = n.value
        o = np.argsort(ids[:k], kind="stable")
        return {"pos": pos[:k][o], "vel": vel[:k][o], "press": press[:k][o], "pnd": pnd[:k][o], "id": ids[:k][o]}

    def matrix(self):
        """The last solve's PPE operator (scipy CSR, solver order), the right-hand side
        and the solver-order particle ids and positions."""
        import scipy.sparse as sp
        n0 = self.scene.n
        nnz = int(self.lib.sim_last_matrix(self.h, None, None, None))
        rowptr = np.zeros(n0 + 1, np.int32)
        col = np.zeros(nnz, np.int32)
        val = np.zeros(nnz)
        self.lib.sim_last_matrix(self.h, ptr(rowptr), ptr(col), ptr(val))
        n = int(np.flatnonzero(rowptr[1:] == nnz)[0]) + 1 if nnz else 0
        pnd, diag, rhs, sol = (np.zeros(n0) for _ in range(4))
        sid = np.zeros(n0, np.int32)
        self.lib.sim_last_ppe(self.h, ptr(pnd), ptr(diag), ptr(rhs), ptr(sol), ptr(sid))
        nb = self.neighbours_sorted()
        A = sp.csr_matrix((val, col, rowptr[:n + 1]), shape=(n, n))
        return A, rhs[:n], sol[:n], nb[:n]

    def neighbours_sorted(self):
        n0 = self.scene.n
        cnt = np.zeros(n0, np.int32)
        idsum = np.zeros(n0)
        pid = np.zeros(n0, np.int32)
        k = self.lib.sim_last_nbr(self.h, ptr(cnt), ptr(idsum), ptr(pid))
        return pid[:k]

    def neighbours(self):
        n0 = self.scene.n
        cnt = np.zeros(n0, np.int32)
        idsum = np.zeros(n0)
        pid = np.zeros(n0, np.int32)
        k = self.lib.sim_last_nbr(self.h, ptr(cnt), ptr(idsum), ptr(pid))
        o = np.argsort(pid[:k], kind="stable")
        return {"id": pid[:k][o], "nbr_count": cnt[:k][o], "nbr_idsum": idsum[:k][o]}

    def close(self):
        if self.h:
            self.lib.sim_destroy(self.h)
            self.h = None


def thermal_scene(sc, seed):
    """Turns on the temperature operator of `sc` with conductivities, wall temperatures
    and clamps that give a visible heat step on a small block; returns a setup hook
    that draws the initial temperatures (out_temperature, original order)."""
    p = sc.param
    p.bUpdateTemperature = True
    p.TemperatureInfluenceRadiusCoefficient = 2.1
    p.FruidThermalConductivity, p.FruidThermalResistance = 0.6, 2e-4
    p.WallThermalConductivity, p.WallThermalResistance = 16.0, 1e-3
    p.FruidSpecificHeat = 4186.0
    p.MaxWallTemperature, p.MinWallTemperature = 330.0, 290.0
    p.ViscosityUpdateParameterA, p.ViscosityUpdateParameterB = -2e-8, 7e-6
    p.Dt = 0.01
    for tp in sc.tri_params:
        tp.Temperature, tp.WallThermalConductivity, tp.WallThermalResistivity = 340.0, 20.0, 5e-4

    def setup(st):
        rng = np.random.default_rng(seed)
        st.out_temperature[:st.n] = rng.uniform(295, 325, st.n).astype(np.float32)
    return setup


def turbulent_scene(sc, seed):
    """Turns on the Smagorinsky turbulence model of `sc` (viscosity cap reached on a
    block with random velocities of 0.5 m/s)."""
    p = sc.param
    p.bTurbulance = True
    p.SmagorinskyConstant, p.FilterWidth = 0.12, 0.02
    p.TurbulanViscosityRatio, p.Cnue, p.Cepsilon, p.TurbulanceIntensity = 2e-5, 0.094, 1.048, 0.5
    sc.vel = np.random.default_rng(seed + 7).normal(0, 0.5, sc.pos.shape)


def linear_walls_scene(seed=0):
    """A block whose box walls are split over three models: model 0 fixed, models 1
    and 2 moving linearly (LinearMovableOrNot) with reset intervals 3 and 5; for
    ResetWallPosition (DeviceProcess_Kernel.h:690-704)."""
    from simulation_project_gb300 import scenes
    sc = scenes.random_block(6, seed=seed)
    rng = np.random.default_rng(seed)
    sc.tri_model = rng.integers(0, 3, size=sc.t).astype(np.int32)
    tps = [scenes._tri_normal_params(dt=sc.param.Dt) for _ in range(3)]
    for m, (vel, interval) in ((1, ((0.3, -0.1, 0.05), 3)), (2, ((-0.2, 0.0, 0.4), 5))):
        tps[m].Velocity = Scalar3(*vel)
        tps[m].LinearMovableOrNot = True
        tps[m].LinearResetInterval = interval
    tps[0].LinearResetInterval = 2   # not movable: never reset
    sc.tri_params = tps
    return sc
