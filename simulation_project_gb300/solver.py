"""Python front end of the GB300-native semi-implicit step (include/mps_solver.h).

    s = Solver(scene, precision="fp32_ir")
    stats = s.step(0)
    state = s.state()          # dict of numpy arrays in particle-id order

The scene supplies the reference's parameter / grid / wall / drag structs
(simulation_project_gb300.scenes.Scene).  All compute runs in libmps_gb300.so.
"""
import ctypes as C

import numpy as np

from . import lib
from .types import CParameter, CGridBox, CTriangleParameters, DragParameter, MpsError

PREC = {"fp64": 0, "fp32_ir": 1}
PRESSURE = {"ppe": 0, "explicit": 1}


class MpsSolverOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("pressure_mode", C.c_int), ("learned", C.c_int), ("n0_pnd", C.c_double),
                ("n0_lap", C.c_double), ("lambda_", C.c_double), ("compressibility", C.c_double),
                ("cg_rtol", C.c_double), ("cg_max_iter", C.c_int), ("ir_inner_rtol", C.c_double),
                ("ir_max_outer", C.c_int), ("max_neighbours", C.c_int), ("check_every", C.c_int),
                ("source_relaxation", C.c_double), ("profile", C.c_int), ("preconditioner", C.c_int),
                ("mg_omega", C.c_double), ("compress_rows", C.c_int), ("mg_sweeps", C.c_int),
                ("matrix_free", C.c_int), ("spmv_stream", C.c_int), ("inner_weights", C.c_int),
                ("spmv_wide", C.c_int), ("warm_start", C.c_int), ("flexible", C.c_int),
                ("learned_gate", C.c_int), ("fine_smoother", C.c_int), ("smoother_weight", C.c_double),
                ("rows_sell", C.c_int)]


class MpsStepStats(C.Structure):
    _fields_ = [("particles", C.c_int), ("interior", C.c_int), ("cg_iterations", C.c_int), ("ir_passes", C.c_int),
                ("fallback", C.c_int), ("max_row", C.c_int), ("cg_relres", C.c_double), ("b_norm", C.c_double),
                ("error_flags", C.c_uint), ("nnz", C.c_longlong), ("pairs", C.c_longlong),
                ("ms_grid", C.c_float), ("ms_walls", C.c_float), ("ms_predictor", C.c_float), ("ms_list", C.c_float),
                ("ms_ppe_setup", C.c_float), ("ms_spmv", C.c_float), ("ms_cg_vec", C.c_float),
                ("ms_correct", C.c_float), ("ms_learned", C.c_float), ("spmv_launches", C.c_int),
                ("ms_precond", C.c_float), ("mg_levels", C.c_int), ("mg_level1", C.c_int),
                ("r0_relres", C.c_double), ("nnz_wide", C.c_longlong), ("rows16", C.c_int),
                ("inner16", C.c_int), ("warm_start", C.c_int), ("learned_applied", C.c_int),
                ("learned_saved_its", C.c_float), ("learned_cost_its", C.c_float), ("flexible", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MpsLearnedInfo(C.Structure):
    _fields_ = [("samples", C.c_int), ("val_samples", C.c_int), ("adam_steps", C.c_int), ("batch", C.c_int),
                ("val_loss_before", C.c_float), ("val_loss_after", C.c_float), ("collect_ms", C.c_double),
                ("train_ms", C.c_double)]


P = C.c_void_p
_SIGS = {
    "mps_solver_default_options": (None, [C.POINTER(MpsSolverOptions)]),
    "mps_solver_create": (C.c_int, [C.POINTER(CParameter), C.POINTER(CGridBox), C.c_int,
                                    C.POINTER(MpsSolverOptions), C.POINTER(P)]),
    "mps_solver_destroy": (None, [P]),
    "mps_solver_set_particles": (C.c_int, [P, C.c_int, P, P, P, P, P]),
    "mps_solver_set_triangles": (C.c_int, [P, C.c_int, P, P, C.c_int, P]),
    "mps_solver_set_drag": (C.c_int, [P, C.c_int, P]),
    "mps_solver_step": (C.c_int, [P, C.c_int, C.POINTER(MpsStepStats)]),
    "mps_solver_get_particles": (C.c_int, [P, C.POINTER(C.c_int), P, P, P, P, P]),
    "mps_solver_get_triangles": (C.c_int, [P, P]),
    "mps_solver_debug_residual": (C.c_int, [P, C.c_int, P, C.POINTER(C.c_double)]),
    "mps_solver_debug_ppe": (C.c_int, [P, P, P, P, P, P, P, P]),
    "mps_solver_debug_history": (C.c_int, [P, P, P, P, P, P]),
    "mps_solver_debug_spmv": (C.c_int, [P, C.c_int, P, P]),
    "mps_solver_debug_level1": (C.c_int, [P, C.c_int, P, C.c_int, C.POINTER(C.c_int)]),
    "mps_solver_debug_wall_bins": (C.c_int, [P, P, P, C.c_int, C.POINTER(C.c_int)]),
    "mps_solver_save_frame": (C.c_int, [P, C.c_char_p, C.c_int, C.c_double, C.c_int, P, P]),
    "mps_solver_add_particles": (C.c_int, [P, C.c_int, P, C.POINTER(C.c_int)]),
    "mps_solver_set_time_step": (C.c_int, [P, C.c_double, C.c_double]),
    "mps_solver_wait_frames": (C.c_int, [P]),
    "mps_solver_copy_pressure": (C.c_int, [P, P]),
    "mps_solver_stream": (C.c_int, [P, C.POINTER(P)]),
    "mps_solver_upload_state": (C.c_int, [P, P, P, P]),
    "mps_solver_download_state": (C.c_int, [P, P, P, P]),
    "mps_solver_set_learned": (C.c_int, [P, P, C.c_int]),
    "mps_solver_learned_samples": (C.c_int, [P, P, P, C.POINTER(C.c_int)]),
    "CalculatePressureCG": (C.c_int, [P, C.POINTER(MpsStepStats)]),
    "CalculatePressureNJPCG": (C.c_int, [P, C.POINTER(MpsStepStats)]),
    "mps_set_precision": (C.c_int, [P, C.c_int]),
    "CalcPoisson": (C.c_int, [P, P, C.c_int, P, P, P, P, C.POINTER(MpsStepStats)]),
    "mps_learned_train": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_ulonglong,
                                    C.POINTER(MpsLearnedInfo)]),
    "mps_learned_infer": (C.c_int, [P, P, C.POINTER(C.c_int)]),
    "mps_solver_collect": (C.c_int, [P, C.c_int]),
}
_bound = False


def _lib():
    global _bound
    L = lib.load()
    if not _bound:
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _bound = True
    return L


def _check(rc, what):
    if rc != 0:
        raise MpsError(rc, f"{what} ({lib.load().mps_last_error().decode()})")


def default_options(precision="fp32_ir", **kw) -> MpsSolverOptions:
    o = MpsSolverOptions()
    _lib().mps_solver_default_options(C.byref(o))
    o.precision = PREC[precision]
    for k, v in kw.items():
        setattr(o, "lambda_" if k == "lam" else k, v)
    return o


# numpy view of the reference's CParticle record (DataType.h:220-240)
CPARTICLE_DTYPE = np.dtype([("ID", "<i4"), ("Position", "<f4", 3), ("Velocity", "<f4", 3), ("Pressure", "<f4"),
                            ("Density", "<f4"), ("Temperature", "<f4"), ("KineticViscosity", "<f4"),
                            ("SolidPhaseRate", "<f4"), ("Type", "<i4")])


def _p(a):
    return None if a is None else a.ctypes.data


class Solver:
    def __init__(self, scene, precision="fp32_ir", physics=True, max_particles=None, **opts):
        L = _lib()
        o = default_options(precision, **opts)
        if physics:
            if o.n0_pnd <= 0:
                o.n0_pnd = scene.n0_pnd
            if o.n0_lap <= 0:
                o.n0_lap = scene.n0_lap
            if o.lambda_ <= 0:
                o.lambda_ = scene.lam
        self.options = o
        self.scene = scene
        h = P()
        # host buffers of the state are sized for this capacity: inflow can raise the
        # particle count above the scene's
        self.capacity = int(max_particles or scene.n)
        _check(L.mps_solver_create(C.byref(scene.param), C.byref(scene.box), self.capacity,
                                   C.byref(o), C.byref(h)), "mps_solver_create")
        self.h = h
        pos = np.ascontiguousarray(scene.pos, dtype=np.float64)
        vel = np.ascontiguousarray(scene.vel, dtype=np.float64)
        press = np.ascontiguousarray(scene.press, dtype=np.float64)
        visc = np.ascontiguousarray(scene.visc, dtype=np.float64)
        ptype = np.ascontiguousarray(scene.ptype, dtype=np.int32)
        _check(L.mps_solver_set_particles(h, scene.n, _p(pos), _p(vel), _p(press), _p(visc), _p(ptype)),
               "mps_solver_set_particles")
        if scene.t > 0:
            v = np.ascontiguousarray(scene.tri_vertices.reshape(-1, 9), dtype=np.float64)
            m = np.ascontiguousarray(scene.tri_model, dtype=np.int32)
            tp = (CTriangleParameters * len(scene.tri_params))(*scene.tri_params)
            _check(L.mps_solver_set_triangles(h, scene.t, _p(v), _p(m), len(scene.tri_params), C.addressof(tp)),
                   "mps_solver_set_triangles")
        if scene.drag:
            dp = (DragParameter * len(scene.drag))(*scene.drag)
            _check(L.mps_solver_set_drag(h, len(scene.drag), C.addressof(dp)), "mps_solver_set_drag")

    def step(self, i: int) -> dict:
        s = MpsStepStats()
        _check(_lib().mps_solver_step(self.h, int(i), C.byref(s)), "mps_solver_step")
        return s.as_dict()

    def state(self, sort_by_id=True) -> dict:
        L = _lib()
        nmax = self.capacity
        n = C.c_int()
        pos = np.zeros((nmax, 3))
        vel = np.zeros((nmax, 3))
        press = np.zeros(nmax)
        pnd = np.zeros(nmax)
        ids = np.zeros(nmax, np.int32)
        _check(L.mps_solver_get_particles(self.h, C.byref(n), _p(pos), _p(vel), _p(press), _p(pnd), _p(ids)),
               "mps_solver_get_particles")
        k = n.value
        out = {"pos": pos[:k], "vel": vel[:k], "press": press[:k], "pnd": pnd[:k], "id": ids[:k]}
        if sort_by_id:
            o = np.argsort(out["id"], kind="stable")
            out = {key: v[o] for key, v in out.items()}
        return out

    def debug_ppe(self) -> dict:
        nmax = self.capacity
        arr = {k: np.zeros(nmax) for k in ("pnd", "diag", "rhs", "sol", "nbr_idsum")}
        ids = np.zeros(nmax, np.int32)
        cnt = np.zeros(nmax, np.int32)
        _check(_lib().mps_solver_debug_ppe(self.h, _p(arr["pnd"]), _p(arr["diag"]), _p(arr["rhs"]), _p(arr["sol"]),
                                           _p(ids), _p(cnt), _p(arr["nbr_idsum"])), "mps_solver_debug_ppe")
        n = self.state(sort_by_id=False)["id"].shape[0]
        out = {k: v[:n] for k, v in arr.items()}
        out["id"] = ids[:n]
        out["nbr_count"] = cnt[:n]
        return out

    def debug_history(self) -> dict:
        """Warm-start pressure history in solver order: dph1 = P_n - P_{n-1}, dph2 =
        P_{n-1} - P_{n-2} (FP32), the interior flags, ids and the number held."""
        n = self.state(sort_by_id=False)["id"].shape[0]
        d1, d2 = np.zeros(max(n, 1), np.float32), np.zeros(max(n, 1), np.float32)
        inner = np.zeros(max(n, 1), np.uint8)
        ids = np.zeros(max(n, 1), np.int32)
        held = C.c_int()
        _check(_lib().mps_solver_debug_history(self.h, _p(d1), _p(d2), _p(inner), _p(ids), C.byref(held)),
               "mps_solver_debug_history")
        return {"dph1": d1[:n], "dph2": d2[:n], "inner": inner[:n].astype(bool), "id": ids[:n], "held": held.value}

    def debug_residual(self, variant: int):
        """(r, ||r|| / ||b||) of the current state: variant 0 FP64 kernel, 1 the
        double-float kernel the solver uses, 2 the double-float register walk."""
        n = self.state(sort_by_id=False)["id"].shape[0]
        r = np.zeros(max(n, 1))
        rel = C.c_double()
        _check(_lib().mps_solver_debug_residual(self.h, int(variant), _p(r), C.byref(rel)), "mps_solver_debug_residual")
        return r[:n], rel.value

    def debug_spmv(self, kernel: int, x: np.ndarray) -> np.ndarray:
        """One FP32 inner SpMV y = A x over the current rows with the named kernel
        (0 register walk, 1 streamed, 3 streamed 32-bit columns, 4 / 8 matrix-free; 2 / 6
        the FP16-weight operator with 16-bit / 32-bit columns), solver order."""
        n = self.state(sort_by_id=False)["id"].shape[0]
        xs = np.ascontiguousarray(x, dtype=np.float32)
        if xs.shape != (n,):
            raise ValueError(f"x must have shape ({n},)")
        y = np.zeros(n, np.float32)
        _check(_lib().mps_solver_debug_spmv(self.h, int(kernel), _p(xs), _p(y)), "mps_solver_debug_spmv")
        return y

    def debug_level1(self, variant: int) -> np.ndarray:
        """Level-1 Galerkin stencil [n1, 27] reassembled from the current rows by the
        register walk (variant 0) or the streamed rows (variant 1)."""
        L = _lib()
        n1 = C.c_int()
        _check(L.mps_solver_debug_level1(self.h, int(variant), None, 0, C.byref(n1)), "mps_solver_debug_level1")
        a = np.zeros((n1.value, 27), np.float32)
        _check(L.mps_solver_debug_level1(self.h, int(variant), _p(a), a.size, C.byref(n1)),
               "mps_solver_debug_level1")
        return a

    def debug_wall_bins(self) -> dict:
        """Per-cell triangle lists of the wall search: {(cell, kind): [triangle ids]} for
        the non-empty lists (kind 0 walls, 1 drag bodies)."""
        L = _lib()
        cells = int(self.scene.box.cell_num)
        nv = C.c_int()
        _check(L.mps_solver_debug_wall_bins(self.h, None, None, 0, C.byref(nv)), "mps_solver_debug_wall_bins")
        bounds = np.zeros(4 * cells, np.int32)
        tids = np.zeros(max(nv.value, 1), np.int32)
        _check(L.mps_solver_debug_wall_bins(self.h, _p(bounds), _p(tids), len(tids), C.byref(nv)),
               "mps_solver_debug_wall_bins")
        ts, te = bounds[:2 * cells], bounds[2 * cells:]
        out = {}
        for c in np.flatnonzero(ts >= 0):
            out[(int(c) // 2, int(c) % 2)] = tids[ts[c]:te[c]].tolist()
        return out

    def set_time_step(self, dt, courant=0.0):
        """Dt (and CourantNumber when > 0) from the next step on (a dt schedule row)."""
        _check(_lib().mps_solver_set_time_step(self.h, float(dt), float(courant)), "mps_solver_set_time_step")

    def add_particles(self, pos, vel=None, press=None, visc=None, ptype=None) -> int:
        """Inflow of a bucket of particles (InsertBucket semantics: the missing IDs first,
        the rest appended if it fits); returns how many were inserted."""
        pos = np.asarray(pos, dtype=np.float32).reshape(-1, 3)
        k = len(pos)
        b = np.zeros(max(k, 1), CPARTICLE_DTYPE)   # CParticle records (52 bytes)
        b["ID"][:k] = -1
        b["Position"][:k] = pos
        if vel is not None:
            b["Velocity"][:k] = np.asarray(vel, np.float32).reshape(k, 3)
        if press is not None:
            b["Pressure"][:k] = press
        b["KineticViscosity"][:k] = 1e-6 if visc is None else np.asarray(visc, np.float32)
        if ptype is not None:
            b["Type"][:k] = ptype
        added = C.c_int()
        _check(_lib().mps_solver_add_particles(self.h, k, b.ctypes.data, C.byref(added)), "mps_solver_add_particles")
        return added.value

    def save_frame(self, path, ascii=False, time=0.0, model_pos=None, model_angle=None):
        """Output frame of the current state (reference format, particles in ID order),
        written by a host thread while later steps run; wait_frames() waits for it."""
        mp = np.ascontiguousarray(np.zeros((0, 3)) if model_pos is None else model_pos, dtype=np.float32).reshape(-1, 3)
        ma = np.ascontiguousarray(np.zeros(0) if model_angle is None else model_angle, dtype=np.float32)
        if len(ma) != len(mp):
            raise ValueError("one angle per model position")
        _check(_lib().mps_solver_save_frame(self.h, str(path).encode(), int(bool(ascii)), float(time), len(ma),
                                            _p(mp), _p(ma)), "mps_solver_save_frame")

    def wait_frames(self):
        _check(_lib().mps_solver_wait_frames(self.h), "mps_solver_wait_frames")

    def pressure(self, njp: bool = False) -> dict:
        """PPE solve at the current state (CalculatePressureNJPCG if njp, else CalculatePressureCG)."""
        st = MpsStepStats()
        f = _lib().CalculatePressureNJPCG if njp else _lib().CalculatePressureCG
        _check(f(self.h, C.byref(st)), "CalculatePressure" + ("NJPCG" if njp else "CG"))
        return st.as_dict()

    def calc_poisson(self, n_ids, d_a, d_b, d_x, d_x0=None, stream=None) -> dict:
        """CalcPoisson on device arrays of n_ids floats indexed by particle ID (device
        pointers as ints; any may be None)."""
        st = MpsStepStats()
        _check(_lib().CalcPoisson(stream, self.h, int(n_ids), d_a, d_b, d_x, d_x0, C.byref(st)), "CalcPoisson")
        return st.as_dict()

    def set_precision(self, precision: str):
        _check(_lib().mps_set_precision(self.h, PREC[precision]), "mps_set_precision")

    def learned_train(self, first_step, steps, max_samples=400_000, epochs=4, batch=8192, lr=2e-3, seed=1) -> dict:
        """mps_learned_train: collect from this solver's own next `steps` steps, train, install."""
        info = MpsLearnedInfo()
        _check(_lib().mps_learned_train(self.h, int(first_step), int(steps), int(max_samples), int(epochs), int(batch),
                                        float(lr), int(seed), C.byref(info)), "mps_learned_train")
        return {k: getattr(info, k) for k, _ in info._fields_}

    def learned_infer(self) -> np.ndarray:
        n = C.c_int()
        out = np.zeros((max(self.capacity, 1), 2), np.float32)
        _check(_lib().mps_learned_infer(self.h, _p(out), C.byref(n)), "mps_learned_infer")
        return out[:n.value]

    def triangles(self) -> np.ndarray:
        v = np.zeros((self.scene.t, 9))
        if self.scene.t:
            _check(_lib().mps_solver_get_triangles(self.h, _p(v)), "mps_solver_get_triangles")
        return v.reshape(-1, 3, 3)

    def set_learned(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        _check(_lib().mps_solver_set_learned(self.h, p.ctypes.data, p.size), "mps_solver_set_learned")

    def collect(self, on=True):
        _check(_lib().mps_solver_collect(self.h, 1 if on else 0), "mps_solver_collect")

    def learned_samples(self):
        """(features [n,12], targets [n,2]) of the last PPE solve, interior rows only."""
        nmax = self.capacity
        f = np.zeros((nmax, 12), np.float32)
        t = np.zeros((nmax, 2), np.float32)
        n = C.c_int()
        _check(_lib().mps_solver_learned_samples(self.h, f.ctypes.data, t.ctypes.data, C.byref(n)),
               "mps_solver_learned_samples")
        f, t = f[:n.value], t[:n.value]
        ok = np.isfinite(t).all(1) & np.isfinite(f).all(1)
        return f[ok], t[ok]

    def upload_state(self, pos, vel, press):
        _check(_lib().mps_solver_upload_state(self.h, pos.ctypes.data, vel.ctypes.data, press.ctypes.data),
               "mps_solver_upload_state")

    def download_state(self, pos, vel, press):
        _check(_lib().mps_solver_download_state(self.h, pos.ctypes.data, vel.ctypes.data, press.ctypes.data),
               "mps_solver_download_state")

    def stream(self):
        s = P()
        _check(_lib().mps_solver_stream(self.h, C.byref(s)), "mps_solver_stream")
        return s.value

    def close(self):
        if getattr(self, "h", None):
            _lib().mps_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
