"""The reference's explicit per-step schedule through the reference-named C-ABI
(include/mps_device_process.h): what a CCellSet caller that links libmps_gb300.so runs.

    s = RefStep(scene)          # allocates and binds CCellSet's device arrays
    n = s.step(i)               # one step of CMultiGPUHandler::Calculate, explicit pressure
    s.close()

The device arrays are the ones CCellSet allocates (radix/SPVSOLVER/MultiGPUSolver/
CGPUCellSet.cpp:487-635): input (sorted) and output (particle-order) particle arrays,
triangles, per-particle wall distance and id, triangle cells, cell start/end, drag
arrays, hash and index.  One step follows CMultiGPUHandler::Calculate
(MultiGPUHandler.cpp:1389-1540) for a single grid: compaction of particles outside the
compute zone, topology (hash, sort, reorder), triangle cells, wall distance, drag, the
viscosity/gravity predictor (CalcExplicitly), topology and wall distance again, the
explicit pressure and its gradient correction, then the walls move.  Every call is a
launcher of the library; there is no host computation on the particle data.
"""
import ctypes as C

import numpy as np

from . import lib
from .lib import DeviceArray, call
from .types import CTriangleParameters, DragParameter, CELL_DTYPE, DISTANCE_DTYPE, TRIANGLE_DTYPE


def _sqrt_stl(x):
    """The reference's sqrt_stl (STLSerializer.h:23-31): 1 / fast inverse square root,
    one Newton step, in float."""
    x = np.asarray(x, np.float32)
    half = np.float32(0.5) * x
    i = np.int32(0x5f3759df) - (x.view(np.int32) >> 1)
    y = i.view(np.float32)
    y = y * (np.float32(1.5) - half * y * y)
    return np.float32(1.0) / y


def triangle_records(vertices, models):
    """CTriangle records with the reference's normals (CalcTriangleNormal, IO.cpp:449-467)."""
    t = len(vertices)
    rec = np.zeros(max(t, 1), TRIANGLE_DTYPE)
    v = np.asarray(vertices, np.float32).reshape(-1, 3, 3)
    rec["ModelIDNumber"][:t] = models
    rec["Vertex"][:t] = v
    a, b = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
    n = np.empty_like(a)
    n[:, 0] = a[:, 1] * b[:, 2] - b[:, 1] * a[:, 2]
    n[:, 1] = a[:, 2] * b[:, 0] - b[:, 2] * a[:, 0]
    n[:, 2] = a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1]
    with np.errstate(divide="ignore", invalid="ignore"):
        ab = _sqrt_stl(n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1] + n[:, 2] * n[:, 2])
        nn = n / ab[:, None]
    nn[ab == 0] = 0
    rec["Normal"][:t] = nn
    return rec


class RefStep:
    """CCellSet's device arrays for one scene, bound once, and the explicit step."""

    IN = ["id", "pos", "vel", "pressure", "density", "temperature", "kin_visc", "solid_rate", "type"]

    # the particle launchers of the step, in call order; _kernel runs them
    PARTICLE_KERNELS = ("CalcSTLDistance", "CalcDragEffect", "CalcExplicitly", "CalcExplicitPressure",
                        "CalcExplicitPressureGradient")

    def __init__(self, scene, explicit_sonic=20.0, capacity=None):
        """capacity: entries allocated per particle array (>= the particle count; the
        entries past it are zero), for callers whose kernels touch whole thread grids."""
        lib.load()
        p = scene.param
        p.bExplicitPressure = True
        p.SonicVelocity = explicit_sonic
        self.param, self.box = p, scene.box
        n = scene.n
        self.n = n
        cap = n if capacity is None else max(int(capacity), n)
        self.capacity = cap
        self.cells = scene.box.cell_num
        self.t = scene.t
        f3 = lambda: np.zeros((n, 3), np.float32)  # noqa: E731
        host = {
            "out_id": np.arange(n, dtype=np.int32), "out_pos": scene.pos.astype(np.float32),
            "out_vel": scene.vel.astype(np.float32), "out_pressure": scene.press.astype(np.float32),
            "out_density": np.zeros(n, np.float32), "out_temperature": np.zeros(n, np.float32),
            "out_kin_visc": scene.visc.astype(np.float32), "out_solid_rate": np.zeros(n, np.float32),
            "out_type": scene.ptype.astype(np.int32),
            "id": np.zeros(n, np.int32), "pos": f3(), "vel": f3(), "pressure": np.zeros(n, np.float32),
            "density": np.zeros(n, np.float32), "temperature": np.zeros(n, np.float32),
            "kin_visc": np.zeros(n, np.float32), "solid_rate": np.zeros(n, np.float32), "type": np.zeros(n, np.int32),
            "triangles": triangle_records(scene.tri_vertices, scene.tri_model),
            "stl_distance": np.zeros(n, DISTANCE_DTYPE), "stl_id": np.full(n, -1, np.int32),
            "cells": np.zeros(self.cells, CELL_DTYPE), "cell_start": np.full(self.cells, -1, np.int32),
            "cell_end": np.full(self.cells, -1, np.int32), "drag_acc": f3(), "drag_temperature": np.zeros(n, np.float32),
            "magnifier_count": np.zeros(n, np.int32), "turb_visc": np.zeros(n, np.float32),
            "strain": np.zeros(n, np.float32), "hash": np.zeros(n, np.int32), "index": np.zeros(n, np.int32),
        }
        if cap > n:
            for k, v in host.items():
                if k not in ("triangles", "cells", "cell_start", "cell_end") and v.shape[0] == n:
                    pad = np.zeros((cap - n,) + v.shape[1:], v.dtype)
                    host[k] = np.concatenate([v, pad])
        self.d = {k: DeviceArray.from_host(np.ascontiguousarray(v)) for k, v in host.items()}
        tp = (CTriangleParameters * max(len(scene.tri_params), 1))(*scene.tri_params)
        dp = (DragParameter * max(len(scene.drag), 1))(*scene.drag)
        self.tp = DeviceArray.from_host(np.frombuffer(bytes(tp), dtype=np.uint8).copy())
        self.dp = DeviceArray.from_host(np.frombuffer(bytes(dp), dtype=np.uint8).copy())
        self.drag_num = len(scene.drag)
        self.stream = lib.Stream()
        d = self.p
        call("InitializeDeviceMemConst", p, n, d("triangles"), self.t, self.tp.ptr, n, d("stl_distance"),
             d("stl_id"), d("cells"), self.cells, d("cell_start"), d("cell_end"), d("index"), scene.box)
        call("InitializeDeviceConstOutPutParticles", *[d(k) for k in
             ["out_id", "out_pos", "out_vel", "out_pressure", "out_density", "out_temperature", "out_kin_visc",
              "out_solid_rate", "out_type"]])
        call("InitializeDeviceConstInputParticles", *[d(k) for k in self.IN + ["turb_visc", "strain"]])
        call("DragParametersToConst", self.dp.ptr, d("drag_acc"), d("drag_temperature"), self.drag_num,
             d("magnifier_count"), None)

    def p(self, k):
        return self.d[k].ptr

    def _topology(self, n):
        s, d = self.stream.ref(), self.p
        call("CaculateCellIDandInitializeHash", s, n, self.cells, d("hash"), d("index"), d("out_pos"))
        self.stream.sync()   # SortUsingThrust runs on the legacy default stream
        call("SortUsingThrust", n, d("hash"), d("index"))
        call("reorderDataAndFindCellStart", s, n, self.cells, d("hash"), d("index"), d("cell_start"),
             d("cell_end"))

    def step(self, i: int) -> int:
        s, d = self.stream.ref(), self.p
        cnt = C.c_int(self.n)
        call("CheckParticleOutsideComputeZone", s, C.byref(cnt))
        n = self.n = cnt.value
        call("ParticleNumberToConst", n)
        self._topology(n)
        call("ResetTriangleTopology", s, self.cells, d("cells"))
        call("RegisterTriangleTopology", s, d("triangles"), self.t, d("cells"), self.cells)
        self._kernel("CalcSTLDistance", n)
        if self.drag_num:
            self._kernel("CalcDragEffect", n)
        self._kernel("CalcExplicitly", n)
        self._topology(n)
        self._kernel("CalcSTLDistance", n)
        self._kernel("CalcExplicitPressure", n)
        self._kernel("CalcExplicitPressureGradient", n)
        call("UpdateTrianglePosition", s, self.t, d("triangles"))
        call("RotateTrianglePosition", s, self.t, d("triangles"), i)
        return n

    def _kernel(self, name, n):
        """One of PARTICLE_KERNELS over n particles on the step's stream."""
        call(name, self.stream.ref(), n)

    def sync(self):
        self.stream.sync()

    def download(self, k):
        self.sync()
        return self.d[k].download()

    def close(self):
        for a in self.d.values():
            a.free()
        self.tp.free()
        self.dp.free()
        self.d = {}


def main(argv=None):
    """python -m simulation_project_gb300.refpath [--l0 L] [--steps K] [--warmup W]: the
    explicit reference schedule on the rotating bucket through the reference-named
    launchers, wall time per step (the command the launch-list profile runs)."""
    import argparse
    import json
    import time
    from . import scenes
    ap = argparse.ArgumentParser()
    ap.add_argument("--l0", type=float, default=0.002)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=2)
    a = ap.parse_args(argv)
    sc = scenes.rotating_bucket(l0=a.l0, dt=5e-5, seed=4, n_drag=64, drag_seed=3)
    g = RefStep(sc)
    for i in range(a.warmup):
        g.step(i)
    g.sync()
    t0 = time.perf_counter()
    for i in range(a.steps):
        g.step(a.warmup + i)
    g.sync()
    dt = time.perf_counter() - t0
    g.close()
    print(json.dumps({"particles": sc.n, "steps": a.steps, "ms_per_step": dt * 1e3 / max(a.steps, 1)}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
