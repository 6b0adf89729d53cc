"""The reference's own particle kernels compiled for sm_103a (oracle/_ref/librefgpu*.so,
oracle/ref_gpu_harness.cu) on the GB300, beside the library's reference-named launchers.

* Parity: built without multiply-add contraction, the reference's CalcSTLDistance,
  CalcDragEffect, CalcExplicitly, CalcExplicitPressure and CalcExplicitPressureGradient
  kernels give bit-identical outputs to the library's launchers over several steps of
  the rotating bucket (radix/SPVSOLVER/MultiGPUSolver/DeviceProcess_Kernel.h:309-1271).
* Second baseline: per-kernel CUDA-event times of the reference's kernels as its project
  builds them (nvcc's default contraction) against the library's, on the bucket at
  l0 = 0.004 and 0.002, printed (run with -s).

Topology (hash, sort, cell tables, reorder, triangle binning) comes from the library's
launchers in both runs: the reference's reorder reads hash[-1] and its triangle binning
races on the per-cell counts, so neither runs here (see the harness's header).  The
per-particle arrays have room for the reference's whole thread grid (its STL kernel has
no thread guard)."""
import ctypes as C
import os

import numpy as np
import pytest

import orc
from simulation_project_gb300 import lib, scenes
from simulation_project_gb300.refpath import RefStep

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KERNEL_IDS = {"CalcSTLDistance": 0, "CalcDragEffect": 1, "CalcExplicitly": 2, "CalcExplicitPressure": 3,
              "CalcExplicitPressureGradient": 4}


def _refgpu(nofma: bool):
    path = os.path.join(ROOT, "oracle", "_ref", "librefgpu_nofma.so" if nofma else "librefgpu.so")
    if not os.path.exists(path):
        pytest.skip("the reference's kernels are not built here (no decoded sources)")
    g = C.CDLL(path)
    g.refgpu_bind.argtypes = [C.POINTER(orc.OrcBindings)]
    g.refgpu_launch.argtypes = [C.c_int, C.c_void_p, C.c_int]
    g.refgpu_particle_num.argtypes = [C.c_int]
    return g


class RefGpuStep(RefStep):
    """RefStep whose five particle kernels are the reference's own (g: a librefgpu
    library), on the same device arrays and stream.  The library's reference-named
    launchers keep one binding per process (as the reference's __constant__ symbols
    do), so the comparisons below use one such object and run both sides on its arrays."""

    def __init__(self, scene, g):
        self.g = g
        super().__init__(scene, capacity=g.refgpu_grid_items(scene.n))
        b = orc.OrcBindings()
        b.param, b.box = self.param, self.box
        b.particle_num, b.max_particle_num = self.n, self.capacity
        for k in ("id", "pos", "vel", "pressure", "density", "temperature", "kin_visc", "solid_rate", "type",
                  "out_id", "out_pos", "out_vel", "out_pressure", "out_density", "out_temperature", "out_kin_visc",
                  "out_solid_rate", "out_type", "triangles", "stl_distance", "stl_id", "cells", "cell_start",
                  "cell_end", "drag_acc", "drag_temperature", "magnifier_count", "turb_visc", "strain"):
            setattr(b, k, self.p(k))
        b.triangle_num, b.cell_num, b.drag_num = self.t, self.cells, self.drag_num
        b.tri_params, b.drag_params = self.tp.ptr, self.dp.ptr
        self.bind = b
        assert g.refgpu_bind(C.byref(b)) == 0

    def _kernel(self, name, n):
        assert self.g.refgpu_particle_num(n) == 0
        assert self.g.refgpu_launch(KERNEL_IDS[name], self.stream.handle, n) == 0

    def library_kernel(self, name, n):
        RefStep._kernel(self, name, n)

    def snapshot(self):
        self.sync()
        return {k: a.download() for k, a in self.d.items()}

    def restore(self, snap):
        self.sync()
        for k, a in self.d.items():
            a.upload(snap[k])


class ABStep(RefGpuStep):
    """Every particle kernel of the step run twice from the same state, the library's
    launcher first and then the reference's kernel; the first particle_num entries of
    every array must agree bit for bit; the step continues from the reference's."""

    def _kernel(self, name, n):
        s0 = self.snapshot()
        self.library_kernel(name, n)
        ours = self.snapshot()
        self.restore(s0)
        super()._kernel(name, n)
        ref = self.snapshot()
        for k in self.d:
            assert ours[k][:n].tobytes() == ref[k][:n].tobytes(), (name, k)
        self.checked.append(name)


def _bucket(l0):
    return scenes.rotating_bucket(l0=l0, explicit_pressure=True)


def test_reference_kernels_on_the_gpu_match_the_library_bit_for_bit():
    g = _refgpu(nofma=True)
    sc = _bucket(0.004)
    s = ABStep(sc, g)
    s.checked = []
    for i in range(3):
        assert s.step(i) == sc.n
    assert len(s.checked) == 3 * 6   # STL x2, drag, predictor, pressure, gradient per step
    s.close()


def _kernel_times(launch, names, stream, reps):
    ev0, ev1 = lib.Event(), lib.Event()
    out = {}
    for name in names:
        launch(name)
        stream.sync()
        ev0.record(stream)
        for _ in range(reps):
            launch(name)
        ev1.record(stream)
        stream.sync()
        out[name] = ev0.elapsed_ms(ev1) / reps * 1e3
    return out


@pytest.mark.parametrize("l0", [0.004, 0.002])
def test_reference_kernels_timed_beside_the_library(l0):
    """Per-kernel times (us) of the reference's kernels as its project builds them
    (nvcc's default contraction) and of the library's reference-named launchers, on the
    same bound state after two steps (each kernel's outputs depend only on its inputs,
    so repeated launches redo the same work)."""
    g = _refgpu(nofma=False)
    sc = _bucket(l0)
    s = RefGpuStep(sc, g)
    for i in range(2):
        s.step(i)
    n = s.n
    names = [k for k in RefStep.PARTICLE_KERNELS if k != "CalcDragEffect" or s.drag_num]
    reps = 10 if n < 300_000 else 4
    t_ref = _kernel_times(lambda k: s._kernel(k, n), names, s.stream, reps)
    t_ours = _kernel_times(lambda k: s.library_kernel(k, n), names, s.stream, reps)
    print(f"\nl0 = {l0}: {n} particles, {sc.t} triangles")
    print("kernel                         reference sm_103a (us)   library (us)   ratio")
    for k in names:
        print(f"{k:30s} {t_ref[k]:14.1f} {t_ours[k]:16.1f} {t_ref[k] / t_ours[k]:9.2f}")
    tr, to = sum(t_ref.values()), sum(t_ours.values())
    print(f"{'sum':30s} {tr:14.1f} {to:16.1f} {tr / to:9.2f}")
    assert all(v > 0 for v in t_ref.values()) and all(v > 0 for v in t_ours.values())
    s.close()
