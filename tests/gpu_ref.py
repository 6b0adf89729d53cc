"""Device mirror of an oracle RefState bound through the reference-named C-ABI
(include/mps_device_process.h).  Test helper."""
import ctypes as C

import numpy as np

import orc
from simulation_project_gb300 import lib
from simulation_project_gb300.lib import DeviceArray, call

ARRAYS = ["id", "pos", "vel", "pressure", "density", "temperature", "kin_visc", "solid_rate", "type",
          "out_id", "out_pos", "out_vel", "out_pressure", "out_density", "out_temperature", "out_kin_visc",
          "out_solid_rate", "out_type", "triangles", "stl_distance", "stl_id", "cells", "cell_start", "cell_end",
          "drag_acc", "drag_temperature", "magnifier_count", "turb_visc", "strain", "hash", "index"]


class GpuRef:
    def __init__(self, st: "orc.RefState"):
        lib.load()
        self.st = st
        self.d = {k: DeviceArray.from_host(getattr(st, k)) for k in ARRAYS}
        self.tp = DeviceArray.from_host(np.frombuffer(bytes(st.tri_params), dtype=np.uint8))
        self.dp = DeviceArray.from_host(np.frombuffer(bytes(st.drag_params), dtype=np.uint8))
        self.stream = lib.Stream()
        self.bind()

    def p(self, k):
        return self.d[k].ptr

    def bind(self):
        st = self.st
        call("InitializeDeviceMemConst", st.param, st.n, self.p("triangles"), st.t, self.tp.ptr, st.max_n,
             self.p("stl_distance"), self.p("stl_id"), self.p("cells"), st.cells_n, self.p("cell_start"),
             self.p("cell_end"), self.p("index"), st.box)
        call("InitializeDeviceConstOutPutParticles", *[self.p(k) for k in
             ["out_id", "out_pos", "out_vel", "out_pressure", "out_density", "out_temperature", "out_kin_visc",
              "out_solid_rate", "out_type"]])
        call("InitializeDeviceConstInputParticles", *[self.p(k) for k in
             ["id", "pos", "vel", "pressure", "density", "temperature", "kin_visc", "solid_rate", "type",
              "turb_visc", "strain"]])
        call("DragParametersToConst", self.dp.ptr, self.p("drag_acc"), self.p("drag_temperature"), st.drag_num,
             self.p("magnifier_count"), None)

    def topology(self, n):
        s = self.stream.ref()
        call("CaculateCellIDandInitializeHash", s, n, self.st.cells_n, self.p("hash"), self.p("index"),
             self.p("out_pos"))
        self.stream.sync()
        call("SortUsingThrust", n, self.p("hash"), self.p("index"))
        call("reorderDataAndFindCellStart", s, n, self.st.cells_n, self.p("hash"), self.p("index"),
             self.p("cell_start"), self.p("cell_end"))
        self.stream.sync()

    def walls(self):
        s = self.stream.ref()
        call("ResetTriangleTopology", s, self.st.cells_n, self.p("cells"))
        call("RegisterTriangleTopology", s, self.p("triangles"), self.st.t, self.p("cells"), self.st.cells_n)
        self.stream.sync()

    def run(self, name, n):
        call(name, self.stream.ref(), n)
        self.stream.sync()

    def download(self):
        return {k: v.download() for k, v in self.d.items()}
