"""The reference's input formats (include/mps_io.h): parameter file, particle file,
ASCII and binary STL, grid geometry, lambda table, lattice constants.  Host-only."""
import ctypes as C
import os
import struct
import zipfile

import numpy as np
import pytest

from simulation_project_gb300 import build
from simulation_project_gb300.types import CParameter, CGridBox, CBox, Scalar3, CTriangle, CParticle_size
from simulation_project_gb300 import scenes

# input deck of the reference checkout ($MPS_REFERENCE_ROOT, by default /root/reference)
REF_ROOT = os.environ.get("MPS_REFERENCE_ROOT", "/root/reference")
TD = os.path.join(REF_ROOT, "solver", "TESTDATA", "velocity simulation in evaporator and heater.zip")


@pytest.fixture(scope="module")
def so():
    L = C.CDLL(build.build())
    L.mps_read_parameter_file.argtypes = [C.c_char_p, C.POINTER(CParameter)]
    L.mps_read_particle_file.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.c_void_p, C.c_int]
    L.mps_read_stl.argtypes = [C.c_char_p, C.c_int, C.POINTER(Scalar3), C.POINTER(C.c_int), C.c_void_p, C.c_int]
    L.mps_lambda_table.argtypes = [C.c_float]
    L.mps_lambda_table.restype = C.c_float
    L.mps_grid_box.argtypes = [C.POINTER(CBox), C.POINTER(CParameter), C.POINTER(CGridBox)]
    L.mps_lattice_constants.argtypes = [C.c_double, C.c_double, C.c_int, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]
    return L


PARAM_FIELDS = ("3 0 0 -9.81 1000 14.4 0.07 0.01 0.97 2.1 4.0 2.1 293 333 0 0 0.6 16 4186 1000 "
                "0.0001 1000 5 1 50 1 1.5 5000 1e-2 OFF 0.1 0.2 300 290 0.2 0 0 0.005 0 0 0 0.5 0 0 "
                "0 0 OFF OFF OFF 0.3 0.8 OFF 0 0 0 0 0 0 ON 1.0 0 OFF 100000 0.001 0 ON OFF 0 0 0 0 0 0 "
                "ON 350 0.01 0.7 OFF OFF 1e7 3.0 OFF 0 0 0 0 0 0 OFF 5")


def test_parameter_file_positional_fields(so, tmp_path):
    f = tmp_path / "parameter.dat"
    f.write_text(PARAM_FIELDS.replace(" ", "\n"))
    p = CParameter()
    assert so.mps_read_parameter_file(str(f).encode(), C.byref(p)) == 0
    assert p.Dimension == 3 and abs(p.GravityConstant.z + 9.81) < 1e-6
    assert p.Density == 1000 and abs(p.ConstantParticleDensity - 14.4) < 1e-6
    assert abs(p.InitialParticleDistance - 0.01) < 1e-9 and abs(p.FreeSurfaceThreshold - 0.97) < 1e-6
    assert p.Dt == np.float32(1e-4) and p.AnalysisStep == 1000 and p.OutputStep == 50
    assert not p.bUpdateTemperature
    assert abs(p.CourantNumber - 0.2) < 1e-7 and abs(p.OffSet - 0.5) < 1e-7
    assert p.bExplicitOut and abs(p.WallFrictionCoeffieicnt - 1.0) < 1e-7
    assert p.StopWallStep == 100000 and abs(p.Tolerance - 0.001) < 1e-9
    assert p.bCGSolver and not p.bUpdateInnerPressure
    assert p.bExplicitPressure and abs(p.SonicVelocity - 350) < 1e-4 and abs(p.r_coeff - 0.7) < 1e-6
    assert abs(p.PressureMax - 1e7) < 1 and abs(p.RLimitCoefficient - 3.0) < 1e-6
    assert not p.bTurbulance and not p.bNegativePressure and p.ConstantCheckStep == 5
    assert p.MaxNeighborhoodNum == 729
    assert p.LambdaValue == so.mps_lambda_table(p.InitialParticleDistance)


def test_parameter_file_truncated_takes_defaults(so, tmp_path):
    f = tmp_path / "short.dat"
    f.write_text(" ".join(PARAM_FIELDS.split()[:30]))
    p = CParameter()
    assert so.mps_read_parameter_file(str(f).encode(), C.byref(p)) == 0
    assert p.StopWallStep == 2 ** 31 - 1 and p.ConstantCheckStep == -1 and p.PressureMax > 1e38
    f.write_text("3 0 0")
    assert so.mps_read_parameter_file(str(f).encode(), C.byref(p)) == 1     # CCT_FILEERR
    assert so.mps_read_parameter_file(b"/nonexistent/param.dat", C.byref(p)) == 1


def _read_particles(so, path):
    n = C.c_int()
    assert so.mps_read_particle_file(path.encode(), C.byref(n), None, 0) == 0
    buf = (C.c_ubyte * (CParticle_size * max(n.value, 1)))()
    assert so.mps_read_particle_file(path.encode(), C.byref(n), buf, n.value) == 0
    a = np.frombuffer(bytes(buf), dtype=np.dtype([("ID", "<i4"), ("pos", "<f4", 3), ("vel", "<f4", 3),
                                                 ("P", "<f4"), ("n", "<f4"), ("T", "<f4"), ("nu", "<f4"),
                                                 ("solid", "<f4"), ("type", "<i4")]))[:n.value]
    return a


def test_particle_file(so, tmp_path):
    rng = np.random.default_rng(0)
    rows = rng.normal(0, 1, (57, 11))
    types = rng.integers(0, 3, 57)
    f = tmp_path / "particle.dat"
    with open(f, "w") as fh:
        for r, t in zip(rows, types):
            fh.write(" ".join(f"{v:.7g}" for v in r) + f" {t}\n")
    a = _read_particles(so, str(f))
    assert len(a) == 57 and np.array_equal(a["ID"], np.arange(57)) and np.array_equal(a["type"], types)
    np.testing.assert_allclose(a["pos"], rows[:, :3].astype(np.float32), rtol=1e-6)
    np.testing.assert_allclose(a["nu"], rows[:, 9].astype(np.float32), rtol=1e-6)


def _write_stl_ascii(path, tris):
    with open(path, "w") as f:
        f.write("solid test\n")
        for t in tris:
            f.write("facet normal 0 0 0\n outer loop\n")
            for v in t:
                f.write(f"  vertex {v[0]:.9g} {v[1]:.9g} {v[2]:.9g}\n")
            f.write(" endloop\nendfacet\n")
        f.write("endsolid test\n")


def _write_stl_binary(path, tris):
    with open(path, "wb") as f:
        f.write(b"binary stl".ljust(80, b" "))
        f.write(struct.pack("<I", len(tris)))
        for t in tris:
            f.write(struct.pack("<3f", 0, 0, 0))
            for v in t:
                f.write(struct.pack("<3f", *v))
            f.write(b"\0\0")


def _read_stl(so, path, model=0, offset=(0, 0, 0)):
    n = C.c_int()
    off = Scalar3(*offset)
    assert so.mps_read_stl(path.encode(), model, C.byref(off), C.byref(n), None, 0) == 0
    out = (CTriangle * max(n.value, 1))()
    assert so.mps_read_stl(path.encode(), model, C.byref(off), C.byref(n), out, n.value) == 0
    return list(out)[:n.value]


@pytest.mark.parametrize("kind", ["ascii", "binary"])
def test_stl_readers_recompute_normals_with_reference_arithmetic(so, tmp_path, kind):
    import orc
    tris = scenes.cylinder_triangles((0, 0, 0), 0.15, 0.3, 16, 4).astype(np.float32)
    f = str(tmp_path / f"c.{kind}.stl")
    (_write_stl_ascii if kind == "ascii" else _write_stl_binary)(f, tris)
    got = _read_stl(so, f, model=3, offset=(0.5, 0.0, -0.25))
    assert len(got) == len(tris)
    v = np.array([[[t.Vertex[q].x, t.Vertex[q].y, t.Vertex[q].z] for q in range(3)] for t in got], np.float32)
    np.testing.assert_array_equal(v, (tris + np.float32([0.5, 0.0, -0.25])).astype(np.float32))
    nrm = np.array([[t.Normal.x, t.Normal.y, t.Normal.z] for t in got], np.float32)
    assert np.array_equal(nrm, orc.triangle_normals_q(v))
    assert all(t.ModelIDNumber == 3 for t in got)


def test_grid_box_lambda_and_lattice(so):
    p = CParameter()
    p.InitialParticleDistance = 0.01
    p.LaplacianInfluenceRadiusCoefficient = 4.0
    p.GradientInfluenceRadiusCoefficient = 2.1
    z = CBox(Scalar3(0, 0, 0), Scalar3(0.8, 0.2, 0.6))
    b = CGridBox()
    assert so.mps_grid_box(C.byref(z), C.byref(p), C.byref(b)) == 0
    from simulation_project_gb300.types import grid_box
    b2 = grid_box((0, 0, 0), (0.8, 0.2, 0.6), p)
    assert bytes(b) == bytes(b2)
    for l0 in (0.0001, 0.002, 0.0025, 0.004, 0.01, 0.05, 0.7, 20.0):
        assert np.float32(so.mps_lambda_table(l0)) == np.float32(scenes.lambda_table(l0))
    n0, lam = C.c_double(), C.c_double()
    assert so.mps_lattice_constants(2.1, 1.0, 3, C.byref(n0), C.byref(lam)) == 0
    assert abs(n0.value - 14.418575408286717) < 1e-9
    assert so.mps_lattice_constants(4.0, 0.002, 3, C.byref(n0), C.byref(lam)) == 0
    assert abs(n0.value - 123.99156470) < 1e-6 and abs(lam.value / 0.002 ** 2 - 5.211991) < 1e-5


@pytest.mark.skipif(not os.path.exists(TD), reason="reference test deck not available")
def test_reference_test_deck_particles_and_stl(so, tmp_path):
    zf = zipfile.ZipFile(TD)
    for name in zf.namelist():
        if name.endswith("IN/particle.dat") or name.endswith(".stl") and "error" not in name:
            zf.extract(name, tmp_path)
    part = str(next(tmp_path.rglob("particle.dat")))
    a = _read_particles(so, part)
    ref = np.loadtxt(part, ndmin=2)
    assert len(a) == len(ref) > 1000
    np.testing.assert_allclose(a["pos"], ref[:, :3].astype(np.float32), rtol=1e-6)
    for stl in tmp_path.rglob("*.stl"):
        tris = _read_stl(so, str(stl))
        assert len(tris) > 0
