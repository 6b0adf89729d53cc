"""Interface struct layouts equal the reference's: sizeof and every field offset of
the ctypes mirror (simulation_project_gb300/types.py, which follows
include/mps_types.h) against offsets recorded from the reference's DataType.h
(tests/golden/layout_reference.txt, made by tests/golden/make_layout.py)."""
import ctypes as C
import os

from simulation_project_gb300 import types as T

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "layout_reference.txt")


def test_layouts_match_reference():
    lines = open(GOLD).read().split()
    rec = dict(zip(lines[0::2], map(int, lines[1::2])))
    checked = 0
    for key, val in rec.items():
        if "." in key:
            s, f = key.split(".")
            cls = getattr(T, s, None)
            if cls is None:
                continue
            assert getattr(cls, f).offset == val, key
        else:
            cls = getattr(T, key, None)
            if cls is None:
                continue
            assert C.sizeof(cls) == val, key
        checked += 1
    assert checked > 140


def test_grid_box_geometry_follows_setcomputezone():
    p = T.CParameter()
    p.InitialParticleDistance = 0.01
    p.LaplacianInfluenceRadiusCoefficient = 4.0
    p.GradientInfluenceRadiusCoefficient = 2.1
    b = T.grid_box((0.0, 0.0, 0.0), (0.8, 0.2, 0.6), p)
    assert abs(b.m_CellSize - 0.04) < 1e-9
    assert (b.m_GridSize.x, b.m_GridSize.y, b.m_GridSize.z) == (24, 9, 19)
    assert abs(b.m_BufferedZone.m_MinBound.x + 0.08) < 1e-7


def test_cparticle_record_size():
    import ctypes as C
    from simulation_project_gb300.types import CParticle, CParticle_size
    from simulation_project_gb300.solver import CPARTICLE_DTYPE
    assert C.sizeof(CParticle) == CParticle_size == 52 == CPARTICLE_DTYPE.itemsize
    assert CParticle.Position.offset == 4 and CParticle.Type.offset == 48
    for name, _ in CParticle._fields_:
        assert CPARTICLE_DTYPE.fields[name][1] == getattr(CParticle, name).offset
