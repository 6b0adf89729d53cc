"""The solver's wall bins on the GPU (k_bin_count, k_bin_fill, the radix sort of the
entries and k_bin_bounds) against a host model of the same rule: a cell's list holds,
in increasing id order, every triangle whose cell box (vertex bounds converted toward
zero, clamped to the grid) grown by one cell holds the cell; walls and drag bodies in
separate lists.  Triangles lie partly and wholly outside the grid, and one spans the
whole grid."""
import itertools

import numpy as np
import pytest

from simulation_project_gb300 import scenes
from simulation_project_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def _model_lists(sc):
    B = sc.box.m_BufferedZone
    lo0 = np.array([B.m_MinBound.x, B.m_MinBound.y, B.m_MinBound.z], np.float64)
    cs = np.float64(sc.box.m_CellSize)
    G = np.array([sc.box.m_GridSize.x, sc.box.m_GridSize.y, sc.box.m_GridSize.z])
    drag = {i for i, tp in enumerate(sc.tri_params) if tp.isDrag}
    lists = {}
    for t, v in enumerate(sc.tri_vertices):
        a = np.trunc((v.min(0) - lo0) / cs)
        b = np.trunc((v.max(0) - lo0) / cs)
        i0 = np.maximum(a, 0).astype(np.int64)
        i1 = np.minimum(b, G - 1).astype(np.int64)
        if (i0 > i1).any():
            continue
        i0 = np.maximum(i0 - 1, 0)
        i1 = np.minimum(i1 + 1, G - 1)
        kind = 1 if sc.tri_model[t] in drag else 0
        for c in itertools.product(*(range(p, q + 1) for p, q in zip(i0, i1))):
            key = (int(c[0] * G[1] * G[2] + c[1] * G[2] + c[2]), kind)
            lists.setdefault(key, []).append(t)
    return lists


def test_wall_bins_match_host_model():
    sc = scenes.random_block(8, seed=3)
    G = np.array([sc.box.m_GridSize.x, sc.box.m_GridSize.y, sc.box.m_GridSize.z])
    B = sc.box.m_BufferedZone
    lo = np.array([B.m_MinBound.x, B.m_MinBound.y, B.m_MinBound.z])
    ext = G * sc.box.m_CellSize
    rng = np.random.default_rng(11)
    tris = []
    for _ in range(400):   # small, medium and large triangles, some outside the grid
        c = lo + rng.uniform(-0.3, 1.3, 3) * ext
        tris.append(c + rng.normal(0, rng.choice([0.2, 1.0, 3.0]) * sc.box.m_CellSize, (3, 3)))
    # one triangle whose box covers the whole grid and more
    tris.append(np.array([lo - ext, [lo[0] + 3 * ext[0], lo[1] - ext[1], lo[2] + 3 * ext[2]], lo + 3 * ext]))
    tris = np.asarray(tris)
    models = (rng.uniform(size=len(tris)) < 0.3).astype(np.int32)
    sc.tri_vertices = tris
    sc.tri_model = models
    sc.tri_params = [scenes._tri_normal_params(dt=sc.param.Dt),
                     scenes._tri_normal_params(dt=sc.param.Dt, is_drag=True)]
    s = Solver(sc, precision="fp64")
    got = s.debug_wall_bins()
    want = _model_lists(sc)
    s.close()
    assert set(got) == set(want)
    for k in want:
        assert got[k] == want[k], k
    # the whole-grid triangle is in every cell's list of its kind
    kind = int(models[-1])
    assert sum(1 for (c, k), v in got.items() if k == kind and len(tris) - 1 in v) == int(np.prod(G))
