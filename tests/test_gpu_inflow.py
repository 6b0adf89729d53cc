"""Particle inflow on the device (mps_solver_add_particles) against the oracle's
restatement of CMultiGPUHandler::InsertBucket (radix/SPVSOLVER/MultiGPUSolver/
MultiGPUHandler.cpp:1163-1210): the holes left by the compute-zone compaction are
filled in increasing ID order, the rest appended only if it all fits."""
import copy
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import bucket_oracle  # noqa: E402

from simulation_project_gb300 import scenes  # noqa: E402
from simulation_project_gb300.solver import Solver  # noqa: E402

pytestmark = pytest.mark.gpu

REMOVED = [3, 50, 51, 400, 777, 1200, 1201, 2500, 3100, 4000]


def _scene():
    sc = copy.deepcopy(scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5))
    sites = sc.pos[REMOVED].copy()
    sc.pos = sc.pos.copy()
    sc.pos[REMOVED] = [10.0, 10.0, 10.0]          # outside the compute zone: removed at step 0
    return sc, sites


@pytest.mark.parametrize("room", [8, 2])
def test_inflow_fills_holes_then_appends(room):
    sc, sites = _scene()
    n0 = sc.n
    s = Solver(sc, precision="fp32_ir", max_particles=n0 + room)
    st = s.step(0)
    assert st["error_flags"] == 0
    before = s.state(sort_by_id=True)
    assert len(before["id"]) == n0 - len(REMOVED)
    far = np.full((4, 3), 10.0)
    bucket = np.concatenate([sites, far]).astype(np.float32)
    want_ids, want_ext = bucket_oracle.insert_bucket(before["id"], n0, n0 + room, len(bucket))
    added = s.add_particles(bucket, visc=np.full(len(bucket), 1e-6))
    assert added == len(want_ids)
    after = s.state(sort_by_id=True)
    assert len(after["id"]) == len(before["id"]) + added
    got = {int(i): p for i, p in zip(after["id"], after["pos"])}
    for j, pid in enumerate(want_ids):
        assert np.array_equal(got[pid], bucket[j].astype(np.float64)), (j, pid)
    assert sorted(got) == sorted(set(before["id"].tolist()) | set(want_ids))
    st = s.step(1)                                 # the outside ones go again; the rest run
    assert st["error_flags"] == 0 and st["cg_relres"] <= 1e-8, st
    assert len(s.state()["id"]) == n0
