"""Output frames of the solver state (mps_solver_save_frame): particles in ID order in
the reference's format (IO::Save, radix/SPVSOLVER/MultiGPUSolver/IO.cpp:649-756),
written asynchronously; checked against the state and the oracle's bytes."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import frame_oracle  # noqa: E402

from simulation_project_gb300 import frames, scenes  # noqa: E402
from simulation_project_gb300.solver import Solver  # noqa: E402

pytestmark = pytest.mark.gpu


def _expected(sc, st, ascii, time, mp, ma):
    n = len(st["id"])
    ids = st["id"]
    visc = np.asarray(sc.visc, np.float32)[ids]
    ptype = np.asarray(sc.ptype, np.int32)[ids]
    z = np.zeros(n, np.float32)
    return frame_oracle.frame_bytes(ascii, st["pos"].astype(np.float32), st["vel"].astype(np.float32),
                                    st["press"].astype(np.float32), st["pnd"].astype(np.float32), z, visc, z,
                                    ptype, time, mp, ma)


@pytest.mark.parametrize("ascii", [False, True])
def test_frame_of_the_state(tmp_path, ascii):
    sc = scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5)
    s = Solver(sc, precision="fp32_ir")
    for i in range(2):
        s.step(i)
    mp = np.array([[0.0, 0.0, 0.1], [0.05, 0.0, 0.1]], np.float32)
    ma = np.array([1.5, 3.0], np.float32)
    path = tmp_path / "frame.dat"
    s.save_frame(path, ascii, time=1e-4, model_pos=mp, model_angle=ma)
    s.wait_frames()
    st = s.state(sort_by_id=True)
    assert open(path, "rb").read() == _expected(sc, st, ascii, 1e-4, mp, ma)
    rec, t, p, a = frames.read_frame(path, ascii)
    assert len(rec) == len(st["id"]) and np.array_equal(p, mp) and np.array_equal(a, ma)


def test_frames_written_while_stepping(tmp_path):
    sc = scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5)
    s = Solver(sc, precision="fp32_ir")
    s.step(0)
    want = [_expected(sc, s.state(sort_by_id=True), False, 0.0, np.zeros((0, 3)), [])]
    s.save_frame(tmp_path / "f0.dat")
    for k in range(1, 4):
        s.step(k)
        want.append(_expected(sc, s.state(sort_by_id=True), False, k * 1e-4, np.zeros((0, 3)), []))
        s.save_frame(tmp_path / f"f{k}.dat", time=k * 1e-4)
    s.wait_frames()
    for k in range(4):
        assert open(tmp_path / f"f{k}.dat", "rb").read() == want[k], k
