"""Output frames (IO::Save, radix/SPVSOLVER/MultiGPUSolver/IO.cpp:649-756): the
library's writer against the oracle's restatement, byte for byte, in both formats."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import frame_oracle  # noqa: E402

from simulation_project_gb300 import frames  # noqa: E402
from simulation_project_gb300.types import MpsError  # noqa: E402


def _arrays(n, seed=5):
    rng = np.random.default_rng(seed)
    mag = 10.0 ** rng.uniform(-7, 6, size=(n, 11))
    v = (mag * rng.choice([-1, 1], size=(n, 11))).astype(np.float32)
    v[::17, 3] = 0.0
    v[::19, 4] = -0.0
    v[:, 7] = np.abs(v[:, 7])
    types = rng.integers(0, 3, n).astype(np.int32)
    mp = rng.uniform(-1, 1, (3, 3)).astype(np.float32)
    ma = rng.uniform(0, 360, 3).astype(np.float32)
    return v, types, mp, ma


@pytest.mark.parametrize("ascii", [True, False])
def test_frame_bytes_match_the_oracle(tmp_path, ascii):
    n = 257
    v, types, mp, ma = _arrays(n)
    path = tmp_path / "frame.dat"
    frames.write_frame(path, ascii, v[:, 0:3], v[:, 3:6], v[:, 6], v[:, 7], v[:, 9], types, time=0.0125,
                       model_pos=mp, model_angle=ma, temperature=v[:, 8], solid=v[:, 10])
    want = frame_oracle.frame_bytes(ascii, v[:, 0:3], v[:, 3:6], v[:, 6], v[:, 7], v[:, 8], v[:, 9], v[:, 10],
                                    types, 0.0125, mp, ma)
    assert open(path, "rb").read() == want


@pytest.mark.parametrize("ascii", [True, False])
def test_empty_frame_and_missing_optional_arrays(tmp_path, ascii):
    path = tmp_path / "empty.dat"
    frames.write_frame(path, ascii, np.zeros((0, 3)), np.zeros((0, 3)), [], [], [], np.zeros(0, np.int32), time=1.5)
    want = frame_oracle.frame_bytes(ascii, np.zeros((0, 3)), np.zeros((0, 3)), [], [], [], [], [], [], 1.5,
                                    np.zeros((0, 3)), [])
    assert open(path, "rb").read() == want
    n = 9
    v, types, _, _ = _arrays(n, seed=6)
    frames.write_frame(path, ascii, v[:, 0:3], v[:, 3:6], v[:, 6], v[:, 7], v[:, 9], types)
    z = np.zeros(n, np.float32)
    want = frame_oracle.frame_bytes(ascii, v[:, 0:3], v[:, 3:6], v[:, 6], v[:, 7], z, v[:, 9], z, types, 0.0,
                                    np.zeros((0, 3)), [])
    assert open(path, "rb").read() == want


def test_frames_read_back(tmp_path):
    n = 100
    v, types, mp, ma = _arrays(n, seed=7)
    for ascii in (False, True):
        path = tmp_path / f"f{int(ascii)}.dat"
        frames.write_frame(path, ascii, v[:, 0:3], v[:, 3:6], v[:, 6], v[:, 7], v[:, 9], types, time=2.0,
                           model_pos=mp, model_angle=ma, temperature=v[:, 8], solid=v[:, 10])
        rec, t, p, a = frames.read_frame(path, ascii)
        rtol = 5e-6 if ascii else 0.0   # %g keeps six significant digits
        np.testing.assert_allclose(rec["pos"], v[:, 0:3], rtol=rtol)
        np.testing.assert_allclose(rec["pressure"], v[:, 6], rtol=rtol)
        np.testing.assert_allclose(rec["solid"], v[:, 10], rtol=rtol)
        assert np.array_equal(rec["type"], types) and t == 2.0
        np.testing.assert_allclose(p, mp, rtol=rtol)
        np.testing.assert_allclose(a, ma, rtol=rtol)


def test_frame_errors(tmp_path):
    with pytest.raises(MpsError) as e:
        frames.write_frame(tmp_path / "no_such_dir" / "f.dat", False, np.zeros((1, 3)), np.zeros((1, 3)), [0.0],
                           [0.0], [0.0], np.zeros(1, np.int32))
    assert e.value.status == 1   # CCT_FILEERR


def test_g_formatting_edge_values(tmp_path):
    """%g switches to exponent form below 1e-4 and at 1e6 after rounding to six
    digits; denormals, the float range limits and signed zeros."""
    vals = np.array([0.0, -0.0, 1e-4, 9.99999e-5, 9.999995e-5, 1e-5, 123456.0, 999999.0, 999999.5, 1e6, 1234567.0,
                     0.1, 1.0 / 3.0, 2.0 / 3.0, 1e-45, 1.17549435e-38, 3.4028235e38, -3.4028235e38, 5e-324 * 0 + 1e-40,
                     0.000123456789, 100000.05, 99999.95, 7.0, 70.0, 700.0], np.float32)
    n = len(vals)
    col = np.resize(vals, n)
    pos = np.stack([col, col[::-1], np.roll(col, 3)], 1)
    types = np.arange(n, dtype=np.int32) % 3
    path = tmp_path / "edge.dat"
    frames.write_frame(path, True, pos, pos, col, np.abs(col), col[::-1], types, time=999999.5,
                       model_pos=pos[:2], model_angle=col[:2], temperature=col, solid=col[::-1])
    want = frame_oracle.frame_bytes(True, pos, pos, col, np.abs(col), col, col[::-1], col[::-1], types, 999999.5,
                                    pos[:2], col[:2])
    assert open(path, "rb").read() == want
