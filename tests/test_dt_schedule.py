"""dt schedule (DtFrame::Load, DtFrame.cpp:11-35; CheckAndUpdateDt,
MultiGPUHandler.cpp:1256-1275) against the oracle's restatement."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import dt_oracle  # noqa: E402

from simulation_project_gb300 import schedule  # noqa: E402
from simulation_project_gb300.types import CParameter  # noqa: E402

CASES = {
    "trailing_newline": "0 5e-5 0.2 10 100\n2000 1e-4 0.25 20 200\n5000 2.5e-5 0.1 5 50\n",
    "no_trailing_whitespace": "0 5e-5 0.2 10 100\n2000 1e-4 0.25 20 200",
    "short_last_row": "0 5e-5 0.2 10 100\n2000 1e-4 0.25\n",
    "bad_token": "0 5e-5 0.2 10 100\nabc 1e-4 0.25 20 200\n3000 1 1 1 1\n",
    "spaces_and_tabs": "  10\t1.5e-4  0.3 7.9 99.5 \n\n",
    "empty": "",
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_dt_file_matches_the_oracle(tmp_path, name):
    path = tmp_path / "dt.txt"
    path.write_text(CASES[name])
    got = schedule.read_dt_file(path)
    want = dt_oracle.read_dt(CASES[name])
    assert len(got) == len(want), (got, want)
    for g, w in zip(got, want):
        assert int(g["step"]) == w[0]
        assert [float(g[k]) for k in ("dt", "courant", "inflow_step", "output_step")] == list(w[1:])


def test_schedule_applies_one_due_row_per_call(tmp_path):
    path = tmp_path / "dt.txt"
    path.write_text(CASES["trailing_newline"])
    rows = schedule.read_dt_file(path)
    want_rows = dt_oracle.read_dt(CASES["trailing_newline"])
    p = CParameter()
    mine, theirs = 0, 0
    ref = {}
    for step in [0, 1, 1999, 2000, 2001, 6000, 6001, 6002]:
        mine, a = schedule.schedule_next(rows, mine, step, p)
        theirs, b = dt_oracle.schedule_next(want_rows, theirs, step, ref)
        assert (mine, a) == (theirs, b)
        if ref:
            assert np.float32(p.Dt) == np.float32(ref["Dt"]) and p.OutputStep == ref["OutputStep"]
            assert p.ParticleGenerationStep == ref["ParticleGenerationStep"]
            assert np.float32(p.CourantNumber) == np.float32(ref["CourantNumber"])
    assert mine == 3


def test_dt_file_errors(tmp_path):
    with pytest.raises(Exception):
        schedule.read_dt_file(tmp_path / "missing.txt")
