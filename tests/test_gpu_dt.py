"""A time step set between steps (a dt schedule row, CheckAndUpdateDt in
radix/SPVSOLVER/MultiGPUSolver/MultiGPUHandler.cpp:1256-1275) leaves the solver exactly
as one created with that time step."""
import copy

import numpy as np
import pytest

from simulation_project_gb300 import scenes
from simulation_project_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp32_ir", "fp64"])
def test_time_step_switch_matches_a_solver_created_with_it(precision):
    a_sc = scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5, dt=5e-5)
    b_sc = copy.deepcopy(a_sc)   # the same walls (their per-step rotation is a model parameter)
    b_sc.param.Dt = 2.5e-5
    a = Solver(a_sc, precision=precision)
    a.set_time_step(2.5e-5, courant=float(b_sc.param.CourantNumber))
    b = Solver(b_sc, precision=precision)
    for i in range(3):
        sa, sb = a.step(i), b.step(i)
        assert sa["error_flags"] == 0 and sa["cg_iterations"] == sb["cg_iterations"]
    x, y = a.state(), b.state()
    for k in ("pos", "vel", "press"):
        assert np.array_equal(x[k], y[k]), k
    with pytest.raises(Exception):
        a.set_time_step(0.0)
