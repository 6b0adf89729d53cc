"""The oracle against golden outputs of the reference's own kernel code
(tests/golden/*.npz, made by tests/golden/make_golden.py from the reference CPU
harness).  Bit-exact."""
import ctypes as C
import os

import numpy as np
import pytest

import orc
from golden.make_golden import explicit_step, math_cases, scene_from_arrays, thermal_turbulent_step

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", ["block", "bucket"])
def test_explicit_step_matches_reference_golden(name):
    g = np.load(os.path.join(GOLD, f"ref_explicit_{name}.npz"))
    pred, final = explicit_step(orc.oracle(), scene_from_arrays(g))
    for stage, arrays in (("pred", pred), ("final", final)):
        for k, v in arrays.items():
            ref = g[f"{stage}_{k}"]
            assert v.tobytes() == ref.tobytes(), f"{stage}_{k}"


def test_thermal_turbulent_step_matches_reference_golden():
    """Temperature operator, Smagorinsky viscosity and the turbulent predictor."""
    g = np.load(os.path.join(GOLD, "ref_thermal_turbulent.npz"))
    mine = thermal_turbulent_step(orc.oracle(), scene_from_arrays(g), g["in_temp"])
    for k, v in mine.items():
        assert v.tobytes() == g[f"out_{k}"].tobytes(), k
    assert (g["out_turb_visc"] > 0).any() and (g["out_out_temperature"] != g["in_temp"][0]).any()


def test_math_matches_reference_golden():
    g = np.load(os.path.join(GOLD, "ref_math.npz"))
    mine = math_cases(orc.oracle())
    for k in g.files:
        assert mine[k].tobytes() == g[k].tobytes(), k


def test_lambda_table_known_values():
    """The chained comparison of CalculateLambdaValueLocal (MultiGPUHandler.cpp:762)
    with l0 as float: 0.01f > 0.01 selects the 0.01-0.02 row, 0.002f > 0.002 the
    0.003-0.004 row; results checked by hand from the table rows."""
    o = orc.oracle()
    f = np.float32
    assert o.lambda_table(f(0.01)) == f(f(0.0369119) * f(0.01)) + f(-0.000210081)
    assert o.lambda_table(f(0.002)) == f(f(0.0107452) * f(0.002)) + f(-1.76386E-05)
    # 0.002 < 0.0025 is true and 1 <= 0.003 false, so the 0.003-0.004 row is taken
    assert o.lambda_table(f(0.0025)) == f(f(0.0107452) * f(0.0025)) + f(-1.76386E-05)
    assert o.lambda_table(f(0.7)) == f(f(1.78861) * f(0.7)) + f(-0.48471)
    assert o.lambda_table(f(20.0)) == f(f(1.78861) * f(20.0)) + f(-0.48471)
