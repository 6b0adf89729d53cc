"""Entry points under the reference's reserved names (CalculatePressureCG /
CalculatePressureNJPCG, CGPUCellSet.h:224-225), mps_set_precision and the C++
training / inference entry points of the learned part, through the C-ABI."""
import numpy as np
import pytest

from simulation_project_gb300 import scenes
from simulation_project_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def _bucket():
    return scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5)


def test_pressure_solves_keep_positions_and_agree():
    sc = _bucket()
    a = Solver(sc, precision="fp32_ir")
    b = Solver(sc, precision="fp32_ir")
    for i in range(2):
        a.step(i)
        b.step(i)
    before = a.state()
    sa = a.pressure(njp=False)
    sb = b.pressure(njp=True)
    for st in (sa, sb):
        assert st["error_flags"] == 0 and st["cg_relres"] <= 1e-8, st
    assert sa["mg_levels"] == 0 and sb["mg_levels"] >= 2
    after = a.state()
    assert np.array_equal(before["id"], after["id"])
    assert np.array_equal(before["pos"], after["pos"]) and np.array_equal(before["vel"], after["vel"])
    pa, pb = a.state()["press"], b.state()["press"]
    assert np.abs(pa - pb).max() <= 1e-5 * np.abs(pa).max()


def test_set_precision_switches_solver():
    sc = _bucket()
    s = Solver(sc, precision="fp32_ir")
    st = s.step(0)
    assert st["ir_passes"] >= 1 and st["cg_relres"] <= 1e-8
    s.set_precision("fp64")
    st = s.step(1)
    assert st["ir_passes"] == 0 and st["mg_levels"] == 0 and st["cg_relres"] <= 1e-8
    s.set_precision("fp32_ir")
    st = s.step(2)
    assert st["ir_passes"] >= 1 and st["cg_relres"] <= 1e-8 and st["error_flags"] == 0


def test_learned_train_and_infer_through_the_c_abi():
    sc = _bucket()
    s = Solver(sc, precision="fp32_ir")
    info = s.learned_train(0, steps=4, max_samples=100_000, epochs=4, batch=2048, lr=2e-3)
    assert info["samples"] > 10_000 and info["adam_steps"] > 0
    assert info["val_loss_after"] < info["val_loss_before"], info
    its = 0
    for i in range(4, 7):
        st = s.step(i)
        assert st["cg_relres"] <= 1e-8 and st["error_flags"] == 0 and st["fallback"] == 0, st
        its += st["cg_iterations"]
    y = s.learned_infer()
    assert y.shape == (sc.n, 2) or y.shape[1] == 2
    assert np.isfinite(y).all()
