"""CalcPoisson (the reserved prototype of the older tree's DeviceProcess.h:50-53) as a
context-handle variant: its ID-indexed outputs equal CalculatePressureCG's solve of the
same state (diagonal, right-hand side and pressure), a start given in dX0 reaches the
same pressure, and an ID beyond ParticleNum is refused."""
import numpy as np
import pytest

from simulation_project_gb300 import scenes
from simulation_project_gb300.lib import DeviceArray
from simulation_project_gb300.solver import Solver
from simulation_project_gb300.types import MpsError

pytestmark = pytest.mark.gpu


def _scene():
    return scenes.dam_break(l0=0.01, column=(0.1, 0.1, 0.2), seed=5)


@pytest.mark.parametrize("precision", ["fp64", "fp32_ir"])
def test_calc_poisson_matches_calculate_pressure_cg(precision):
    sc = _scene()
    a, b = Solver(sc, precision=precision), Solver(sc, precision=precision)
    for i in range(2):   # a flow state with a pressure history
        a.step(i)
        b.step(i)
    st_a = a.pressure(njp=False)
    ppe = a.debug_ppe()
    sa = a.state()
    n = sc.n
    dA, dB, dX = (DeviceArray((n,), np.float32) for _ in range(3))
    st_b = b.calc_poisson(n, dA.ptr, dB.ptr, dX.ptr)
    assert st_b["cg_relres"] <= 1e-8 and st_a["cg_iterations"] == st_b["cg_iterations"]
    x, diag, rhs = dX.download(), dA.download(), dB.download()
    assert np.array_equal(x[sa["id"]], sa["press"].astype(np.float32))
    o = np.argsort(ppe["id"])
    h = a.debug_history()
    inner = np.zeros(n, bool)
    inner[h["id"]] = h["inner"]
    assert inner.sum() > n // 2
    assert np.array_equal(diag[inner], ppe["diag"][o][inner].astype(np.float32))
    assert np.array_equal(rhs[inner], ppe["rhs"][o][inner].astype(np.float32))
    assert not diag[~inner].any() and not rhs[~inner].any()
    # a start from zero reaches the same pressure
    x0 = DeviceArray.from_host(np.zeros(n, np.float32))
    st_c = b.calc_poisson(n, None, None, dX.ptr, x0.ptr)
    assert st_c["cg_relres"] <= 1e-8 and st_c["r0_relres"] > 0.5
    scale = np.abs(sa["press"]).max()
    assert np.abs(dX.download()[sa["id"]] - sa["press"]).max() <= 2e-3 * scale
    a.close()
    b.close()


def test_calc_poisson_rejects_ids_beyond_particle_num():
    sc = _scene()
    s = Solver(sc, precision="fp64")
    s.step(0)
    dX = DeviceArray((sc.n,), np.float32)
    with pytest.raises(MpsError):
        s.calc_poisson(sc.n // 2, None, None, dX.ptr)
    s.close()
