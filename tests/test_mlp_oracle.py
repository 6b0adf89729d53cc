"""The MLP oracle's backward pass against central finite differences (FP64, BF16
rounding switched off)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp_oracle as mo  # noqa: E402


def test_oracle_gradient_matches_finite_differences(monkeypatch):
    monkeypatch.setattr(mo, "bf16", lambda x: np.asarray(x, dtype=np.float64))
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.2, mo.NPARAMS)
    X = rng.normal(0, 1, (7, mo.FIN))
    T = rng.normal(0, 1, (7, mo.FOUT))
    loss, g = mo.loss_grad(p, X, T)
    idx = rng.choice(mo.NPARAMS, 60, replace=False)
    idx = np.concatenate([idx, [0, mo.NPARAMS - 1, mo.NPARAMS - 3]])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mo.loss_grad(pp, X, T)[0] - mo.loss_grad(pm, X, T)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0e-3, 65504.0], np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0            # tie -> even
    assert r[2] == 1.0078125      # above tie -> up
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)


def test_parameter_count_matches_headers_and_binding():
    import re
    from simulation_project_gb300 import learned
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    hdr = open(os.path.join(root, "include", "mps_solver.h")).read()
    n = int(re.search(r"#define MPS_MLP_PARAMS (\d+)", hdr).group(1))
    assert n == mo.NPARAMS == learned.NPARAMS
