"""The learned PPE initial guess / scaling: BF16 tensor-core GEMM, MLP forward and
backward against the numpy oracle (oracle/mlp_oracle.py, same BF16 rounding points),
training on the GPU, and what the trained network gains inside the solver."""
import os
import sys

import numpy as np
import pytest

from simulation_project_gb300 import lib, scenes
from simulation_project_gb300.lib import DeviceArray
from simulation_project_gb300.learned import Mlp, gemm_bf16, collect_samples, train
from simulation_project_gb300.solver import Solver

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp_oracle as mo  # noqa: E402

pytestmark = pytest.mark.gpu


def to_bf16_bits(a):
    a = np.ascontiguousarray(np.asarray(a, np.float32))
    b = a.view(np.uint32).astype(np.uint64)
    return (((b + 0x7FFF + ((b >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


@pytest.mark.parametrize("variant", [0, 1], ids=["tcgen05", "mma_sync"])
@pytest.mark.parametrize("M,N,K,ta,tb,split", [(64, 64, 32, 0, 0, 1), (100, 128, 48, 0, 0, 1), (128, 16, 1000, 1, 0, 8),
                                               (333, 128, 16, 0, 1, 1), (16, 128, 517, 1, 0, 4),
                                               (1000, 48, 200, 1, 1, 1), (8192, 128, 128, 0, 0, 1)])
def test_gemm_bf16_matches_numpy(M, N, K, ta, tb, split, variant):
    rng = np.random.default_rng(M + N + K)
    A = rng.normal(0, 1, (K, M) if ta else (M, K)).astype(np.float32)
    B = rng.normal(0, 1, (N, K) if tb else (K, N)).astype(np.float32)
    dA, dB = DeviceArray.from_host(to_bf16_bits(A)), DeviceArray.from_host(to_bf16_bits(B))
    C = DeviceArray((M, N), np.float32)
    C.fill_bytes(0)
    gemm_bf16(M, N, K, dA.ptr, M if ta else K, ta, dB.ptr, K if tb else N, tb, C.ptr, N, beta=1.0 if split > 1 else 0.0,
              split=split, variant=variant)
    Am = mo.bf16(A.T if ta else A)
    Bm = mo.bf16(B.T if tb else B)
    ref = Am @ Bm
    got = C.download()
    assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max() + 1e-3 * np.sqrt(K) * 1e-2


@pytest.mark.parametrize("variant", [0, 1], ids=["tcgen05", "mma_sync"])
def test_gemm_bf16_epilogue(variant):
    """Bias, FP32 pre-activation, SiLU, FP32 and BF16 outputs of one GEMM (the forward
    layer of training) against numpy."""
    M, N, K = 300, 128, 128
    rng = np.random.default_rng(7)
    A = rng.normal(0, 1, (M, K)).astype(np.float32)
    B = rng.normal(0, 0.1, (K, N)).astype(np.float32)
    bias = rng.normal(0, 0.5, N).astype(np.float32)
    dA, dB = DeviceArray.from_host(to_bf16_bits(A)), DeviceArray.from_host(to_bf16_bits(B))
    dbias = DeviceArray.from_host(bias)
    C, Z = DeviceArray((M, N), np.float32), DeviceArray((M, N), np.float32)
    Cb = DeviceArray((M, N), np.uint16)
    gemm_bf16(M, N, K, dA.ptr, K, 0, dB.ptr, N, 0, C.ptr, N, Cb=Cb.ptr, ldcb=N, Cz=Z.ptr, bias=dbias.ptr, act=1,
              variant=variant)
    z = mo.bf16(A) @ mo.bf16(B) + bias
    y = z / (1 + np.exp(-z))
    assert np.abs(Z.download() - z).max() <= 1e-3 * np.abs(z).max()
    assert np.abs(C.download() - y).max() <= 1e-3 * np.abs(y).max()
    yb = (Cb.download().astype(np.uint32) << 16).view(np.float32)
    assert np.abs(yb - y).max() <= 1e-2 * np.abs(y).max()


def _net(seed=3):
    m = Mlp(max_batch=4096, seed=seed)
    p = m.params().astype(np.float64)
    return m, p


def test_mlp_forward_matches_oracle():
    m, p = _net()
    X = np.random.default_rng(1).normal(0, 1, (1000, 12)).astype(np.float32)
    dX, dY = DeviceArray.from_host(X), DeviceArray((1000, 2), np.float32)
    m.forward(dX.ptr, dY.ptr, 1000)
    ref = mo.forward(p, X)
    got = dY.download()
    assert np.abs(got - ref).max() <= 2e-2 * np.abs(ref).max() + 1e-4


@pytest.mark.parametrize("rows", [1, 127, 128, 1000, 50021, 200003])
def test_tcgen05_inference_matches_mma_sync_and_oracle(rows):
    """The tcgen05 kernel (four 128-row tiles in flight, ragged last tile; FP16 weights,
    activations and hidden accumulators, biases through columns of ones, FP32 output
    accumulator) against the mma.sync kernel (BF16 / FP32, the rounding points of
    training) and the FP64 oracle: within the oracle tolerance of the forward test and
    within 1e-2 of max |y| of each other (measured on a GB300: 3.5e-3)."""
    m, p = _net(seed=7)
    X = np.random.default_rng(rows).normal(0, 1, (rows, 12)).astype(np.float32)
    dX = DeviceArray.from_host(X)
    dY0, dY1 = DeviceArray((rows, 2), np.float32), DeviceArray((rows, 2), np.float32)
    m.forward(dX.ptr, dY0.ptr, rows, variant=0)
    m.forward(dX.ptr, dY1.ptr, rows, variant=1)
    y0, y1 = dY0.download(), dY1.download()
    ref = mo.forward(p, X)
    scale = np.abs(ref).max()
    assert np.isfinite(y0).all()
    assert np.abs(y0 - ref).max() <= 2e-2 * scale + 1e-4
    assert np.abs(y0 - y1).max() <= 1e-2 * scale + 1e-4
    assert Mlp.tc_timeouts() == 0


@pytest.mark.parametrize("variant", [2, 3, 4, 5])
def test_tcgen05_inference_with_fma_pipe_silu(variant):
    """The tcgen05 kernel with 0, 1, 2 or 3 of every 4 pairs of hidden activations on
    the FMA pipe (polynomial tanh, SiLU error <= 3.6e-3 absolute) and the rest on the
    SFU: within the oracle tolerance of the forward test, within 1e-2 of max |y| of the
    SFU-only kernel, ragged tiles included."""
    rows = 50021
    m, p = _net(seed=7)
    X = np.random.default_rng(rows).normal(0, 1, (rows, 12)).astype(np.float32)
    dX = DeviceArray.from_host(X)
    dY, dS = DeviceArray((rows, 2), np.float32), DeviceArray((rows, 2), np.float32)
    m.forward(dX.ptr, dY.ptr, rows, variant=variant)
    m.forward(dX.ptr, dS.ptr, rows, variant=2)
    y, ys = dY.download(), dS.download()
    ref = mo.forward(p, X)
    scale = np.abs(ref).max()
    assert np.isfinite(y).all()
    assert np.abs(y - ref).max() <= 2e-2 * scale + 1e-4
    assert np.abs(y - ys).max() <= 1e-2 * scale + 1e-4
    assert Mlp.tc_timeouts() == 0


def test_tcgen05_inference_wait_that_runs_out():
    """The stop path of the tcgen05 inference kernel: with its MMA completion waits
    limited to zero polls every 128-row tile stops after issuing its first layer
    (the slot's barrier reduction makes the stop uniform, the issuing thread drains its
    MMAs before TMEM is freed), the timeout flag is set and no output row is written;
    with the default limit restored the next launch is complete and correct."""
    m, _ = _net(seed=9)
    rows = 50021
    X = np.random.default_rng(6).normal(0, 1, (rows, 12)).astype(np.float32)
    dX = DeviceArray.from_host(X)
    want = DeviceArray((rows, 2), np.float32)
    m.forward(dX.ptr, want.ptr, rows, variant=0)
    ref = want.download()
    assert Mlp.tc_timeouts() == 0
    dY = DeviceArray.from_host(np.full((rows, 2), np.nan, np.float32))
    try:
        Mlp.debug_wait_spins(0)
        m.forward(dX.ptr, dY.ptr, rows, variant=0)
        lib.call("mps_device_sync")
        assert Mlp.tc_timeouts() != 0
        assert np.isnan(dY.download()).all()
    finally:
        Mlp.debug_wait_spins(-1)
    assert Mlp.tc_timeouts() == 0
    m.forward(dX.ptr, dY.ptr, rows, variant=0)
    assert np.array_equal(dY.download(), ref)
    assert Mlp.tc_timeouts() == 0


def test_mlp_gradient_matches_oracle():
    m, p = _net(seed=5)
    rng = np.random.default_rng(2)
    X = rng.normal(0, 1, (2048, 12)).astype(np.float32)
    T = rng.normal(0, 1, (2048, 2)).astype(np.float32)
    dX, dT = DeviceArray.from_host(X), DeviceArray.from_host(T)
    g = DeviceArray((mo.NPARAMS,), np.float32)
    loss = m.loss_grad(dX.ptr, dT.ptr, 2048, g.ptr)
    ref_loss, ref_g = mo.loss_grad(p, X, T)
    got = g.download().astype(np.float64)
    assert abs(loss - ref_loss) <= 1e-3 * abs(ref_loss)
    # per-layer relative error of the gradient blocks
    o = 0
    for fi, fo in ((12, 128), (128, 128), (128, 128), (128, 2)):
        for size in (fi * fo, fo):
            a, b = got[o:o + size], ref_g[o:o + size]
            assert np.linalg.norm(a - b) <= 3e-2 * np.linalg.norm(b) + 1e-7, (o, size)
            o += size
    assert o == mo.NPARAMS


def test_training_reduces_loss_on_a_smooth_target():
    rng = np.random.default_rng(4)
    X = rng.normal(0, 1, (40000, 12)).astype(np.float32)
    T = np.stack([np.tanh(X[:, 0] + 0.5 * X[:, 1] * X[:, 2]), 0.3 * X[:, 3] - 0.2 * X[:, 4] ** 2], 1).astype(np.float32)
    p, info = train(X, T, epochs=6, batch=4096, lr=3e-3)
    assert info["val_loss_after"] < 0.2 * info["val_loss_before"], info


def test_learned_solver_converges_and_reports_gain():
    """Trains on the plain solver's own solves of a small bucket, then runs the same
    steps with and without the network: both reach 1e-8, and in every step after the
    first few (the network is trained on steady steps) the learned start leaves a
    smaller initial residual than the extrapolated warm start.  It saves no CG
    iterations on this scene (measured: 102 against 101 over steps 2-7): the residual it
    removes is the local, high-frequency part that the first preconditioned iteration
    removes anyway, so the test bounds the cost at one iteration per step instead of
    claiming a gain.  The line search minimises the A-norm error, so the residual norm
    itself may rise in an early step (step 1 here)."""
    sc = scenes.rotating_bucket(l0=0.008, n_drag=8)
    f, t = collect_samples(sc, steps=6, precision="fp64")
    p, info = train(f, t, epochs=6, batch=4096, lr=2e-3)
    assert info["val_loss_after"] < info["val_loss_before"]
    plain = Solver(sc, precision="fp32_ir")
    learned = Solver(sc, precision="fp32_ir", learned=1, learned_gate=0)
    learned.set_learned(p)
    scaled = Solver(sc, precision="fp32_ir", learned=3, learned_gate=0)
    scaled.set_learned(p)
    it_p, it_l, it_s = 0, 0, 0
    for i in range(8):
        sp = plain.step(i)
        sl = learned.step(i)
        ss = scaled.step(i)
        for s in (sp, sl, ss):
            assert s["cg_relres"] <= 1e-8 and s["error_flags"] == 0, s
        print(f"step {i}: r0 plain {sp['r0_relres']:.4e} learned {sl['r0_relres']:.4e} scaled {ss['r0_relres']:.4e}; "
              f"its {sp['cg_iterations']} {sl['cg_iterations']} {ss['cg_iterations']}")
        if i >= 2:
            it_p += sp["cg_iterations"]
            it_l += sl["cg_iterations"]
            it_s += ss["cg_iterations"]
        if i >= 3:
            assert sl["r0_relres"] < sp["r0_relres"], (i, sl["r0_relres"], sp["r0_relres"])
    print(f"\nCG iterations steps 2-7: plain {it_p}, learned guess {it_l} (saved {it_p - it_l}, "
          f"{100.0 * (it_p - it_l) / max(it_p, 1):.1f}%), guess+scaling {it_s}; training {info}")
    # no iteration gain is claimed; the guess costs at most one iteration per step
    assert it_l <= it_p + 6
    a, b = plain.state(), learned.state()
    assert np.array_equal(a["id"], b["id"])
    pm = np.abs(a["press"]).max()
    # both converged to 1e-8 residual: pressures agree to the solve tolerance
    assert np.abs(a["press"] - b["press"]).max() <= 1e-3 * pm


@pytest.mark.parametrize("precond", [0, 1], ids=["jacobi", "multilevel"])
def test_flexible_cg_matches_pcg_for_a_fixed_preconditioner(precond):
    """Flexible CG (beta = -(z.q)/(p.q), one direction kept) equals PCG in exact
    arithmetic for a fixed SPD preconditioner: same 1e-8 residual, iterations within a
    few per step, pressures within the solve tolerance."""
    sc = scenes.rotating_bucket(l0=0.008, n_drag=8)
    a = Solver(sc, precision="fp32_ir", preconditioner=precond, flexible=-1)
    b = Solver(sc, precision="fp32_ir", preconditioner=precond, flexible=1)
    ia = ib = 0
    for i in range(5):
        sa, sb = a.step(i), b.step(i)
        assert sa["cg_relres"] <= 1e-8 and sb["cg_relres"] <= 1e-8, (sa, sb)
        assert sa["flexible"] == 0 and sb["flexible"] == 1
        ia += sa["cg_iterations"]
        ib += sb["cg_iterations"]
    assert abs(ia - ib) <= max(3, ia // 10), (ia, ib)
    pa, pb = a.state()["press"], b.state()["press"]
    assert np.abs(pa - pb).max() <= 1e-3 * np.abs(pa).max()


def test_learned_scaling_runs_flexible_cg_and_the_gate_skips_a_guess_that_does_not_pay():
    """The learned diagonal scaling makes the inner solve flexible CG by default; the
    gate measures each learned guess (iterations saved against its cost in iterations,
    both from the step's own CUDA events and residuals) and skips the guess in the
    following steps when it cost more than it saved."""
    sc = scenes.rotating_bucket(l0=0.008, n_drag=8)
    f, t = collect_samples(sc, steps=4, precision="fp64")
    p, _ = train(f, t, epochs=4, batch=4096, lr=2e-3)
    s = Solver(sc, precision="fp32_ir", learned=3)
    s.set_learned(p)
    rows = []
    for i in range(12):
        st = s.step(i)
        assert st["cg_relres"] <= 1e-8 and st["error_flags"] == 0, st
        assert st["flexible"] == 1
        rows.append(st)
    print("\nstep applied saved_its cost_its iterations")
    for i, st in enumerate(rows):
        print(i, st["learned_applied"], round(st["learned_saved_its"], 2), round(st["learned_cost_its"], 2),
              st["cg_iterations"])
    # step 0 runs the guess, step 1 measures the span without it (the baseline)
    assert rows[0]["learned_applied"] == 1 and rows[1]["learned_applied"] == 0
    measured = [st for st in rows[2:] if st["learned_applied"]]
    assert measured and all(st["learned_cost_its"] != 0 for st in measured)
    for a, b in zip(rows[2:], rows[3:]):
        if a["learned_applied"] and a["learned_saved_its"] < a["learned_cost_its"]:
            assert b["learned_applied"] == 0   # a guess that did not pay sits out the next step
        if not b["learned_applied"]:
            assert b["learned_saved_its"] == 0 and b["learned_cost_its"] == 0
