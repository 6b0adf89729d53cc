"""The GB300-native semi-implicit step against the FP64 oracle solver.

FP64 mode: neighbour sets (count and id checksum per particle) identical; pressure
within 1e-6 relative (max-norm, relative to max |P|) and positions within 1e-6*l0
after 10 steps.  FP32 operators inside FP64 refinement: PPE residual <= 1e-8 and the
stated FP32 tolerances (pressure 2e-3 relative, positions 1e-4*l0 after 10 steps)."""
import numpy as np
import pytest

import orc
from simulation_project_gb300 import scenes
from simulation_project_gb300.solver import Solver
from simulation_project_gb300.types import MpsError

pytestmark = pytest.mark.gpu


def small_dam(seed=1):
    # reduced dam break: 10 x 10 x 20 column at l0 = 0.01 in the 0.8 x 0.2 x 0.6 tank
    return scenes.dam_break(l0=0.01, column=(0.1, 0.1, 0.2), seed=seed)


def _compare_neighbours(gpu: Solver, o: orc.OracleSim):
    g = gpu.debug_ppe()
    og = np.argsort(g["id"], kind="stable")
    on = o.neighbours()
    assert np.array_equal(g["id"][og], on["id"])
    assert np.array_equal(g["nbr_count"][og], on["nbr_count"])
    assert np.array_equal(g["nbr_idsum"][og], on["nbr_idsum"])


def test_fp64_first_step_neighbour_sets_and_pressure():
    sc = small_dam()
    o = orc.OracleSim(sc)
    g = Solver(sc, precision="fp64")
    rc, ost = o.step(0)
    gst = g.step(0)
    assert rc == 0 and gst["error_flags"] == 0, gst
    _compare_neighbours(g, o)
    a, b = g.state(), o.state()
    assert np.array_equal(a["id"], b["id"])
    pmax = np.abs(b["press"]).max()
    assert pmax > 0
    assert np.abs(a["press"] - b["press"]).max() <= 1e-6 * pmax
    np.testing.assert_allclose(a["pnd"], b["pnd"], rtol=1e-12, atol=1e-12)
    assert np.abs(a["pos"] - b["pos"]).max() <= 1e-6 * sc.param.InitialParticleDistance
    assert gst["cg_relres"] <= 1e-8


def test_fp64_ten_steps_match_oracle():
    sc = small_dam(seed=2)
    o = orc.OracleSim(sc)
    g = Solver(sc, precision="fp64")
    for i in range(10):
        rc, _ = o.step(i)
        st = g.step(i)
        assert rc == 0 and st["error_flags"] == 0
    _compare_neighbours(g, o)
    a, b = g.state(), o.state()
    assert np.array_equal(a["id"], b["id"])
    pmax = np.abs(b["press"]).max()
    assert np.abs(a["press"] - b["press"]).max() <= 1e-6 * pmax
    assert np.abs(a["pos"] - b["pos"]).max() <= 1e-6 * sc.param.InitialParticleDistance


@pytest.mark.parametrize("precond", [0, 1], ids=["jacobi", "multilevel"])
def test_fp32_ir_converges_and_tracks_fp64(precond):
    sc = small_dam(seed=3)
    o = orc.OracleSim(sc)
    g = Solver(sc, precision="fp32_ir", preconditioner=precond)
    for i in range(10):
        rc, _ = o.step(i)
        st = g.step(i)
        assert rc == 0 and st["error_flags"] == 0, st
        assert st["cg_relres"] <= 1e-8
        assert st["ir_passes"] >= 1
    a, b = g.state(), o.state()
    assert np.array_equal(a["id"], b["id"])
    pmax = np.abs(b["press"]).max()
    err_p = np.abs(a["press"] - b["press"]).max() / pmax
    err_x = np.abs(a["pos"] - b["pos"]).max() / sc.param.InitialParticleDistance
    assert err_p <= 2e-3, err_p
    assert err_x <= 1e-4, err_x


def test_bucket_with_walls_and_drag_fp64():
    sc = scenes.rotating_bucket(l0=0.012, n_drag=6, drag_index=0.5)
    o = orc.OracleSim(sc)
    g = Solver(sc, precision="fp64")
    for i in range(3):
        rc, _ = o.step(i)
        st = g.step(i)
        assert rc == 0 and st["error_flags"] == 0, st
    _compare_neighbours(g, o)
    a, b = g.state(), o.state()
    assert np.array_equal(a["id"], b["id"])
    pmax = np.abs(b["press"]).max()
    assert np.abs(a["press"] - b["press"]).max() <= 1e-6 * pmax
    assert np.abs(a["pos"] - b["pos"]).max() <= 1e-6 * sc.param.InitialParticleDistance
    np.testing.assert_allclose(g.triangles().reshape(-1, 9), _tri(o, sc), rtol=0, atol=1e-12)


def _tri(o, sc):
    import ctypes as C
    v = np.zeros((sc.t, 9))
    o.lib.sim_get_triangles(o.h, orc.ptr(v))
    return v


def test_multilevel_cuts_iterations_and_is_deterministic():
    """The cell-aggregate multilevel preconditioner reaches the same 1e-8 FP64 residual
    in far fewer CG iterations than Jacobi, and two runs give identical pressures."""
    sc = scenes.rotating_bucket(l0=0.006, n_drag=4, drag_index=0.5)
    its, press = {}, {}
    for precond in (0, 1, 1):
        g = Solver(sc, precision="fp32_ir", preconditioner=precond)
        n = 0
        for i in range(3):
            st = g.step(i)
            assert st["error_flags"] == 0 and st["cg_relres"] <= 1e-8, st
            n += st["cg_iterations"]
        if precond:
            assert st["mg_levels"] >= 2 and st["mg_level1"] > 100, st
        its.setdefault(precond, n)
        press.setdefault(precond, []).append(g.state()["press"])
    assert its[1] <= 0.75 * its[0], its
    assert np.array_equal(press[1][0], press[1][1])
    # both preconditioners solve the same system to 1e-8
    scale = np.abs(press[0][0]).max()
    assert np.abs(press[1][0] - press[0][0]).max() <= 2e-3 * scale


def test_post_smoother_cuts_iterations_with_flexible_cg():
    """The fine level's post-smoothing through the short-range couplings (fine_smoother
    1) reaches the same 1e-8 residual in fewer inner iterations than the additive Jacobi
    fine level (the default), runs as flexible CG, and is deterministic."""
    sc = scenes.rotating_bucket(l0=0.006, n_drag=4, drag_index=0.5)
    its, press = {}, []
    for fs in (0, 1, 1):
        g = Solver(sc, precision="fp32_ir", preconditioner=1, fine_smoother=fs)
        n = 0
        for i in range(4):
            st = g.step(i)
            assert st["error_flags"] == 0 and st["cg_relres"] <= 1e-8, st
            assert st["flexible"] == fs
            if i >= 1:
                n += st["cg_iterations"]
        its.setdefault(fs, n)
        if fs:
            press.append(g.state()["press"])
        g.close()
    print(f"\ninner iterations steps 1-3: additive {its[0]}, post-smoothing {its[1]}")
    assert its[1] < its[0], its
    assert np.array_equal(press[0], press[1])


def test_double_float_residual_matches_fp64_residual():
    """The refinement residual runs in double-float arithmetic (exact FP32 products,
    TwoSum accumulation); it agrees with the FP64 kernel far below the 1e-8 target."""
    sc = scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5)
    g = Solver(sc, precision="fp32_ir")
    for i in range(2):
        g.step(i)
    r64, rel64 = g.debug_residual(0)
    rdf, reldf = g.debug_residual(1)
    bnorm_inf = np.abs(g.debug_ppe()["rhs"]).max()
    assert bnorm_inf > 0 and rel64 <= 1e-8
    assert np.abs(rdf - r64).max() <= 1e-10 * bnorm_inf, np.abs(rdf - r64).max() / bnorm_inf
    assert abs(reldf - rel64) <= 1e-3 * rel64 + 1e-12


@pytest.mark.parametrize("mf", [4, 8])
def test_matrix_free_spmv_gives_identical_results(mf):
    """Matrix-free inner SpMV: each weight recomputed from the FP32 positions by the
    neighbour pass's own expression, summed in the same order, so the FP32-IR step is
    bit-identical to the stored-weight SpMV."""
    sc = scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5)
    a = Solver(sc, precision="fp32_ir", matrix_free=mf)
    b = Solver(sc, precision="fp32_ir", matrix_free=0, spmv_stream=0)
    for i in range(3):
        sa, sb = a.step(i), b.step(i)
        assert sa["error_flags"] == 0 and sa["cg_relres"] <= 1e-8
        assert sa["cg_iterations"] == sb["cg_iterations"] and sa["cg_relres"] == sb["cg_relres"]
    x, y = a.state(), b.state()
    assert np.array_equal(x["press"], y["press"]) and np.array_equal(x["pos"], y["pos"])


def test_spmv_kernels_give_identical_rows():
    """The register walk, the streamed kernel and both matrix-free unrolls compute
    every row of y = A x in the same order: bit-identical y."""
    sc = scenes.rotating_bucket(l0=0.006, n_drag=4, drag_index=0.5)
    s = Solver(sc, precision="fp32_ir")
    for i in range(2):
        s.step(i)
    n = s.state(sort_by_id=False)["id"].shape[0]
    x = np.random.default_rng(7).standard_normal(n).astype(np.float32)
    y0 = s.debug_spmv(0, x)
    assert np.isfinite(y0).all() and np.count_nonzero(y0) > n // 2
    for k in (1, 3, 4, 8):
        yk = s.debug_spmv(k, x)
        assert np.array_equal(y0.view(np.uint32), yk.view(np.uint32)), (k, np.abs(yk - y0).max())


@pytest.mark.parametrize("wide", [0, 1], ids=["16bit", "wide"])
def test_row_transpose_variants_give_identical_steps(wide):
    """The list pass writes each row contiguously; the asynchronous (swizzled,
    double-buffered) and the register-staged SELL-32 transposes make the same slices,
    so the steps are bit-identical, over 16-bit and over 32-bit columns."""
    sc = scenes.rotating_bucket(l0=0.006, n_drag=4, drag_index=0.5)
    a = Solver(sc, precision="fp32_ir", rows_sell=0, spmv_wide=wide)
    b = Solver(sc, precision="fp32_ir", rows_sell=1, spmv_wide=wide)
    for i in range(3):
        sa, sb = a.step(i), b.step(i)
        assert sa["error_flags"] == 0 and sb["error_flags"] == 0 and sa["cg_relres"] <= 1e-8
        assert sa["cg_iterations"] == sb["cg_iterations"] and sa["cg_relres"] == sb["cg_relres"]
        assert sa["nnz_wide"] == sb["nnz_wide"] and sa["rows16"] == 1
    x, y = a.state(), b.state()
    assert np.array_equal(x["press"], y["press"]) and np.array_equal(x["pos"], y["pos"])


def test_streamed_residual_is_bit_identical():
    """The double-float refinement residual over streamed rows does the register
    walk's operations in the same order: identical r and norms."""
    sc = scenes.rotating_bucket(l0=0.006, n_drag=4, drag_index=0.5)
    s = Solver(sc, precision="fp32_ir")
    for i in range(2):
        s.step(i)
    r1, rel1 = s.debug_residual(1)
    r2, rel2 = s.debug_residual(2)
    r3, rel3 = s.debug_residual(3)
    # rows bit-identical; the norms are grid reductions over different grids
    assert np.array_equal(r1, r2) and abs(rel1 - rel2) <= 1e-12 * rel1
    assert np.array_equal(r1, r3) and abs(rel1 - rel3) <= 1e-12 * rel1
    r0, rel0 = s.debug_residual(0)
    assert np.abs(r1 - r0).max() <= 1e-10 * np.abs(s.debug_ppe()["rhs"]).max()


def test_fp16_inner_operator():
    """FP16 copies of the weights for the inner CG (diagonal recomputed from them):
    the SpMV is within the FP16 rounding of the FP32 one, and the refinement still
    drives the FP32-weight residual to the tolerance."""
    sc = scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5)
    a = Solver(sc, precision="fp32_ir", inner_weights=16)
    b = Solver(sc, precision="fp32_ir", inner_weights=32)
    for i in range(3):
        sa, sb = a.step(i), b.step(i)
        assert sa["error_flags"] == 0 and sa["cg_relres"] <= 1e-8, sa
        assert sa["cg_iterations"] <= 1.5 * sb["cg_iterations"] + 8, (sa["cg_iterations"], sb["cg_iterations"])
    pa, pb = a.state()["press"], b.state()["press"]
    assert np.abs(pa - pb).max() <= 1e-4 * np.abs(pb).max()
    n = a.state(sort_by_id=False)["id"].shape[0]
    x = np.random.default_rng(3).standard_normal(n).astype(np.float32)
    y32, y16 = a.debug_spmv(0, x), a.debug_spmv(2, x)
    assert np.linalg.norm(y16 - y32) <= 1e-3 * np.linalg.norm(y32)
    assert not np.array_equal(y16, y32)
    assert np.array_equal(y16.view(np.uint32), a.debug_spmv(6, x).view(np.uint32))


@pytest.mark.parametrize("inner", [16, 32])
def test_wide_column_streaming_step(inner):
    """Streaming every slice's 32-bit columns (the choice for grids whose x planes
    exceed the 16-bit offsets) converges like the 16-bit slices."""
    sc = scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5)
    a = Solver(sc, precision="fp32_ir", inner_weights=inner, spmv_wide=1)
    b = Solver(sc, precision="fp32_ir", inner_weights=inner, spmv_wide=-1)
    for i in range(3):
        sa, sb = a.step(i), b.step(i)
        assert sa["error_flags"] == 0 and sa["cg_relres"] <= 1e-8, sa
        assert abs(sa["cg_iterations"] - sb["cg_iterations"]) <= 2
    pa, pb = a.state()["press"], b.state()["press"]
    assert np.abs(pa - pb).max() <= 1e-4 * np.abs(pb).max()


def test_streamed_spmv_step_matches():
    """FP32-IR steps with the streamed SpMV: same row values, the CG's p.q sums in
    another order (persistent grid), so the step agrees to the solve tolerance."""
    sc = scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5)
    a = Solver(sc, precision="fp32_ir", spmv_stream=1, inner_weights=32)
    b = Solver(sc, precision="fp32_ir", spmv_stream=0)
    for i in range(3):
        sa, sb = a.step(i), b.step(i)
        assert sa["error_flags"] == 0 and sa["cg_relres"] <= 1e-8, sa
        assert abs(sa["cg_iterations"] - sb["cg_iterations"]) <= 2
    pa, pb = a.state()["press"], b.state()["press"]
    assert np.abs(pa - pb).max() <= 1e-6 * np.abs(pb).max()


def test_spmv_options_are_checked():
    sc = scenes.rotating_bucket(l0=0.008, n_drag=0)
    for bad in ({"matrix_free": 3}, {"spmv_stream": 2}, {"inner_weights": 8}, {"spmv_wide": 2},
                {"warm_start": 3}, {"warm_start": -2}):
        with pytest.raises(MpsError) as e:
            Solver(sc, precision="fp32_ir", **bad)
        assert e.value.status == 2   # CCT_PARAMERR


def test_compressed_rows_give_identical_results():
    """16-bit column offsets (the default) and 32-bit columns: same columns in the same
    order, so the FP32-IR step is bit-identical."""
    sc = scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5)
    a = Solver(sc, precision="fp32_ir", compress_rows=1, spmv_stream=0)
    b = Solver(sc, precision="fp32_ir", compress_rows=0, spmv_stream=0)
    for i in range(3):
        sa, sb = a.step(i), b.step(i)
        assert sa["cg_iterations"] == sb["cg_iterations"] and sa["cg_relres"] == sb["cg_relres"]
    x, y = a.state(), b.state()
    assert np.array_equal(x["press"], y["press"]) and np.array_equal(x["pos"], y["pos"])


def test_warm_start_history_follows_particles():
    """The increments held for the warm start are, per particle, exactly the FP32 values of
    P_n - P_{n-1} (interior rows of the last solve, else 0) and the previous increment,
    through the sort and compaction of every step; the order used grows 0, 1, 2."""
    sc = scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5)
    g = Solver(sc, precision="fp32_ir")
    prev_p, prev_d1 = None, None
    for i in range(5):
        st = g.step(i)
        assert st["error_flags"] == 0 and st["cg_relres"] <= 1e-8, st
        assert st["warm_start"] == min(i, 2)
        p = g.state()["press"]                      # by id
        h = g.debug_history()
        o = np.argsort(h["id"], kind="stable")
        d1, d2, inner = h["dph1"][o], h["dph2"][o], h["inner"][o]
        assert h["held"] == min(i + 1, 2)
        if prev_p is not None:
            want = np.where(inner, (p - prev_p).astype(np.float32), np.float32(0))
            assert d1.tobytes() == want.tobytes()
            assert d2.tobytes() == prev_d1.tobytes()
            assert np.abs(d1).max() > 0
        prev_p, prev_d1 = p, d1


@pytest.mark.parametrize("order", [1, 2])
def test_warm_start_extrapolation_converges_to_the_same_pressure(order):
    """Any warm start reaches cg_rtol; after 6 steps the pressures agree with those of
    the previous-pressure start to 1e-4 of max |P| (two solutions within a relative
    residual of 1e-8 differ by up to the condition number times it)."""
    sc = scenes.rotating_bucket(l0=0.008, n_drag=4, drag_index=0.5)
    a = Solver(sc, precision="fp32_ir", warm_start=order)
    b = Solver(sc, precision="fp32_ir", warm_start=0)
    for i in range(6):
        sa, sb = a.step(i), b.step(i)
        assert sa["error_flags"] == 0 and sa["cg_relres"] <= 1e-8, sa
        assert sb["warm_start"] == 0 and sa["warm_start"] == min(i, order)
    pa, pb = a.state()["press"], b.state()["press"]
    assert np.abs(pa - pb).max() <= 1e-4 * np.abs(pb).max()


@pytest.mark.parametrize("precision", ["fp32_ir", "fp64"])
def test_neighbour_row_overflow_is_flagged_and_capped(precision):
    """A Laplacian row longer than its capacity (max_neighbours = 128 against about 250
    neighbours at re = 4 l0) sets MPS_ERR_NEIGHBOUR_CAP, keeps the row at the capacity
    and reports the uncapped length as max_row: no row is cut silently and no store
    leaves the row.  Counts are those of a full-capacity solver of the same scene,
    capped."""
    sc = scenes.rotating_bucket(l0=0.012, n_drag=0)
    full = Solver(sc, precision=precision)
    capped = Solver(sc, precision=precision, max_neighbours=128)
    sf, sc_ = full.step(0), capped.step(0)
    assert sf["error_flags"] == 0 and sf["max_row"] > 128, sf
    assert sc_["error_flags"] & 2, sc_
    assert sc_["max_row"] == sf["max_row"]
    a, b = full.debug_ppe(), capped.debug_ppe()
    oa, ob = np.argsort(a["id"], kind="stable"), np.argsort(b["id"], kind="stable")
    assert np.array_equal(a["id"][oa], b["id"][ob])
    assert np.array_equal(np.minimum(a["nbr_count"][oa], 128), b["nbr_count"][ob])
    assert b["nbr_count"].max() == 128
    # the solver stays usable: a second step runs and flags the overflow again
    assert capped.step(1)["error_flags"] & 2


def test_streamed_level1_assembly_is_bit_identical():
    """The multilevel preconditioner's level-1 Galerkin stencil assembled over rows
    streamed through shared memory (the default) equals the register walk's bit for bit:
    each row's slot sums add its entries in row order either way."""
    sc = scenes.rotating_bucket(l0=0.006, n_drag=4, drag_index=0.5)
    g = Solver(sc, precision="fp32_ir")
    for i in range(2):
        st = g.step(i)
        assert st["error_flags"] == 0 and st["mg_levels"] >= 2, st
    a1 = g.debug_level1(1)
    a0 = g.debug_level1(0)
    assert a1.shape == (st["mg_level1"], 27)
    assert a0.tobytes() == a1.tobytes()
    assert (a0[:, 13] > 0).sum() > a0.shape[0] // 2   # interior aggregates: positive diagonal
    assert (a0[:, np.arange(27) != 13] <= 0).all()    # off-diagonal couplings: -coef w sums
    # the stencil the step used (streamed) is reproduced
    g.step(2)
    a2 = g.debug_level1(1)
    assert a2.tobytes() == g.debug_level1(0).tobytes()


def _emptied(sc, shift=None):
    import copy
    e = copy.copy(sc)
    if shift is None:   # no particles at all
        for k in ("pos", "vel"):
            setattr(e, k, getattr(sc, k)[:0])
        for k in ("press", "visc", "ptype"):
            setattr(e, k, getattr(sc, k)[:0])
    else:               # every particle outside the compute zone
        e.pos = sc.pos + np.asarray(shift)
    return e


@pytest.mark.parametrize("precision", ["fp32_ir", "fp64"])
@pytest.mark.parametrize("case", ["no_particles", "all_outside_the_zone"])
def test_steps_without_particles(precision, case):
    """A scene without particles, and one whose particles all lie outside the compute
    zone (the first compaction removes them), step without error: no particles, no CG
    work, error flags clear, and the walls still rotate as in a step with particles."""
    sc = scenes.rotating_bucket(l0=0.012, n_drag=0)
    e = _emptied(sc, None if case == "no_particles" else (10.0, 10.0, 10.0))
    g = Solver(e, precision=precision, max_particles=max(sc.n, 1))
    ref = Solver(sc, precision=precision)
    for i in range(3):
        st = g.step(i)
        ref.step(i)
        assert st["error_flags"] == 0 and st["particles"] == 0, st
        assert st["cg_iterations"] == 0 and st["nnz"] == 0, st
    assert g.state()["id"].shape == (0,)
    # the wall motion does not depend on the particles
    assert np.array_equal(g.triangles(), ref.triangles())
    assert not np.array_equal(g.triangles(), sc.tri_vertices.reshape(-1, 3, 3))


def test_refinement_residual_update_tracks_the_true_residual():
    """Between refinement passes the residual follows from the pass's correction (x += s d,
    r -= s A d with A d in double-float).  After every step the true residual b - A x,
    recomputed in FP64 from the final pressure, meets the 1e-8 target and agrees with the
    residual the solver stopped on to 1e-11 of ||b||."""
    sc = scenes.rotating_bucket(l0=0.006, n_drag=4, drag_index=0.5)
    s = Solver(sc, precision="fp32_ir")
    passes = 0
    for i in range(5):
        st = s.step(i)
        assert st["error_flags"] == 0 and st["cg_relres"] <= 1e-8, st
        _, rel_true = s.debug_residual(0)
        assert rel_true <= 1e-8, (i, rel_true)
        assert abs(rel_true - st["cg_relres"]) <= 1e-11, (i, rel_true, st["cg_relres"])
        passes = max(passes, st["ir_passes"])
    assert passes >= 2   # at least one residual came from an update
