"""Generates tests/golden/*.npz from the reference solver's own kernel code.

    python tests/golden/make_golden.py

Runs the reference CPU harness (oracle/_ref/libref.so: the reference's
DeviceProcess_Kernel.h compiled for the CPU, see oracle/build_ref.py) on small seeded
scenes and stores its inputs-derived outputs.  tests/test_golden.py checks the oracle
against these files, so the oracle stays pinned on machines without the reference
checkout.  Requires the reference checkout; the outputs are deterministic.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import orc  # noqa: E402
from simulation_project_gb300 import scenes  # noqa: E402
from simulation_project_gb300.types import Scalar3, CTriangle  # noqa: E402

OUT_FIELDS = ["hash", "index", "cell_start", "cell_end", "id", "pos", "vel", "out_id", "out_pos", "out_vel",
              "out_pressure", "out_density", "out_solid_rate", "out_type", "stl_distance", "stl_id", "cells",
              "drag_acc"]


def explicit_step(lib, scene):
    st = orc.RefState(scene)
    b = st.bindings()
    orc.ref_topology(lib, st, b)
    lib.reset_triangle_topology(st.cells_n, orc.ptr(st.cells))
    lib.register_triangle_topology(C.byref(b), orc.ptr(st.triangles), st.t, orc.ptr(st.cells), st.cells_n)
    lib.calc_stl_distance(C.byref(b), st.n)
    if st.drag_num:
        lib.calc_drag_effect(C.byref(b), st.n)
    lib.calc_explicitly(C.byref(b), st.n)
    after_predictor = {f: getattr(st, f).copy() for f in OUT_FIELDS}
    orc.ref_topology(lib, st, b)
    lib.calc_stl_distance(C.byref(b), st.n)
    lib.calc_explicit_pressure(C.byref(b), st.n)
    lib.calc_explicit_pressure_gradient(C.byref(b), st.n)
    final = {f: getattr(st, f).copy() for f in OUT_FIELDS}
    return after_predictor, final


HEAT_FIELDS = OUT_FIELDS + ["temperature", "out_temperature", "out_kin_visc", "turb_visc", "strain"]


def thermal_turbulent_step(lib, scene, temps):
    """Wall distance, the temperature operator, the Smagorinsky viscosity and the
    turbulent predictor (CalcTemperatureFactor, CalcTurbulenceViscosity, CalcExplicitly)
    from the initial temperatures `temps` (original order)."""
    st = orc.RefState(scene)
    st.out_temperature[:st.n] = temps
    b = st.bindings()
    orc.ref_topology(lib, st, b)
    lib.reset_triangle_topology(st.cells_n, orc.ptr(st.cells))
    lib.register_triangle_topology(C.byref(b), orc.ptr(st.triangles), st.t, orc.ptr(st.cells), st.cells_n)
    lib.calc_stl_distance(C.byref(b), st.n)
    lib.calc_temperature_factor(C.byref(b), st.n)
    lib.calc_turbulence_viscosity(C.byref(b), st.n)
    lib.calc_explicitly(C.byref(b), st.n)
    return {f: getattr(st, f).copy() for f in HEAT_FIELDS}


def thermal_turbulent_scene():
    sc = scenes.random_block(9, seed=5)
    hook = orc.thermal_scene(sc, 5)
    orc.turbulent_scene(sc, 5)
    probe = orc.RefState(sc)
    hook(probe)
    return sc, probe.out_temperature[:probe.n].copy()


def golden_scenes():
    s1 = scenes.random_block(8, seed=11)
    s2 = scenes.rotating_bucket(l0=0.025, n_drag=4, drag_index=5.0)
    s2.vel = np.random.default_rng(12).normal(0, 0.2, s2.pos.shape)
    return {"block": s1, "bucket": s2}


def scene_to_arrays(sc):
    """The scene inputs as plain arrays (stored with the golden outputs, so the
    fixture does not depend on the scene generator)."""
    import ctypes as C
    from simulation_project_gb300.types import CTriangleParameters, DragParameter
    tp = (CTriangleParameters * len(sc.tri_params))(*sc.tri_params)
    dp = (DragParameter * max(len(sc.drag), 1))(*sc.drag)
    return {"in_pos": sc.pos, "in_vel": sc.vel, "in_press": sc.press, "in_visc": sc.visc, "in_type": sc.ptype,
            "in_tri": sc.tri_vertices, "in_tri_model": sc.tri_model,
            "in_param": np.frombuffer(bytes(sc.param), np.uint8), "in_box": np.frombuffer(bytes(sc.box), np.uint8),
            "in_tparams": np.frombuffer(bytes(tp), np.uint8), "in_drag": np.frombuffer(bytes(dp), np.uint8),
            "in_ndrag": np.array([len(sc.drag)])}


def scene_from_arrays(g):
    import ctypes as C
    from simulation_project_gb300.scenes import Scene
    from simulation_project_gb300.types import CParameter, CGridBox, CTriangleParameters, DragParameter
    param = CParameter.from_buffer_copy(g["in_param"].tobytes())
    box = CGridBox.from_buffer_copy(g["in_box"].tobytes())
    ntp = g["in_tparams"].nbytes // C.sizeof(CTriangleParameters)
    tps = (CTriangleParameters * ntp).from_buffer_copy(g["in_tparams"].tobytes())
    nd = int(g["in_ndrag"][0])
    dps = (DragParameter * max(nd, 1)).from_buffer_copy(g["in_drag"].tobytes())
    return Scene(name="golden", param=param, box=box, pos=g["in_pos"], vel=g["in_vel"], press=g["in_press"],
                 visc=g["in_visc"], ptype=g["in_type"], tri_vertices=g["in_tri"], tri_model=g["in_tri_model"],
                 tri_params=list(tps), drag=list(dps)[:nd])


def math_cases(lib):
    rng = np.random.default_rng(13)
    rs = (np.concatenate([rng.uniform(0, 4.5, 400), np.arange(0, 4.2, 0.05)]) * 0.004).astype(np.float32)
    out = {"r": rs}
    for fn in ["zgrad", "zlap", "zgrad2d", "zlap2d"]:
        out[fn] = np.array([getattr(lib, fn)(r, np.float32(0.004)) for r in rs], dtype=np.float32)
    xs = rng.uniform(0, 2, 300).astype(np.float32)
    out["sqrt_x"] = xs
    out["sqrt"] = np.array([lib.sqrt_utility(x) for x in xs], dtype=np.float32)
    tv = rng.normal(0, 0.05, (300, 3, 3)).astype(np.float32)
    tp = rng.normal(0, 0.05, (300, 3)).astype(np.float32)
    tn = orc.triangle_normals_q(tv)
    mags, dirs = [], []
    for i in range(300):
        t = CTriangle()
        for q in range(3):
            t.Vertex[q] = Scalar3(*tv[i, q])
        t.Normal = Scalar3(*tn[i])
        d = Scalar3()
        mags.append(lib.triangle_distance(C.byref(t), C.byref(Scalar3(*tp[i])), C.byref(d)))
        dirs.append((d.x, d.y, d.z))
    out.update(tri_v=tv, tri_p=tp, tri_n=tn, tri_mag=np.array(mags, np.float32), tri_dir=np.array(dirs, np.float32))
    return out


def main():
    ref = orc.reference()
    if ref is None:
        raise SystemExit("reference sources not available")
    for name, sc in golden_scenes().items():
        pred, final = explicit_step(ref, sc)
        arrays = scene_to_arrays(sc)
        arrays.update({f"pred_{k}": v for k, v in pred.items()})
        arrays.update({f"final_{k}": v for k, v in final.items()})
        np.savez_compressed(os.path.join(HERE, f"ref_explicit_{name}.npz"), **arrays)
    np.savez_compressed(os.path.join(HERE, "ref_math.npz"), **math_cases(ref))
    sc, temps = thermal_turbulent_scene()
    arrays = scene_to_arrays(sc)
    arrays["in_temp"] = temps
    arrays.update({f"out_{k}": v for k, v in thermal_turbulent_step(ref, sc, temps).items()})
    np.savez_compressed(os.path.join(HERE, "ref_thermal_turbulent.npz"), **arrays)
    print("written")


if __name__ == "__main__":
    main()
