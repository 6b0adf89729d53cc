"""Benchmark: particle-steps/s of the semi-implicit MPS step on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--l0 0.002]

Workload: the rotating bucket (cylinder r = 0.15 m, L = 0.3 m, 4096 wall triangles,
30 rpm, 64 drag spheres of radius 3*l0) filled 35 % at l0 = 0.002 m (~0.9M
particles), PPE solved to relative residual 1e-8.  Synthetic inputs: seeded jittered
lattice, no dataset.  One "step" is one full solver step (topology, walls, drag,
predictor, topology, PND, PPE solve, pressure-gradient correction, wall motion).

value       = particle-steps/s of the FP32-operator / FP64-refined solver with the
              multilevel preconditioner and the learned initial guess (trained on the
              GPU by the library's own BF16 tensor-core kernels before the timed
              region), states resident in HBM, the solver's per-phase CUDA events off
              (the default);
plain_fp64  = the same steps with every operator and Jacobi-PCG in FP64 (its CG SpMV
              streamed as the FP32 one, over FP64 weights), with the roofline of
              that SpMV;
e2e         = the learned solver driven through the public C-ABI from pinned host
              buffers: each step uploads the state, steps, and downloads it.
roofline    = the PPE SpMV (the dominant kernel) timed with CUDA events on the solver
              stream over the metric's steps run a second time with the per-phase
              events on (which also give fast_solver.phases_ms); algorithmic bytes per
              launch = 4 B per neighbour entry (16-bit column + FP16 weight) + 25 B per
              interior row;
              traffic = DRAM bytes per entry from one ncu capture at full size
              (SPMV_DRAM_BYTES_PER_ENTRY) times the live entry count.
sort        = SortUsingThrust (stable LSD radix sort of (cell key, index)) on the
              particle count with keys in the cell-key range, keys/s and GB/s.
accuracy    = the FP32-IR solver against the FP64 solver on the same scene after
              10 steps: pressure, PND, velocity, kinetic energy, positions.
cpu_baseline= the FP64 oracle solver with OpenMP on the host cores, on a bounded
              sample (the same bucket at l0 = 0.004, ~1e5 particles, 1 step).
--impl reference: the reference's own explicit-schedule kernels compiled for the CPU
              (oracle/_ref/libref.so, OpenMP over particles), timed per step on the
              same scene as the GPU arm (the reference has no PPE solver: its scheme
              is the explicit equation-of-state pressure).
Multi-GPU: replicas only (each rank runs its own scene; value = sum over ranks).
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
# compulsory bytes per particle of one step, per FP32 CG iteration and per FP64
# refinement pass (hash, sort, reorder, walls, predictor, PND/RHS, correction;
# SpMV + dots + vector updates; residual)
STEP_FIXED_B, STEP_ITER_B, STEP_IR_B = 760.0, 72.0, 48.0
# DRAM bytes per neighbour entry of one k_spmv_stream launch, measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum, one pass) on the default workload
# with 16-bit column offsets: 1.3376 GB read + 2.2 MB written for 201.36M entries
# (SELL padding included)
SPMV_DRAM_BYTES_PER_ENTRY = (1.33758e9 + 2.24e6) / 201.362e6
# warp instructions per particle of the two FP32 neighbour passes, counted by ncu
# (smsp__inst_executed.sum, one launch on the bucket at l0 = 0.004, 108,186 particles):
# the list pass 233.67M, the predictor 213.7M
NB_LIST_INST_PER_PARTICLE = 233.67e6 / 108186
NB_PRED_INST_PER_PARTICLE = 213.7e6 / 108186
# the same for the FP16-weight kernel of the inner CG (k_spmv_stream<..., __half>):
# 898.3 MB read + 1.8 MB written for 201.36M entries
SPMV16_DRAM_BYTES_PER_ENTRY = (898.3e6 + 1.8e6) / 201.362e6


def load_peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_bf16_peak():
    """Measured dense BF16 tensor throughput (burst) in TFLOP/s, else the fallback 1900."""
    try:
        with open(MEASURED_PEAKS) as f:
            return float(json.load(f)["bf16_tflops"])
    except Exception:
        return 1900.0


class ClockSampler:
    """nvidia-smi samples (SM clock, max clock, throttle reasons) during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "25"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
            # the timed region starts once samples flow (nvidia-smi takes a moment to start)
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.lines.clear()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_scene(l0, seed=4, workload="bucket"):
    from simulation_project_gb300 import scenes
    if workload == "mixer":
        # four rotating cylinders (radii 0.10-0.18 m, 20-45 rpm, seeded), 40 % fill, 512 drag spheres
        return scenes.mixer(l0=l0, dt=5e-5, seed=6 + seed - 4)
    return scenes.rotating_bucket(l0=l0, dt=5e-5, seed=seed, n_drag=64, drag_seed=3)


WORKLOADS = {
    "bucket": "rotating bucket r=0.15 L=0.3, 35% fill, l0={l0}, 30 rpm, 4096 wall + 64 drag-sphere STL models, "
              "dt=5e-5, PPE rtol 1e-8",
    "mixer": "4-cylinder mixer (r 0.10-0.18 m, L=0.3, 20-45 rpm, seed 6), 40% fill, l0={l0}, 512 drag spheres, "
             "dt=5e-5, PPE rtol 1e-8",
}


def barrier():
    """Host barrier over the replica ranks (no-op for one process)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def combine_replicas(units, ms, steps):
    """Whole-job throughput of independent replicas: the particle-steps every rank
    completed over the slowest rank's timed region.  `units` and `ms` are the ranks'
    own (particle-steps, milliseconds) in a list over ranks."""
    slowest = max(ms)
    return {"value": sum(units) / (slowest / 1e3), "ms_per_step": slowest / steps}


def gather_replicas(res):
    """Replace a rank's own value / ms_per_step with the whole-job numbers (all ranks
    call this; a gloo group carries two numbers per rank, nothing on the data path)."""
    import torch.distributed as dist
    world = dist.get_world_size()
    mine = (res["units"], res["ms_per_step"] * res["steps"])
    rows = [None] * world
    dist.all_gather_object(rows, mine)
    res.update(combine_replicas([u for u, _ in rows], [m for _, m in rows], res["steps"]))
    res["n_gpus"] = world
    return res


def time_steps(solver, steps, warmup, first_step=0):
    from simulation_project_gb300 import lib
    for i in range(warmup):
        solver.step(first_step + i)
    stream = C.c_void_p(solver.stream())
    ev0, ev1 = lib.Event(), lib.Event()
    lib.call("mps_device_sync")
    barrier()
    stats = []
    launches0 = lib.kernel_launches()
    ev0.record(_S(stream))
    t0 = time.perf_counter()
    for i in range(steps):
        stats.append(solver.step(first_step + warmup + i))
    ev1.record(_S(stream))
    lib.call("mps_device_sync")
    wall = time.perf_counter() - t0
    barrier()
    if stats:
        stats[0]["launches_in_region"] = lib.kernel_launches() - launches0
    return ev0.elapsed_ms(ev1), wall, stats


class _S:
    def __init__(self, h):
        self.handle = h


def train_learned(solver_cls, scene, steps_data, device_log):
    """Generates (state, converged pressure) pairs with the plain solver and trains the
    MLP on the GPU; returns the parameters (or None if the learned part is absent)."""
    try:
        from simulation_project_gb300 import learned
    except Exception as e:  # pragma: no cover
        device_log.append(f"learned part unavailable: {e}")
        return None, {}
    return learned.train_on_scene(scene, steps=steps_data, log=device_log)


def run_gpu(args):
    from simulation_project_gb300 import lib
    from simulation_project_gb300.solver import Solver
    lib.load()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    lib.call("mps_set_device", local)
    scene = build_scene(args.l0, seed=4 + rank, workload=args.workload)
    n = scene.n
    log = []
    peak_gbs, peak_kind = load_peaks()

    # learned part: data from the plain solver, training on the GPU (untimed)
    params, train_info = (None, {})
    if not args.no_learned:
        params, train_info = train_learned(Solver, scene, args.train_steps, log)

    # plain FP64 Jacobi-CG (metric denominator), from the previous pressure
    plain = Solver(scene, precision="fp64", profile=0, warm_start=0)
    ms_plain, _, st_plain = time_steps(plain, args.steps, args.warmup)
    plain.close()
    pps_plain = n * args.steps / (ms_plain / 1e3)
    plain_roof = plain_fp64_roofline(scene, args, peak_gbs)

    # FP32 / FP64-refined solver without the network: Jacobi, then multilevel
    # the FP32 arms all run without phase events, as the metric's timed solver does, so
    # that they compare like for like
    ir = Solver(scene, precision="fp32_ir", profile=0, preconditioner=0)
    ms_ir, _, st_ir = time_steps(ir, args.steps, args.warmup)
    ir.close()
    pps_ir = n * args.steps / (ms_ir / 1e3)
    irm = Solver(scene, precision="fp32_ir", profile=0, preconditioner=1)
    ms_irm, _, st_irm = time_steps(irm, args.steps, args.warmup)
    irm.close()
    pps_irm = n * args.steps / (ms_irm / 1e3)
    # the same from the previous pressure (no extrapolation of the pressure history)
    irm0 = Solver(scene, precision="fp32_ir", profile=0, preconditioner=1, warm_start=0)
    ms_irm0, _, st_irm0 = time_steps(irm0, args.steps, args.warmup)
    irm0.close()
    pps_irm0 = n * args.steps / (ms_irm0 / 1e3)

    # learned FP32 / FP64-refined solver (metric numerator), timed as a user runs it:
    # without the per-phase CUDA events (an event at every phase switch, four per CG
    # iteration, adds ~0.3 ms per step)
    def fast_solver(profile):
        s = Solver(scene, precision="fp32_ir", profile=profile, preconditioner=args.precond,
                   learned=args.learned_mode if params is not None else 0)
        if params is not None:
            s.set_learned(params)
        return s

    fast = fast_solver(0)
    clocks = ClockSampler(local)
    for i in range(args.warmup):
        fast.step(i)
    clocks.start()
    ms_fast, wall_fast, st_fast = time_steps(fast, args.steps, 0, first_step=args.warmup)
    clk = clocks.stop()
    pps_fast = n * args.steps / (ms_fast / 1e3)
    # the same steps again with the phase events on the solver stream: per-phase times
    # and the SpMV's event-timed launches for the roofline
    fast_prof = fast_solver(1)
    ms_prof, _, st_prof = time_steps(fast_prof, args.steps, args.warmup)
    fast_prof.close()

    # roofline of the dominant kernel (PPE SpMV, FP32 rows)
    spmv_ms = sum(s["ms_spmv"] for s in st_prof)
    # SpMVs that did work: one per CG iteration.  The CG runs in batches of 8 and the
    # launches of a batch after convergence return at once; their few microseconds
    # each stay in spmv_ms (so the figure is slightly conservative).
    spmv_n = sum(s["cg_iterations"] for s in st_prof)
    spmv_issued = sum(s["spmv_launches"] for s in st_prof)
    nnz = np.mean([s["nnz"] for s in st_prof])
    nnz_wide = np.mean([s["nnz_wide"] if s["rows16"] else s["nnz"] for s in st_prof])
    interior = np.mean([s["interior"] for s in st_prof])
    inner16 = all(s["inner16"] for s in st_prof)
    # weight (2 B FP16 or 4 B FP32) + 2 B (16-bit offset) or 4 B column per entry, 25 B
    # per interior row
    wb = 2.0 if inner16 else 4.0
    bytes_launch = (wb + 2.0) * (nnz - nnz_wide) + (wb + 4.0) * nnz_wide + 25.0 * interior
    avg_ms = spmv_ms / max(spmv_n, 1)
    achieved = bytes_launch / (avg_ms / 1e3) / 1e9 if spmv_n else 0.0
    wide = nnz_wide * 2 > nnz   # the solver streams every slice's 32-bit columns then
    if wide:
        kname = ("k_spmv_stream<0,8,2,8,4,%s,true> (inner-CG SpMV, %s weights + 32-bit columns streamed by bulk copies)"
                 % (("__half", "FP16") if inner16 else ("float", "FP32")))
    else:
        kname = ("k_spmv_stream<0,16,2,8,4,__half> (inner-CG SpMV, FP16 weights + 16-bit columns streamed by bulk copies)"
                 if inner16 else
                 "k_spmv_stream<0,8,2,8,4> (inner-CG SpMV, FP32 weights + 16-bit columns streamed by bulk copies)")
    # DRAM bytes per entry were captured for the 16-bit-column kernels only
    per_entry = None if wide else (SPMV16_DRAM_BYTES_PER_ENTRY if inner16 else SPMV_DRAM_BYTES_PER_ENTRY)
    roofline = {"bound": "hbm", "kernel": kname,
                "achieved": round(achieved, 1), "peak": peak_gbs, "unit": "GB/s",
                "frac": round(achieved / peak_gbs, 3), "peak_kind": peak_kind,
                "traffic": int(per_entry * nnz) if per_entry else None,
                "traffic_source": ("ncu dram bytes per entry x entries" if per_entry else
                                   "not captured for the 32-bit-column layout"),
                "entries": int(nnz), "entries_32bit_columns": int(nnz_wide),
                "bytes_per_launch": int(bytes_launch), "launches": spmv_n, "launches_issued": spmv_issued,
                "avg_launch_us": round(avg_ms * 1e3, 2),
                "timed_in": "the metric's steps run again with phase events on the solver stream"}
    phases = {k: round(float(np.mean([s[k] for s in st_prof])), 3) for k in
              ("ms_grid", "ms_walls", "ms_predictor", "ms_list", "ms_ppe_setup", "ms_spmv", "ms_cg_vec",
               "ms_correct", "ms_learned", "ms_precond")}
    # compulsory bytes of the whole step: N (760 + k_CG 72 + k_IR 48) B with the FP32
    # operator recomputed from positions (the stored SELL rows are extra, reported beside)
    k_cg = float(np.mean([s["cg_iterations"] for s in st_fast]))
    k_ir = float(np.mean([s["ir_passes"] for s in st_fast]))
    step_bytes = n * (STEP_FIXED_B + k_cg * STEP_ITER_B + k_ir * STEP_IR_B)
    step_gbs = step_bytes / (ms_fast / args.steps / 1e3) / 1e9
    step_model = {"model": "N*(760 + k_CG*72 + k_IR*48) bytes per step", "k_cg": k_cg, "k_ir": k_ir,
                  "bytes_per_step": int(step_bytes), "achieved_gbs": round(step_gbs, 1),
                  "frac": round(step_gbs / peak_gbs, 4),
                  "stored_row_bytes_per_step": int(k_cg * bytes_launch)}
    # accepted Laplacian pairs of the two neighbour passes (predictor and rows/PND)
    pairs = float(np.mean([s["pairs"] for s in st_fast]))
    nb_ms = phases["ms_predictor"] + phases["ms_list"]
    pair_evals = {"accepted_pairs_per_pass": int(pairs), "accepted_per_particle": round(pairs / n, 1),
                  "passes": 2, "pairs_per_s": 2.0 * pairs / (nb_ms / 1e3) if nb_ms > 0 else None}
    # each neighbour pass against the HBM roofline with its algorithmic bytes (list: 8 B
    # per stored entry + 48 B per row; predictor: 96 B per row), and against the issue
    # rate that bounds them: the warp instructions ncu counted per particle over the
    # event-timed pass, against one instruction per cycle per scheduler (4 per SM) at the
    # SM clock sampled during the timed steps
    nb_passes = {}
    sms = lib_sm_count()
    sm_hz = (clk.get("sm_mhz") or 0.0) * 1e6
    for key, ms, nbytes, ipp in (("list", phases["ms_list"], 8.0 * pairs + 48.0 * n, NB_LIST_INST_PER_PARTICLE),
                                 ("predictor", phases["ms_predictor"], 96.0 * n, NB_PRED_INST_PER_PARTICLE)):
        gbs = nbytes / (ms / 1e3) / 1e9 if ms > 0 else 0.0
        issue = (ipp * n / (ms / 1e3)) / (4.0 * sms * sm_hz) if ms > 0 and sms and sm_hz else None
        nb_passes[key] = {"ms": round(ms, 3), "bytes": int(nbytes), "achieved_gbs": round(gbs, 1),
                          "hbm_frac": round(gbs / peak_gbs, 4), "bound": "issue",
                          "warp_instructions_per_particle": round(ipp, 1),
                          "issue_frac": round(issue, 3) if issue is not None else None}
    pair_evals["passes_vs_hbm"] = nb_passes

    # end to end through the C-ABI from pinned host buffers
    e2e = run_e2e(fast, args)
    frames = frames_bench(fast, n, args)
    inflow = inflow_bench(scene, n)
    fast.close()
    sort = sort_bench(n, scene.box.cell_num, peak_gbs)
    mlp = mlp_bench(params, n, load_bf16_peak())
    training_gemms = gemm_bench(load_bf16_peak())
    ref_named = reference_named_bench()
    accuracy = accuracy_vs_fp64(scene, params, args, steps=args.accuracy_steps)

    result = {
        "metric": "particle-steps/s @1M on 1 GB300, learned-precond vs plain CG at 1e-8 PPE residual",
        "value": pps_fast,
        "units": n * args.steps,
        "unit": "particle-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_fast / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic (seeded jittered lattice in a triangulated rotating cylinder)",
        "config": gpu_config(args, scene, world),
        "plain_fp64": {"value": pps_plain, "ms_per_step": ms_plain / args.steps,
                       "cg_iterations_per_step": float(np.mean([s["cg_iterations"] for s in st_plain])),
                       "relres_max": float(max(s["cg_relres"] for s in st_plain)),
                       "roofline": plain_roof},
        "speedup_vs_plain_fp64": pps_fast / pps_plain,
        "fp32_ir_jacobi_without_network": {"value": pps_ir, "ms_per_step": ms_ir / args.steps,
                                           "cg_iterations_per_step": float(np.mean([s["cg_iterations"] for s in st_ir])),
                                           "ir_passes_per_step": float(np.mean([s["ir_passes"] for s in st_ir]))},
        "fp32_ir_multilevel_without_network": {
            "value": pps_irm, "ms_per_step": ms_irm / args.steps,
            "cg_iterations_per_step": float(np.mean([s["cg_iterations"] for s in st_irm])),
            "ir_passes_per_step": float(np.mean([s["ir_passes"] for s in st_irm]))},
        "fp32_ir_multilevel_previous_pressure": {
            "value": pps_irm0, "ms_per_step": ms_irm0 / args.steps,
            "cg_iterations_per_step": float(np.mean([s["cg_iterations"] for s in st_irm0])),
            "ir_passes_per_step": float(np.mean([s["ir_passes"] for s in st_irm0]))},
        "extrapolation_iterations_saved_per_step": float(
            np.mean([s["cg_iterations"] for s in st_irm0]) - np.mean([s["cg_iterations"] for s in st_irm])),
        "network_iterations_saved_per_step": float(
            np.mean([s["cg_iterations"] for s in (st_irm if args.precond else st_ir)]) -
            np.mean([s["cg_iterations"] for s in st_fast])),
        "fast_solver": {"cg_iterations_per_step": float(np.mean([s["cg_iterations"] for s in st_fast])),
                        "ir_passes_per_step": float(np.mean([s["ir_passes"] for s in st_fast])),
                        "relres_max": float(max(s["cg_relres"] for s in st_fast)),
                        "fallbacks": int(sum(s["fallback"] for s in st_fast)),
                        "error_flags": int(np.bitwise_or.reduce([s["error_flags"] for s in st_fast])),
                        "learned": params is not None, "preconditioner": ["jacobi", "multilevel"][args.precond],
                        "learned_gate": {
                            "steps_with_learned_guess": int(sum(s["learned_applied"] for s in st_fast)),
                            "steps": len(st_fast),
                            "saved_its_when_applied": [round(s["learned_saved_its"], 3) for s in st_fast
                                                       if s["learned_applied"]],
                            "cost_its_when_applied": [round(s["learned_cost_its"], 3) for s in st_fast
                                                      if s["learned_applied"]]},
                        "flexible_cg": bool(all(s["flexible"] for s in st_fast)),
                        "warm_start_order": int(st_fast[-1]["warm_start"]),
                        "mg_levels": int(st_fast[-1]["mg_levels"]), "mg_level1": int(st_fast[-1]["mg_level1"]),
                        "phases_ms": phases,
                        "ms_per_step_with_phase_events": ms_prof / args.steps},
        "learned_training": train_info,
        "roofline": roofline,
        "step_bytes": step_model,
        "pair_evaluations": pair_evals,
        "sort": sort,
        "mlp_inference": mlp,
        "mlp_training_gemms": training_gemms,
        "reference_named_step": ref_named,
        "accuracy_vs_fp64": accuracy,
        "e2e": e2e,
        "frames": frames,
        "inflow": inflow,
        "gpu_launches": int(st_fast[0]["launches_in_region"]),
        "clocks": clk,
    }
    if rank == 0 and world == 1:
        result["cpu_baseline"] = cpu_baseline(args)
    if log:
        result["notes"] = log
    return result


def plain_fp64_roofline(scene, args, peak_gbs, steps=3):
    """Roofline of the plain FP64 solver's CG SpMV (k_spmv_stream64 over 16-bit columns
    and FP64 weights, or the register walk where no slice fits 16 bits): a separate
    profiled run of `steps` steps after the warm-up (phase events on the solver stream),
    so that the timed denominator carries no event overhead.  Algorithmic bytes per
    launch: 8 B weight + 2 B (16-bit) or 4 B (32-bit) column per neighbour entry, and
    33 B per interior row (x, y, diagonal: 8 B each; count 4 B; interior flag 1 B)."""
    from simulation_project_gb300.solver import Solver
    s = Solver(scene, precision="fp64", profile=1, warm_start=0)
    _, _, st = time_steps(s, steps, args.warmup)
    s.close()
    spmv_ms = sum(x["ms_spmv"] for x in st)
    its = sum(x["cg_iterations"] for x in st)
    nnz = float(np.mean([x["nnz"] for x in st]))
    rows16 = all(x["rows16"] for x in st)
    nnz_wide = float(np.mean([x["nnz_wide"] for x in st])) if rows16 else nnz
    interior = float(np.mean([x["interior"] for x in st]))
    wide = nnz_wide * 2 > nnz
    bytes_launch = 10.0 * (nnz - nnz_wide) + 12.0 * nnz_wide + 33.0 * interior
    avg_ms = spmv_ms / max(its, 1)
    achieved = bytes_launch / (avg_ms / 1e3) / 1e9 if its else 0.0
    kname = ("k_spmv_stream64<0,8,2,8,4%s> (FP64 CG SpMV, FP64 weights + %s columns streamed by bulk copies)"
             % ((",true", "32-bit") if wide else ("", "16-bit"))) if rows16 else \
        "k_spmv<double,double,double,0> (FP64 CG SpMV, register walk)"
    return {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1), "peak": peak_gbs, "unit": "GB/s",
            "frac": round(achieved / peak_gbs, 3), "bytes_per_launch": int(bytes_launch), "entries": int(nnz),
            "entries_32bit_columns": int(nnz_wide), "launches": its, "avg_launch_us": round(avg_ms * 1e3, 2),
            "fp64_flop_per_launch": int(2 * nnz), "steps_profiled": steps}


def mlp_bench(params, n, tflops_peak, reps=20):
    """The learned guess's MLP inference on n rows of features: the tcgen05 kernel the
    solver runs (variant 0), the mma.sync cross-check kernel (variant 1) and the tcgen05
    kernel with 0..3 of every 4 pairs of hidden activations on the FMA pipe (variants
    2..5, the share variant 0 uses among them), CUDA events on the legacy stream around
    `reps` launches after 3 warm-up launches."""
    from simulation_project_gb300 import lib
    from simulation_project_gb300.learned import Mlp
    if params is None:
        return None
    m = Mlp(max_batch=8192, seed=1)
    m.set_params(params)
    X = lib.DeviceArray.from_host(np.random.default_rng(11).normal(0, 1, (n, 12)).astype(np.float32))
    Y = lib.DeviceArray((n, 2), np.float32)
    out = {"rows": n, "flop_per_row_padded": 73728}
    ev0, ev1 = lib.Event(), lib.Event()
    for v, name in ((0, "tcgen05"), (1, "mma_sync"), (2, "tcgen05_silu_sfu_only"), (3, "tcgen05_silu_fma_1of4"),
                    (4, "tcgen05_silu_fma_2of4"), (5, "tcgen05_silu_fma_3of4")):
        for _ in range(3):
            m.forward(X.ptr, Y.ptr, n, variant=v)
        lib.call("mps_device_sync")
        ev0.record(None)
        for _ in range(reps):
            m.forward(X.ptr, Y.ptr, n, variant=v)
        ev1.record(None)
        lib.call("mps_device_sync")
        us = ev0.elapsed_ms(ev1) / reps * 1e3
        tf = 73728.0 * n / (us / 1e6) / 1e12
        out[name] = {"us_per_launch": round(us, 1), "tflops": round(tf, 1),
                     "frac_of_bf16_peak": round(tf / tflops_peak, 3) if tflops_peak else None}
    out["timeouts"] = Mlp.tc_timeouts()
    X.free()
    Y.free()
    m.close()
    return out


def reference_named_bench(steps=5, warmup=2):
    """The reference's explicit schedule through the reference-named launchers
    (simulation_project_gb300.refpath.RefStep: CCellSet's device arrays bound once, one
    step of CMultiGPUHandler::Calculate per call): wall time per step, including the
    host synchronisations the reference's launcher API implies (compaction count, the
    sort on the legacy stream), on the bench bucket at l0 = 0.002 and 0.004."""
    from simulation_project_gb300 import lib
    from simulation_project_gb300.refpath import RefStep
    out = {"scheme": "explicit (equation-of-state) pressure, the reference's own schedule and kernels' arithmetic"}
    for name, l0 in (("l0_0.002", 0.002), ("l0_0.004", 0.004)):
        sc = build_scene(l0)
        g = RefStep(sc)
        for i in range(warmup):
            g.step(i)
        g.sync()
        lib.call("mps_device_sync")
        t0 = time.perf_counter()
        for i in range(steps):
            g.step(warmup + i)
        g.sync()
        dt = time.perf_counter() - t0
        out[name] = {"particles": sc.n, "steps": steps, "ms_per_step": round(dt * 1e3 / steps, 3),
                     "particle_steps_per_s": sc.n * steps / dt}
        g.close()
    return out


def gemm_bench(tflops_peak, reps=20):
    """The MLP's training GEMMs (mps_gemm_bf16_variant) on the shapes of one Adam step of
    8192 rows: a hidden layer's forward (8192 x 128 x 128, bias + SiLU epilogue) and a
    weight gradient (128 x 128 over K = 8192, split 16); the tcgen05 kernel training
    uses (variant 0) and the mma.sync cross-check (variant 1), CUDA events on the legacy
    stream around `reps` launches after 3 warm-up launches."""
    from simulation_project_gb300 import lib
    from simulation_project_gb300.learned import gemm_bf16
    rng = np.random.default_rng(3)
    Mb, H = 8192, 128
    X = lib.DeviceArray.from_host(rng.integers(0, 1 << 15, (Mb, H), dtype=np.uint16))
    W = lib.DeviceArray.from_host(rng.integers(0, 1 << 15, (H, H), dtype=np.uint16))
    G = lib.DeviceArray.from_host(rng.integers(0, 1 << 15, (Mb, H), dtype=np.uint16))
    bias = lib.DeviceArray.from_host(np.zeros(H, np.float32))
    Y = lib.DeviceArray((Mb, H), np.float32)
    Yb = lib.DeviceArray((Mb, H), np.uint16)
    dW = lib.DeviceArray((H, H), np.float32)
    ev0, ev1 = lib.Event(), lib.Event()
    out = {}
    shapes = {
        "forward_8192x128x128": (lambda v: gemm_bf16(Mb, H, H, X.ptr, H, 0, W.ptr, H, 0, None, H, Cb=Yb.ptr, ldcb=H,
                                                      Cz=Y.ptr, bias=bias.ptr, act=1, variant=v), 2.0 * Mb * H * H),
        "weight_grad_128x128_k8192": (lambda v: gemm_bf16(H, H, Mb, X.ptr, H, 1, G.ptr, H, 0, dW.ptr, H, beta=1.0,
                                                           split=16, variant=v), 2.0 * Mb * H * H),
    }
    for name, (fn, flop) in shapes.items():
        out[name] = {}
        for v, vname in ((0, "tcgen05"), (1, "mma_sync")):
            for _ in range(3):
                fn(v)
            lib.call("mps_device_sync")
            ev0.record(None)
            for _ in range(reps):
                fn(v)
            ev1.record(None)
            lib.call("mps_device_sync")
            us = ev0.elapsed_ms(ev1) / reps * 1e3
            tf = flop / (us / 1e6) / 1e12
            out[name][vname] = {"us_per_launch": round(us, 2), "tflops": round(tf, 1),
                                "frac_of_bf16_peak": round(tf / tflops_peak, 4)}
    for a in (X, W, G, bias, Y, Yb, dW):
        a.free()
    return out


def sort_bench(n, cells, peak_gbs, reps=10):
    """SortUsingThrust on n keys uniform in [0, cells) (the cell-key range of the
    workload), timed with CUDA events on the legacy stream the sort runs on."""
    from simulation_project_gb300 import lib
    rng = np.random.default_rng(9)
    keys0 = rng.integers(0, cells, n, dtype=np.int32)
    dk, dv = lib.DeviceArray((n,), np.int32), lib.DeviceArray((n,), np.int32)
    L = lib.load()
    L.SortUsingThrust.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    idx = np.arange(n, dtype=np.int32)
    ev0, ev1 = lib.Event(), lib.Event()
    total = 0.0
    for r in range(reps + 2):
        dk.upload(keys0)
        dv.upload(idx)
        lib.call("mps_device_sync")
        ev0.record(None)
        if L.SortUsingThrust(n, dk.ptr, dv.ptr) != 0:
            raise RuntimeError("SortUsingThrust failed")
        ev1.record(None)
        lib.call("mps_device_sync")
        if r >= 2:
            total += ev0.elapsed_ms(ev1)
    ok = bool(np.array_equal(dk.download(), np.sort(keys0, kind="stable")))
    ms = total / reps
    passes = max(1, (int(cells - 1).bit_length() + 7) // 8)
    gbs = 16.0 * n * passes / (ms / 1e3) / 1e9   # read + write of key and value per pass
    dk.free()
    dv.free()
    return {"keys": n, "key_range": int(cells), "passes": passes, "ms": round(ms, 4),
            "keys_per_s": n / (ms / 1e3), "achieved_gbs": round(gbs, 1), "peak_gbs": peak_gbs,
            "frac": round(gbs / peak_gbs, 3), "sorted_correctly": ok}


def _compare_states(sa, sb, scene):
    """Errors of state sb against state sa over the particle ids both still hold."""
    common, ia, ib = np.intersect1d(sa["id"], sb["id"], return_indices=True)
    pa, pb = sa["press"][ia], sb["press"][ib]
    va, vb = sa["vel"][ia], sb["vel"][ib]
    na, nb = sa["pnd"][ia], sb["pnd"][ib]
    ke_a, ke_b = 0.5 * np.sum(va * va), 0.5 * np.sum(vb * vb)
    l0 = scene.param.InitialParticleDistance
    q = np.array([50, 90, 99])
    return {"particles_compared": int(len(common)),
            "pressure_max_rel": float(np.abs(pb - pa).max() / np.abs(pa).max()),
            "pressure_rms_rel": float(np.sqrt(np.mean((pb - pa) ** 2)) / np.sqrt(np.mean(pa ** 2))),
            "pressure_mean_rel": float(abs(pb.mean() - pa.mean()) / np.abs(pa).mean()),
            "pressure_percentiles_rel": [float(x) for x in
                                         np.abs(np.percentile(pb, q) - np.percentile(pa, q)) / np.abs(pa).max()],
            "pnd_max_rel": float(np.abs(nb - na).max() / scene.n0_pnd),
            "velocity_max_rel": float(np.abs(vb - va).max() / np.abs(va).max()),
            "kinetic_energy_rel": float(abs(ke_b - ke_a) / ke_a),
            "position_max_over_l0": float(np.abs(sb["pos"][ib] - sa["pos"][ia]).max() / l0)}


def accuracy_vs_fp64(scene, params, args, steps=10):
    """The metric's solver (FP32 operators, FP64 refinement, multilevel, learned guess)
    against the FP64 solver on the same scene after `steps` steps, and a control:
    the FP64 solver against itself started from positions moved by 5e-6 l0, about the
    resolution of an FP32 coordinate in this box (the divergence that perturbations of
    FP32 size reach in a free-surface particle flow)."""
    import copy
    from simulation_project_gb300.solver import Solver
    pert = copy.copy(scene)
    rng = np.random.default_rng(11)
    pert.pos = scene.pos + 5e-6 * scene.param.InitialParticleDistance * rng.standard_normal(scene.pos.shape)
    a = Solver(scene, precision="fp64")
    c = Solver(pert, precision="fp64")
    b = Solver(scene, precision="fp32_ir", preconditioner=args.precond,
               learned=args.learned_mode if params is not None else 0)
    if params is not None:
        b.set_learned(params)
    for i in range(steps):
        a.step(i)
        b.step(i)
        c.step(i)
    sa, sb, sc_ = a.state(), b.state(), c.state()
    for x in (a, b, c):
        x.close()
    out = {"steps": steps, "reference": "FP64 solver on the GPU (matches the FP64 oracle to 1e-6 on the parity cases)"}
    out.update(_compare_states(sa, sb, scene))
    out["control_fp64_perturbed_5e-6_l0"] = _compare_states(sa, sc_, scene)
    return out


def run_profile_case(args):
    """Only the FP32-IR solver steps (no training, no other arms): the command the ncu
    captures under profiles/ run."""
    from simulation_project_gb300 import lib
    from simulation_project_gb300.solver import Solver
    lib.load()
    scene = build_scene(args.l0, workload=args.workload)
    params = None
    if args.profile_learned:
        params, _ = train_learned(Solver, scene, args.train_steps, [])
    s = Solver(scene, precision="fp64" if args.fp64 else "fp32_ir", profile=1, preconditioner=args.precond,
               learned=args.learned_mode if params is not None else 0)
    if params is not None:
        s.set_learned(params)
    # the last step separately, with the library's launch count before it (the -s of an
    # ncu launch list of that step)
    ms, _, st = time_steps(s, args.steps - 1, args.warmup) if args.steps > 1 else (0.0, None, [])
    before = lib.kernel_launches()
    ms1, _, st1 = time_steps(s, 1, 0, first_step=args.warmup + args.steps - 1)
    after = lib.kernel_launches()
    ms, st = ms + ms1, st + st1
    s.close()
    print(json.dumps({"profile_case": True, "particles": scene.n, "ms_per_step": ms / args.steps,
                      "launches_before_last_step": before, "launches_last_step": after - before,
                      "phases": {k: st[-1][k] for k in st[-1] if k.startswith("ms_")},
                      "spmv_launches": st[-1]["spmv_launches"], "nnz": st[-1]["nnz"],
                      "cg_iterations": st[-1]["cg_iterations"], "mg_levels": st[-1]["mg_levels"]}))
    return 0


def run_accuracy_only(args):
    """The FP32-IR learned solver against the FP64 solver after --accuracy-steps steps."""
    from simulation_project_gb300 import lib
    from simulation_project_gb300.solver import Solver
    lib.load()
    scene = build_scene(args.l0, workload=args.workload)
    params, info = (None, {}) if args.no_learned else train_learned(Solver, scene, args.train_steps, [])
    t0 = time.perf_counter()
    acc = accuracy_vs_fp64(scene, params, args, steps=args.accuracy_steps)
    print(json.dumps({"accuracy_vs_fp64": acc, "workload": WORKLOADS[args.workload].format(l0=args.l0),
                      "particles": scene.n, "learned": params is not None, "seconds": time.perf_counter() - t0}))
    return 0


def inflow_bench(scene, n, bucket=10_000):
    """Device-side inflow (mps_solver_add_particles, InsertBucket semantics) outside the
    timed region: a separate solver of the same scene with room for the bucket, warmed
    up; the time to insert a bucket (hole scan over the IDs, count read-back, upload,
    insert kernel) and the next step (which sorts the new particles in; the bucket sits
    outside the compute zone, so that step also removes it again)."""
    from simulation_project_gb300 import lib
    from simulation_project_gb300.solver import Solver
    try:
        s = Solver(scene, precision="fp32_ir", max_particles=n + 2 * bucket)
        for k in range(3):
            s.step(k)
        b = np.full((bucket, 3), 10.0, np.float32) + np.arange(bucket, dtype=np.float32)[:, None] * 1e-3
        lib.call("mps_device_sync")
        t0 = time.perf_counter()
        added = s.add_particles(b)
        t1 = time.perf_counter()
        st = s.step(3)
        lib.call("mps_device_sync")
        t2 = time.perf_counter()
        out = {"particles": n, "bucket": bucket, "added": added, "add_ms": round((t1 - t0) * 1e3, 3),
               "next_step_ms": round((t2 - t1) * 1e3, 3), "next_step_error_flags": int(st["error_flags"]),
               "particles_after_next_step": int(st["particles"])}
        s.close()
        return out
    except Exception as e:  # pragma: no cover - reported, not fatal for the metric
        return {"error": str(e)}


def frames_bench(solver, n, args, steps=10):
    """Output frames (reference format, mps_solver_save_frame) outside the timed region:
    wall time per step with and without a binary frame after every step (the pack, the
    pinned copy and the file write overlap the next steps), and the latency of one frame
    in each format.  Files go to a temporary directory."""
    import shutil
    import tempfile
    from simulation_project_gb300 import lib
    tmp = tempfile.mkdtemp(prefix="mps_frames_")
    try:
        first = 10_000
        def run(with_frames):
            lib.call("mps_device_sync")
            t0 = time.perf_counter()
            for k in range(steps):
                solver.step(first + k)
                if with_frames:
                    solver.save_frame(os.path.join(tmp, f"f{k % 2}.dat"), ascii=False, time=k * 5e-5)
            t1 = time.perf_counter()
            solver.wait_frames()   # the last frame's write, after the last step
            lib.call("mps_device_sync")
            return (t1 - t0) * 1e3 / steps, (time.perf_counter() - t1) * 1e3
        run(False)
        base, _ = run(False)
        first += steps
        with_f, tail = run(True)
        out = {"particles": n, "steps": steps, "wall_ms_per_step": round(base, 3),
               "wall_ms_per_step_binary_frame_each_step": round(with_f, 3),
               "overhead_ms_per_step": round(with_f - base, 3), "last_frame_wait_ms": round(tail, 2),
               "binary_bytes": 4 + 48 * n + 8}
        for ascii in (False, True):
            lib.call("mps_device_sync")
            t0 = time.perf_counter()
            solver.save_frame(os.path.join(tmp, "one.dat"), ascii=ascii)
            solver.wait_frames()
            out["ascii_frame_ms" if ascii else "binary_frame_ms"] = round((time.perf_counter() - t0) * 1e3, 2)
            if ascii:
                out["ascii_bytes"] = os.path.getsize(os.path.join(tmp, "one.dat"))
        return out
    except Exception as e:  # pragma: no cover - reported, not fatal for the metric
        return {"error": str(e)}
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def run_e2e(solver, args):
    from simulation_project_gb300 import lib
    n = solver.state(sort_by_id=False)["pos"].shape[0]
    # pinned host buffers
    bufs = []
    for shape in ((n, 3), (n, 3), (n,)):
        p = C.c_void_p()
        nbytes = int(np.prod(shape)) * 8
        lib.call("mps_host_alloc_pinned", C.byref(p), nbytes)
        arr = np.ctypeslib.as_array((C.c_double * int(np.prod(shape))).from_address(p.value)).reshape(shape)
        bufs.append((p, arr))
    pos, vel, press = (b[1] for b in bufs)
    solver.download_state(pos, vel, press)
    steps = max(2, args.steps // 2)
    lib.call("mps_device_sync")
    t0 = time.perf_counter()
    for i in range(steps):
        solver.upload_state(pos, vel, press)
        solver.step(1000 + i)
        solver.download_state(pos, vel, press)
    dt = time.perf_counter() - t0
    for p, _ in bufs:
        lib.call("mps_host_free_pinned", p)
    return {"value": n * steps / dt, "unit": "particle-steps/s", "h2d_bytes_per_step": n * 56,
            "d2h_bytes_per_step": n * 56, "steps": steps}


def lib_sm_count():
    """SMs of the current device (the library's runtime query), 0 if unavailable."""
    from simulation_project_gb300 import lib
    c = C.c_int(0)
    return c.value if lib.load().mps_device_sm_count(C.byref(c)) == 0 else 0


def cpu_baseline(args):
    """The FP64 oracle solver (OpenMP) on a bounded sample: the same bucket at
    l0 = 0.004 for one step after one warm-up step."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import orc
    sc = build_scene(0.004)
    sim = orc.OracleSim(sc)
    sim.step(0)
    t0 = time.perf_counter()
    sim.step(1)
    dt = time.perf_counter() - t0
    sim.close()
    return {"value": sc.n / dt, "unit": "particle-steps/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"FP64 oracle PPE step (OpenMP) on the bucket at l0=0.004 ({sc.n} particles), 1 step"}


def gpu_config(args, scene, world=1):
    """The `config` object of a bench line (the same for both arms)."""
    return {"workload": WORKLOADS[args.workload].format(l0=args.l0),
            "particles": scene.n, "triangles": scene.t, "cells": scene.box.cell_num,
            "l2": "inputs larger than L2 (neighbour rows ~8 B x nnz per SpMV)",
            "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"}


def run_reference(args):
    """The reference's explicit-schedule kernels compiled for the CPU (oracle/_ref), on
    the same scene as the GPU arm."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import orc
    ref = orc.reference()
    kind = "reference"
    if ref is None:
        ref = orc.oracle()
        kind = "port"
    sc = build_scene(args.l0, workload=args.workload)
    config = gpu_config(args, sc)
    sc.param.bExplicitPressure = True
    sc.param.SonicVelocity = 20.0
    st = orc.RefState(sc)
    b = st.bindings()

    def one_step(i):
        n = C.c_int(st.n)
        if hasattr(ref, "check_outside_compute_zone"):
            ref.check_outside_compute_zone(C.byref(b), C.byref(n))
        orc.ref_topology(ref, st, b)
        ref.reset_triangle_topology(st.cells_n, orc.ptr(st.cells))
        ref.register_triangle_topology(C.byref(b), orc.ptr(st.triangles), st.t, orc.ptr(st.cells), st.cells_n)
        ref.calc_stl_distance(C.byref(b), st.n)
        if st.drag_num:
            ref.calc_drag_effect(C.byref(b), st.n)
        ref.calc_explicitly(C.byref(b), st.n)
        orc.ref_topology(ref, st, b)
        ref.calc_stl_distance(C.byref(b), st.n)
        ref.calc_explicit_pressure(C.byref(b), st.n)
        ref.calc_explicit_pressure_gradient(C.byref(b), st.n)
        ref.update_triangle_position(C.byref(b), st.t)
        ref.rotate_triangle_position(C.byref(b), st.t, i)

    for i in range(args.warmup):
        one_step(i)
    t0 = time.perf_counter()
    for i in range(args.steps):
        one_step(args.warmup + i)
    dt = time.perf_counter() - t0
    v = st.n * args.steps / dt
    return {"impl": "reference", "metric": "particle-steps/s @1M on 1 GB300, learned-precond vs plain CG at 1e-8 "
            "PPE residual", "value": v, "unit": "particle-steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config,
            "reference_scheme": "the reference's only pressure scheme: explicit (equation of state), no PPE solve; "
                                "its kernels compiled for the host CPU, OpenMP over particles",
            "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": _threads(), "kind": kind,
                             "sample": f"reference explicit schedule (EOS pressure, its own kernels on the CPU) "
                                       f"on the GPU arm's scene ({st.n} particles), every step of the run"},
            "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def _threads():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--l0", type=float, default=0.002)
    ap.add_argument("--train-steps", type=int, default=6)
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--learned-mode", type=int, default=1, help="bit 0 initial guess, bit 1 diagonal scaling")
    ap.add_argument("--precond", type=int, default=1, help="0 Jacobi, 1 multilevel (FP32 inner solve)")
    ap.add_argument("--accuracy-steps", type=int, default=10, help="steps of the FP32-IR vs FP64 comparison")
    ap.add_argument("--accuracy-only", action="store_true", help="only the FP32-IR vs FP64 comparison")
    ap.add_argument("--workload", default="bucket", choices=sorted(WORKLOADS), help="bucket (default) or mixer")
    ap.add_argument("--profile-case", action="store_true", help="only the solver steps (for ncu captures)")
    ap.add_argument("--fp64", action="store_true", help="with --profile-case: the plain FP64 solver")
    ap.add_argument("--profile-learned", action="store_true", help="with --profile-case: train, then the learned solver")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", "0"))
    if args.profile_case:
        return run_profile_case(args)
    if args.accuracy_only:
        return run_accuracy_only(args)
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args)))
        return 0
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        # replicas: one independent bucket per GPU; gloo carries only barriers and the
        # final two numbers per rank
        import torch.distributed as dist
        dist.init_process_group("gloo")
    res = run_gpu(args)
    if world > 1:
        gather_replicas(res)
        dist.destroy_process_group()
    res.pop("units", None)
    if rank == 0:
        print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
