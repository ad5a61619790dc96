"""Benchmark of the GB300 APIC/FLIP step: particle-steps/s on the single large scene.

Workload (N=1): 1024 x 1024 MAC grid, dx = 1/1024, dam break x < 0.5, y < 0.5
at 4 particles per cell (seed 1) plus a disk of radius 0.08 at (0.7, 0.8)
moving at (0, -2); gravity -9.81, cfl 5, border damping 0.1; one step = one
Apic::update of dt = 1/480 (one frame, split into CFL substeps as the
reference does).  The pressure solve runs FP32 MG-PCG inside FP64 iterative
refinement to a true relative residual of 1e-6 (``--solver`` selects the plain
FP32 or the reference's own exits).  Inputs are synthetic (deterministic
hash-jittered particles); the state stays resident in HBM across steps.

Printed JSON line: ``value`` = particles x steps / device time of the timed
steps (CUDA events on the scene's stream, L2 flushed between steps);
``e2e`` = the same through the C-ABI with a host force field uploaded from
pinned memory and the particle state read back every step (pipelined: the
copies of neighbouring steps overlap the updates); ``roofline`` for
the pressure solve (the dominant part of a step, timed inside the update
graph by the device's global timer), ``cpu_baseline`` = the C++ restatement
of the reference step (OpenMP, all host cores) over the same updates;
``batched_config4`` = a brief run of 256 uneven scenes through
apic_update_batch (``--workload batched`` in a child process).

``--impl reference`` times that CPU restatement alone as the reference arm.
Under torchrun (N > 1) each rank runs an independent replica on its own GPU
(the single-scene path does not shard), rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "apic-fluid-simulation_gb300"))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s"
UNIT_NOTE = ("1 particle-step = 1 particle through one CFL substep of the update pipeline; an update of dt "
             "splits into substeps by the CFL condition (updates_per_s is reported beside)")
SIDE = 1024
FRAME_DT = 1.0 / 480.0
STRESS = False  # --workload stress: config 3 instead of the 1024^2 scene
NOISE_PERIOD = 1.0 / 64.0  # value-noise lattice period of config 3 (domain units)


def scene_params(A, side=SIDE):
    if STRESS:
        # config 3: value-noise mask > 0.5 (seed 2), 4 ppc, v ~ N(0, 0.5^2) per component
        return A.scene_params(A.SCENE_NOISE, side, cell_size=1.0 / side, sub=2, seed=2,
                              noise_period=NOISE_PERIOD, noise_threshold=0.5, vel_sigma=0.5)
    return A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=1.0 / side, sub=2, seed=1, fluid_x=0.5,
                          fluid_y=0.5, disk=(0.7, 0.8, 0.08), disk_v=(0.0, -2.0))


def workload_name(side):
    if STRESS:
        return (f"stress: value-noise fluid mask > 0.5 (period {NOISE_PERIOD:g}, seed 2), {side}x{side} MAC grid, "
                f"dx=1/{side}, 4 ppc, v ~ N(0, 0.5^2), dt=1/1000 per step, Morton sort every step")
    return f"dam break + disk, {side}x{side} MAC grid, dx=1/{side}, 4 ppc, seed 1, dt=1/480 per step"


def props(A):
    return A.WorldProperties(gravity=-9.81, border_damping=0.1, cfl=5.0, solve_error=1e-5)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.rows = []
        if self.proc is None:
            return
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def summary(self):
        rows = getattr(self, "rows", [])
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank, local


def dist_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    # NCCL reduces device tensors; gloo (CPU-only runs) host tensors
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def place_on_ranks(A, scenes, world, budget_bytes):
    """Device (rank) of each independent scene: apic_place_scenes with each
    GPU's memory budget; every rank computes the same placement, so no
    exchange is needed before the run."""
    counts = [A.scene_count(sc) for sc in scenes]
    sizes = [A.scene_bytes(sc.width, sc.height, n) for sc, n in zip(scenes, counts)]
    return A.place_scenes(sizes, counts, [budget_bytes] * world)


def dist_barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------- CPU arm --
def cpu_restatement_rate(n_steps: int, warmup: int, budget_s: float, side: int = 0, threads: int = 0):
    """Particle-steps/s of the C++ restatement of the reference step (OpenMP).

    Only the oracle's library is loaded (it carries the benchmark scenes'
    particle generator too); apic_gb300 supplies plain Python parameter types."""
    import apic_gb300 as A
    side = side or SIDE  # SIDE is read at call time: --workload stress changes it
    from oracle.oracle import OracleSim, generate_scene
    threads = threads or os.cpu_count() or 1
    px, py, vx, vy = generate_scene(scene_params(A, side))
    o = OracleSim(side, side, 1.0 / side, props(A), threads=threads)
    o.set_particles(px, py, vx, vy)
    o.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
    opts = A.DebugOptions()
    for _ in range(warmup):
        o.update(opts, FRAME_DT)
    times, substeps = [], 0
    t_start = time.perf_counter()
    for _ in range(n_steps):
        t0 = time.perf_counter()
        o.update(opts, FRAME_DT)
        times.append(time.perf_counter() - t0)
        substeps += o.stats().substeps
        if time.perf_counter() - t_start > budget_s:
            break
    n = len(px)
    total = sum(times)
    return {"value": n * substeps / total, "steps": len(times), "substeps": substeps,
            "updates_per_s": len(times) / total, "seconds": total, "threads": threads,
            "particles": n, "ms_per_step": 1e3 * total / len(times),
            "p50_ms": 1e3 * float(np.percentile(times, 50)), "p99_ms": 1e3 * float(np.percentile(times, 99))}


def run_reference_arm(args, world, rank):
    if rank != 0:
        return
    r = cpu_restatement_rate(args.steps, args.warmup, budget_s=150.0)
    line = {
        "impl": "reference", "metric": METRIC, "value": r["value"], "unit": METRIC, "n_gpus": args.gpus,
        "steps": r["steps"], "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(SIDE), "particles": r["particles"], "substeps": r["substeps"],
                   "unit": UNIT_NOTE, "solver": "FP32 MG-PCG + FP64 refinement to 1e-6"},
        "updates_per_s": r["updates_per_s"],
        "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"],
        "cpu_baseline": {"value": r["value"], "unit": METRIC, "cores": r["threads"], "kind": "port",
                         "sample": f"{r['steps']} updates after {args.warmup} warm-up updates from t=0"},
        "e2e": {"value": r["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU arm --
def level_fluid_counts(A, sim):
    info = sim.info()
    counts = [info.fluid_cells]
    for lvl in range(info.mg_levels):
        bits = sim.read_field(A.mg_field("fluid_bits", lvl))
        counts.append(int(np.unpackbits(bits.view(np.uint8)).sum()))
    return counts


def run_gpu_arm(args, world, rank, local):
    import apic_gb300 as A
    from apic_gb300 import build as gpu_build
    gpu_build.build()
    import torch

    dev = local
    torch.cuda.set_device(dev)
    px, py, vx, vy = A.generate_scene(scene_params(A, args.side))
    n = len(px)
    sim = A.Apic(args.side, args.side, 1.0 / args.side, props(A))
    sim.set_particles(px, py, vx, vy)
    mode = {"mixed": A.SOLVER_REL_MIXED, "fp32": A.SOLVER_REL_FP32, "reference": A.SOLVER_REFERENCE}[args.solver]
    sim.set_solver(mode, 1e-6, 500)
    if args.no_pdl:
        sim.set_option(A.OPT_PDL, 0)
    if args.no_dsm:
        sim.set_option(A.OPT_DSM_VCYCLE, 0)
    dsm = sim.get_option(A.OPT_DSM_VCYCLE)
    opts = A.DebugOptions()
    stream_ptr = ctypes_stream(sim)
    ext_stream = torch.cuda.ExternalStream(stream_ptr)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > 129 MB L2

    for _ in range(args.warmup):
        sim.update(opts, FRAME_DT)
    sim.synchronize()

    # ---- timed region: K updates, device time per update, L2 flushed in between
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    substeps, iters, launches, solve_ms = 0, 0, 0, 0.0
    true_res = []
    if args.eager:  # stage-by-stage launches (what an ncu launch list can see)
        sim.set_profiling(True)
    dist_barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(dev) as clocks:
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            starts[k].record(ext_stream)
            sim.update(opts, FRAME_DT)
            ends[k].record(ext_stream)
            st = sim.stats()
            substeps += st.substeps
            iters += st.pcg_iterations_total
            launches += st.kernel_launches
            solve_ms += st.solve_ms
            true_res.append(st.true_residual_rel)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    dist_barrier(world)
    if args.eager:
        sim.set_profiling(False)
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    dev_s = sum(step_ms) / 1e3
    dev_s_max = dist_max(dev_s, world)
    value = world * n * substeps / dev_s_max  # substeps: summed over the timed updates (same on every replica)

    # ---- e2e through the C-ABI with host buffers (pinned), copies inside the
    # timed region: a second scene from the same start, over the same updates
    # (warm-up updates, then the timed ones), so e2e and value cover the same
    # part of the flow
    sim2 = A.Apic(args.side, args.side, 1.0 / args.side, props(A))
    sim2.set_particles(px, py, vx, vy)
    sim2.set_solver(mode, 1e-6, 500)
    for opt in (A.OPT_PDL, A.OPT_DSM_VCYCLE):
        v = sim.get_option(opt)
        if sim2.get_option(opt) != v:
            sim2.set_option(opt, v)
    for _ in range(args.warmup):
        sim2.update(opts, FRAME_DT)
    fu = torch.zeros(sim2.field_shape(A.FIELDS["ext_force_u"])[0], dtype=torch.float32).pin_memory()
    fv = torch.zeros(sim2.field_shape(A.FIELDS["ext_force_v"])[0], dtype=torch.float32).pin_memory()
    nc = sim2.num_chunks
    # one destination per step and field pair (a result is kept, not overwritten)
    pos_h = [torch.empty(nc * 16, dtype=torch.float32).pin_memory() for _ in range(2)]
    vel_h = [torch.empty(nc * 16, dtype=torch.float32).pin_memory() for _ in range(2)]
    e2e_steps = args.steps
    torch.cuda.synchronize()
    dist_barrier(world)
    te = time.perf_counter()
    e2e_sub = 0
    # pipelined through the C-ABI: step k+1's forces are uploaded and step k's
    # particles read back while step k+1 / step k run (apic_stage_field,
    # apic_update_async / apic_update_wait, apic_read_vec2x8_async)
    sim2.stage_field("ext_force_u", fu.data_ptr(), fu.numel() * 4)
    sim2.stage_field("ext_force_v", fv.data_ptr(), fv.numel() * 4)
    for k in range(e2e_steps):
        sim2.update_async(opts, FRAME_DT)
        if k >= 2:
            sim2.read_wait()  # step k-2's read-back landed: its host buffers are reused now
        sim2.read_vec2x8_async(0, pos_h[k % 2].data_ptr(), nc * 16)
        sim2.read_vec2x8_async(1, vel_h[k % 2].data_ptr(), nc * 16)
        if k + 1 < e2e_steps:
            sim2.stage_field("ext_force_u", fu.data_ptr(), fu.numel() * 4)
            sim2.stage_field("ext_force_v", fv.data_ptr(), fv.numel() * 4)
        sim2.update_wait()
        e2e_sub += sim2.stats().substeps
    sim2.read_wait()
    e2e_s = dist_max(time.perf_counter() - te, world)
    e2e_value = world * n * e2e_sub / e2e_s
    h2d = (fu.numel() + fv.numel()) * 4
    d2h = 2 * nc * 16 * 4
    sim2.close()

    # ---- per-stage device times (events around each stage) for the roofline
    sim.set_profiling(True)
    sim.reset_stage_times()
    prof_steps = max(1, min(args.steps, 5))
    prof_sub = 0
    prof_iters = 0
    for _ in range(prof_steps):
        sim.update(opts, FRAME_DT)
        prof_sub += sim.stats().substeps
        prof_iters += sim.stats().pcg_iterations_total
    stages = sim.stage_times()
    sim.set_profiling(False)
    counts = level_fluid_counts(A, sim)
    peak, peak_kind = peaks()
    roof = roofline(iters, solve_ms, args.steps, counts, peak, peak_kind) if solve_ms > 0 and not args.eager else None
    if roof is not None:
        l2 = l2_copy_gbs(torch)
        roof["l2"] = {"copy_gbs_measured": l2, "frac": roof["achieved"] / l2,
                      "how": "the same algorithmic bytes per second against a device copy of a 32 MiB buffer "
                             "into another (64 MiB working set, resident in the 129 MB L2; read + write bytes, "
                             "best of 20 repetitions, CUDA events)"}
    compare = None
    if args.solver == "mixed" and not args.no_solver_compare and not args.eager:
        compare = solver_compare(A, torch, args, px, py, vx, vy, mode)
    batched = None
    if rank == 0 and world == 1 and not args.eager and not args.no_batched_summary:
        batched = batched_summary()

    result = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline and world == 1:
            # the same updates as the timed GPU region: warm-up updates, then the timed ones
            c = cpu_restatement_rate(n_steps=args.cpu_steps or args.steps, warmup=args.warmup,
                                     budget_s=args.cpu_budget, side=args.side)
            cpu = {"value": c["value"], "unit": METRIC, "cores": c["threads"], "kind": "port",
                   "sample": f"C++ restatement of the reference step (OpenMP, {c['threads']} threads), updates "
                             f"{args.warmup + 1}..{args.warmup + c['steps']} of the same scene (the GPU's timed "
                             f"updates), {c['seconds']:.1f} s"}
        result = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dev_s_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_name(args.side), "particles": n,
                       "solver": {"mixed": "FP32 MG-PCG + FP64 refinement, true rel. residual <= 1e-6",
                                  "fp32": "FP32 MG-PCG to recursive rel. residual 1e-6",
                                  "reference": "reference exits (max|r| < 1e-5, 100 iterations)"}[args.solver],
                       "unit": UNIT_NOTE, "substeps": substeps, "pcg_iterations": iters,
                       "true_residual_rel_max": max(true_res) if true_res else None,
                       "l2": "flushed (256 MB write) between timed steps", "parallelism": f"replicas x{world}",
                       "solve_form": "graph of per-phase kernels",
                       "vcycle": "one kernel per sweep and transfer" + (
                           "; coarse levels in one cluster's distributed shared memory" if dsm else ""),
                       "launch": ("stage by stage" if args.eager else "one CUDA graph per update")
                       + ("" if args.no_pdl else "; programmatic dependent launch in the PCG loop")},
            "updates_per_s": world * args.steps / dev_s_max,
            "p50_ms": float(np.percentile(step_ms, 50)), "p99_ms": float(np.percentile(step_ms, 99)),
            "wall_s": wall,
            "clocks": clocks.summary(),
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": e2e_steps,
                    "what": "every step: the ext force fields u, v uploaded from pinned host memory "
                            "(apic_stage_field), apic_update_async + apic_update_wait, positions and velocities "
                            "read back to pinned host memory (apic_read_vec2x8_async, all landed before the "
                            "clock stops); pipelined: step k+1's upload and step k's read-back overlap the "
                            "updates; wall clock, on a second scene over the same updates as the timed region"},
            "gpu_launches": launches if not args.eager else None,
            "roofline": roof,
            "solver_compare": compare,
            "batched_config4": batched,
            "stage_ms_profiling": {
                "note": "profiling mode, not additive to ms_per_step: each stage of each substep launched on "
                        "its own between CUDA events and the solve's loops driven from the host (every PCG "
                        "iteration pays host round trips the update graph does not); for the split between "
                        "stages, not their sum",
                "ms_per_step": {k: v[0] / prof_steps for k, v in stages.items() if v[1]}},
            "cpu_baseline": cpu,
        }
        print(json.dumps(result), flush=True)
    sim.close()
    return result


def batched_summary() -> dict:
    """Config 4 in brief, beside the single-scene line: 256 uneven scenes
    through apic_update_batch as tuned, against the same updates one scene at
    a time and with every scene on its own stream (bench.py --workload
    batched in a child process, so that CUDA_DEVICE_MAX_CONNECTIONS=32 holds
    for it from CUDA's start)."""
    cmd = [sys.executable, os.path.abspath(__file__), "--workload", "batched", "--steps", "5", "--compare-steps", "3"]
    env = dict(os.environ, CUDA_DEVICE_MAX_CONNECTIONS="32")
    try:
        out = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=600)
        line = json.loads(out.stdout.strip().splitlines()[-1])
    except Exception as e:  # the summary is evidence beside the headline, never a reason to lose it
        return {"error": f"{type(e).__name__}: {str(e)[:300]}"}
    keep = ("value", "unit", "batched_vs_plain", "round_ms_p50", "round_ms_p99", "gpu_launches", "clocks",
            "true_residual_rel_max")
    res = {k: line.get(k) for k in keep}
    res["config"] = {k: line["config"].get(k) for k in ("workload", "particles", "sides_min_median_max", "batching",
                                                        "tuner", "cuda_device_max_connections")}
    res["command"] = " ".join(["python", "bench.py"] + cmd[2:])
    return res


def ctypes_stream(sim) -> int:
    import ctypes
    out = ctypes.c_void_p()
    sim._lib.apic_get_stream(sim._h, ctypes.byref(out))
    return int(out.value or 0)


# Algorithmic bytes of one PCG iteration per fluid cell (each array read or
# written once per pass; neighbour reads hit cached lines): 132 B per base
# fluid cell for the SpMV with its dot product, the pressure/residual update,
# the SOR pre- and post-smoothing, restriction, prolongation, r.z and the
# search update; 76 B per coarse fluid cell (pre-smoothing 24, restriction
# 20, prolongation 8, post-smoothing 24).  The coarse tail and the coarsest
# CG run in shared memory and are not counted.
SOLVE_BYTES_BASE = 132
SOLVE_BYTES_COARSE = 76


def l2_copy_gbs(torch) -> float:
    """Device copy bandwidth with an L2-resident working set (GB/s, read + write)."""
    n = 32 * 1024 * 1024 // 4
    a = torch.ones(n, dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    for _ in range(5):
        b.copy_(a)
    best = None
    for _ in range(20):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            b.copy_(a)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / 10
        best = t if best is None else min(best, t)
    return 2 * n * 4 / best / 1e9


def solver_compare(A, torch, args, px, py, vx, vy, mixed_mode):
    """The plain FP32 solve (PCG on the recursive residual, tolerance 1e-6)
    beside the mixed-precision one on the same scene and updates: device ms
    per update, PCG iterations and the true relative residual (FP64) each
    reaches."""
    out = {}
    for name, mode in (("plain_fp32", A.SOLVER_REL_FP32), ("mixed", mixed_mode)):
        g = A.Apic(args.side, args.side, 1.0 / args.side, props(A))
        g.set_particles(px, py, vx, vy)
        g.set_solver(mode, 1e-6, 500)
        opts = A.DebugOptions()
        for _ in range(args.warmup):
            g.update(opts, FRAME_DT)
        g.synchronize()
        st_ptr = torch.cuda.ExternalStream(ctypes_stream(g))
        steps = min(args.steps, 10)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        iters, res, notc, sub, solve = 0, [], 0, 0, 0.0
        e0.record(st_ptr)
        for _ in range(steps):
            g.update(opts, FRAME_DT)
            st = g.stats()
            iters += st.pcg_iterations_total
            res.append(float(st.true_residual_rel))
            notc += st.not_converged
            sub += st.substeps
            solve += st.solve_ms
        e1.record(st_ptr)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[name] = {"ms_per_update": ms, "solve_ms_per_update": solve / steps, "pcg_iterations": iters,
                     "substeps": sub, "true_residual_rel_max": max(res), "true_residual_rel_min": min(res),
                     "substeps_not_converged": notc, "updates": steps}
        g.close()
    out["note"] = ("both asked for relative residual 1e-6 with at most 500 iterations; the plain FP32 PCG stops on "
                   "its recursive residual, whose true value (FP64, reported) stays far above 1e-6 because FP32 "
                   "rounding of the pressure limits it; the mixed solve refines in FP64 until the true residual "
                   "is below 1e-6 (updates after the same warm-up, L2 not flushed)")
    return out


def solve_traffic():
    """DRAM bytes per PCG iteration from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "solve_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_iteration"])
    except (OSError, KeyError, ValueError):
        return None


def roofline(iters, solve_ms, steps, counts, peak, peak_kind):
    """Roofline of the pressure solve, the dominant part of a step.

    The solve is a CUDA graph of per-phase kernels inside device-side WHILE
    loops, so CUDA events cannot bracket it; its first and last kernels read
    the GPU's global nanosecond timer instead (apic_step_stats.solve_ms),
    summed here over the timed updates.  achieved = algorithmic bytes of the
    iterations run / that time.
    """
    f0 = counts[0]
    fl = sum(counts[1:])
    per_iter = SOLVE_BYTES_BASE * f0 + SOLVE_BYTES_COARSE * fl
    sec = solve_ms / 1e3
    achieved = per_iter * iters / sec / 1e9
    traffic = solve_traffic()
    return {"bound": "hbm", "kernel": "pressure solve: MG-preconditioned CG (per iteration k_spmv_dot, "
                                      "k_pcg_update, k_smooth_exit, the V-cycle's sweep and transfer kernels, "
                                      "k_vcycle_dsm, k_prolong_red_rz)",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
            "traffic": traffic, "traffic_unit": "DRAM bytes per PCG iteration" if traffic else None,
            "algorithmic_bytes_per_iteration": per_iter, "iterations": iters,
            "us_per_iteration": solve_ms * 1e3 / max(iters, 1), "solve_ms_per_step": solve_ms / steps}


# ---------------------------------------------------------- batched / served --
def batched_scenes(A, count, seed=3, lo=64, hi=512):
    """Config 4: sides log-uniform in [lo, hi] rounded to a multiple of 8, dam
    break filling a square of a uniform [0.2, 0.6] share of the domain, 4 ppc."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        side = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi))) / 8.0)) * 8
        f = float(np.sqrt(rng.uniform(0.2, 0.6)))
        out.append(A.scene_params(A.SCENE_DAM_BREAK, side, cell_size=1.0 / side, sub=2, seed=seed * 100000 + i,
                                  fluid_x=f, fluid_y=f))
    return out


def make_sims(A, scenes, dsm=True):
    sims = []
    for sc in scenes:
        g = A.Apic(sc.width, sc.height, sc.cell_size, props(A))
        px, py, vx, vy = A.generate_scene(sc)
        g.set_particles(px, py, vx, vy)
        g.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
        if not dsm:
            g.set_option(A.OPT_DSM_VCYCLE, 0)
        sims.append(g)
    return sims


def run_batched(args, world=1, rank=0, local=0):
    """Config 4: many uneven scenes, one batched update per round, against the
    plain path (one scene's update after another) over the same updates.
    Under torchrun the scenes are placed on the ranks' GPUs by
    apic_place_scenes (memory budget per GPU, least-loaded first); each rank
    runs its own scenes, with no collective on the data path, and rank 0
    reports the summed particle-substeps over the slowest rank's time."""
    import apic_gb300 as A
    from apic_gb300 import build as gpu_build
    gpu_build.build()
    import torch
    torch.cuda.set_device(local)
    scenes = batched_scenes(A, args.scenes)
    placement = None
    if world > 1:
        where = place_on_ranks(A, scenes, world, int(args.budget_gb * (1 << 30)))
        if any(d < 0 for d in where):
            raise SystemExit("a scene fits no GPU's budget")
        placement = [where.count(r) for r in range(world)]
        scenes = [sc for sc, d in zip(scenes, where) if d == rank]
    dt = 1.0 / 240.0
    # plain: fresh scenes, the first `cmp` updates one scene at a time
    cmp_steps = args.compare_steps
    sims = make_sims(A, scenes, not args.no_dsm)
    counts = [g.num_particles for g in sims]
    n_tot = sum(counts)
    for g in sims:  # warm-up: graph capture and first-touch of every scene
        g.update(A.DebugOptions(), dt)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sub_plain = 0
    for _ in range(cmp_steps):
        for g, n in zip(sims, counts):
            g.update(A.DebugOptions(), dt)
            sub_plain += n * g.stats().substeps
    plain_s = time.perf_counter() - t0
    for g in sims:
        g.close()
    # the stream-per-scene batch: fresh scenes, the same updates
    sims = make_sims(A, scenes, not args.no_dsm)
    A.update_batch(sims, A.DebugOptions(), dt, streams=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sub_streams = 0
    for _ in range(cmp_steps):
        A.update_batch(sims, A.DebugOptions(), dt, streams=True)
        sub_streams += sum(n * g.stats().substeps for g, n in zip(sims, counts))
    streams_s = time.perf_counter() - t0
    # the library's batch tuner settles on a form for this makeup of scenes
    # (on these scenes' further updates; untimed)
    tune_calls = 0
    while tune_calls < 40:
        A.update_batch(sims, A.DebugOptions(), dt)
        tune_calls += 1
        if A.batch_last_info()["tuned"]:
            break
    for g in sims:
        g.close()
    # the tuned batch: fresh scenes, the same updates, then the rest of the
    # run; the first call builds its graph
    sims = make_sims(A, scenes, not args.no_dsm)
    A.update_batch(sims, A.DebugOptions(), dt)
    chosen = A.batch_last_info()
    joint = chosen["joint"]
    torch.cuda.synchronize()
    round_ms, sub_cmp, sub_all, res_max, kern_all = [], 0, 0, 0.0, 0
    with ClockSampler(0) as clocks:
        t0 = time.perf_counter()
        for k in range(args.steps):
            tr = time.perf_counter()
            A.update_batch(sims, A.DebugOptions(), dt)
            round_ms.append((time.perf_counter() - tr) * 1e3)
            stats = [g.stats() for g in sims]
            sub = sum(n * st.substeps for n, st in zip(counts, stats))
            res_max = max(res_max, max(float(st.true_residual_rel) for st in stats))
            info = A.batch_last_info()
            kern_all += sum(int(st.kernel_launches) for st in stats) + int(info["batch_kernel_launches"])
            sub_all += sub
            if k < cmp_steps:
                sub_cmp += sub
                if k == cmp_steps - 1:
                    cmp_s = time.perf_counter() - t0
        all_s = time.perf_counter() - t0
    # every rank ran its own scenes: totals summed, times of the slowest rank
    sub_all, sub_cmp, sub_plain = dist_sum(sub_all, world), dist_sum(sub_cmp, world), dist_sum(sub_plain, world)
    all_s, cmp_s, plain_s = dist_max(all_s, world), dist_max(cmp_s, world), dist_max(plain_s, world)
    sub_streams, streams_s = dist_sum(sub_streams, world), dist_max(streams_s, world)
    kern_all, n_tot = int(dist_sum(kern_all, world)), int(dist_sum(n_tot, world))
    res_max = dist_max(res_max, world)
    if rank != 0:
        for g in sims:
            g.close()
        return
    sides = [sc.width for sc in batched_scenes(A, args.scenes)]
    line = {
        "metric": METRIC, "value": sub_all / all_s, "unit": "particle-substeps/s (aggregate over all scenes)",
        "workload": "batched", "n_gpus": world, "steps": args.steps, "higher_is_better": True,
        "scaling": "strong" if world > 1 else None,
        "placement": None if placement is None else {
            "scenes_per_gpu": placement, "how": "apic_place_scenes: largest first, least-loaded GPU whose "
                                               "memory budget holds the scene; no collective on the data path"},
        "config": {"workload": f"{len(scenes)} independent dam-break scenes, side log-uniform in [64, 512] "
                               f"(rounded to x8, seed 3), fluid share U[0.2, 0.6], 4 ppc, dt=1/240, "
                               f"mixed-precision PCG to true rel. residual 1e-6",
                   "particles": n_tot, "sides_min_median_max": [min(sides), int(np.median(sides)), max(sides)],
                   "batching": ("apic_update_batch, joint: one graph per batch; every scene's stages before "
                                "and after the pressure solve are its own kernels, the pressure solves of all "
                                "scenes run as one launch per solve phase over a scene table")
                               if joint else "apic_update_batch: every scene's update on its own stream",
                   "tuner": {"calls": tune_calls, "joint": int(chosen["joint"]), "chunk_segs": chosen["chunk_segs"],
                             "block_group": chosen["block_group"],
                             "how": "the library's batch tuner: the first calls for this makeup of scenes try the "
                                    "stream-per-scene form and the joint form with 12 shapes, each twice, cost = "
                                    "wall time per PCG iteration over all scenes; the lowest mean cost is kept"},
                   "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS", "8 (default)"),
                   "dsm_vcycle": not args.no_dsm},
        "batched_vs_plain": {"updates_compared": cmp_steps, "batched": sub_cmp / cmp_s, "plain": sub_plain / plain_s,
                             "ratio": (sub_cmp / cmp_s) / (sub_plain / plain_s),
                             "plain_is": "the same scenes' updates one after another through apic_update",
                             "streams": sub_streams / streams_s,
                             "streams_is": "the same updates batched with every scene's whole update on its own "
                                           "stream (APIC_UPDATE_BATCH_STREAMS)"},
        "round_ms_p50": float(np.percentile(round_ms, 50)), "round_ms_p99": float(np.percentile(round_ms, 99)),
        "last_round": info,
        "gpu_launches": kern_all, "kernels_per_s": kern_all / all_s,
        "true_residual_rel_max": res_max, "clocks": clocks.summary(), "data": "synthetic",
    }
    print(json.dumps(line), flush=True)
    for g in sims:
        g.close()


def served_stream(A, rate, seconds, seed=4, lo=64, hi=1024):
    """Config 5: Poisson arrivals; side log-uniform in [lo, hi] (even, x8),
    steps U[20, 200], dam break or disk drop 50/50, 4 ppc."""
    rng = np.random.default_rng(seed)
    t, out, i = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        side = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi))) / 8.0)) * 8
        steps = int(rng.integers(20, 201))
        if rng.uniform() < 0.5:
            f = float(np.sqrt(rng.uniform(0.2, 0.6)))
            sc = A.scene_params(A.SCENE_DAM_BREAK, side, cell_size=1.0 / side, sub=2, seed=seed * 100000 + i,
                                fluid_x=f, fluid_y=f)
        else:
            sc = A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=1.0 / side, sub=2, seed=seed * 100000 + i,
                                fluid_x=0.4, fluid_y=0.3, disk=(0.7, 0.75, 0.08), disk_v=(0.0, -2.0))
        out.append((t, sc, steps))
        i += 1
    return out


def parse_scene_options(A, specs):
    """--scene-option NAME=VALUE[@[MIN_CELLS:]MAX_CELLS]: (option, value, min_cells, max_cells)."""
    out = []
    for spec in specs or []:
        name, rest = spec.split("=", 1)
        value, _, cells = rest.partition("@")
        lo, hi = 0, (1 << 64) - 1
        if cells:
            a, sep, b = cells.partition(":")
            lo, hi = (int(a), int(b)) if sep else (0, int(a))
        out.append((getattr(A, "OPT_" + name.upper()), int(value), lo, hi))
    return out


def serve_stream(A, stream, budget, max_active, dt, time_limit, mode, threads, rules=(), max_cells=0):
    sv = A.Server(budget, max_active, mode=mode, prepare_threads=threads)
    sv.set_work_limit(max_cells)
    for opt, value, lo, hi in rules:
        sv.scene_option(opt, value, lo, hi)
    t0 = time.perf_counter()
    nxt = 0
    while True:
        now = time.perf_counter() - t0
        while nxt < len(stream) and stream[nxt][0] <= now:
            sv.submit(stream[nxt][1], props(A), stream[nxt][2], dt)
            nxt += 1
        rd = sv.step()
        if rd.active == 0 and rd.queued == 0:
            if nxt >= len(stream):
                break
            time.sleep(max(0.0, min(stream[nxt][0] - (time.perf_counter() - t0), 0.01)))
        if time.perf_counter() - t0 > time_limit:
            break
    st = sv.stats()
    sv.close()
    return st, nxt


def run_served(args):
    """Config 5: the continuous-batching server on a Poisson request stream,
    against the plain path (one scene at a time: max_active = 1)."""
    import apic_gb300 as A
    from apic_gb300 import build as gpu_build
    gpu_build.build()
    import torch
    torch.cuda.set_device(0)
    stream = served_stream(A, args.rate, args.seconds, hi=args.served_max_side)
    budget = int(args.budget_gb * (1 << 30))
    dt = 1.0 / 240.0
    res = {}
    rules = parse_scene_options(A, args.scene_option)
    cells = args.max_active_cells
    arms = [("served", args.max_active, A.SERVER_CONTINUOUS, args.prepare_threads, rules, cells)]
    if args.served_rounds:
        arms.append(("served_rounds", args.max_active, A.SERVER_ROUNDS, 0, rules, cells))
    if not args.no_plain:
        arms.append(("plain", 1, A.SERVER_ROUNDS, 0, (), 0))
    for name, active, mode, threads, arm_rules, arm_cells in arms:
        st, n_sub = serve_stream(A, stream, budget, active, dt, args.time_limit, mode, threads, arm_rules,
                                 arm_cells)
        res[name] = {"particle_substeps_per_s": st.particle_substeps / (st.elapsed_ms / 1e3),
                     "requests_submitted": n_sub, "requests_completed": st.completed, "failed": st.failed,
                     "updates": st.updates, "kernel_launches": st.kernel_launches,
                     "kernels_per_s": st.kernel_launches / (st.elapsed_ms / 1e3),
                     "step_p50_ms": st.step_p50_ms, "step_p99_ms": st.step_p99_ms,
                     "request_p50_ms": st.request_p50_ms, "request_p99_ms": st.request_p99_ms,
                     "memory_peak_gb": st.memory_peak / (1 << 30), "elapsed_s": st.elapsed_ms / 1e3,
                     "busy_s": st.busy_ms / 1e3, "prepare_s": st.prepare_ms / 1e3, "host_s": st.host_ms / 1e3,
                     "max_active": active, "max_active_cells": arm_cells,
                     "mode": "continuous" if mode == A.SERVER_CONTINUOUS else "rounds",
                     "prepare_threads": threads}
    line = {
        "metric": METRIC, "value": res["served"]["particle_substeps_per_s"],
        "unit": "particle-substeps/s (aggregate)", "workload": "served", "n_gpus": 1, "higher_is_better": True,
        "config": {"workload": f"Poisson arrivals at {args.rate}/s for {args.seconds} s (seed 4), side log-uniform "
                               f"in [64, {args.served_max_side}] (x8), steps U[20, 200], dam break or disk drop 50/50, 4 ppc, "
                               f"dt=1/240, mixed-precision PCG to 1e-6, budget {args.budget_gb} GB",
                   "time_limit_s": args.time_limit, "scene_options": args.scene_option or [],
                   "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS", "8 (default)")},
        **res,
        "ratio": (res["served"]["particle_substeps_per_s"] / max(res["plain"]["particle_substeps_per_s"], 1e-9)
                  if "plain" in res else None),
        "data": "synthetic",
    }
    print(json.dumps(line), flush=True)


def run_criterion(args):
    """The reference's own benchmark shape (benches/fluid_benchmark.rs:5-41):
    Apic::new(size, size, 1.0) with its default particle block for sizes
    64..1024, 15 warm-up update(0.016) calls, then timed update(0.016) calls,
    through the C-ABI (apic_update returns after the update, as Apic::update
    does); the CPU restatement runs the same sequence per size."""
    import apic_gb300 as A
    from apic_gb300 import build as gpu_build
    from oracle.oracle import OracleSim
    gpu_build.build()
    import torch
    torch.cuda.set_device(0)
    dt, warm = 0.016, 15
    solver = {"reference": A.SOLVER_REFERENCE, "fp32": A.SOLVER_REL_FP32, "mixed": A.SOLVER_REL_MIXED}[
        args.criterion_solver]
    threads = os.cpu_count() or 1
    rows = []
    with ClockSampler(0) as clocks:
        for size in (64, 128, 256, 512, 1024):
            g = A.Apic(size, size, 1.0, props(A))
            g.set_solver(solver, 1e-6, 500 if solver != A.SOLVER_REFERENCE else 100)
            n = g.num_particles
            for _ in range(warm):
                g.update(A.DebugOptions(), dt)
            g.synchronize()
            wall, sub = [], 0
            for _ in range(args.steps):
                t0 = time.perf_counter()
                g.update(A.DebugOptions(), dt)
                wall.append(time.perf_counter() - t0)
                sub += g.stats().substeps
            g.close()
            row = {"size": f"{size}x{size}", "particles": n, "gpu_ms_mean": 1e3 * float(np.mean(wall)),
                   "gpu_ms_p50": 1e3 * float(np.percentile(wall, 50)),
                   "gpu_particle_steps_per_s": n * sub / sum(wall), "substeps": sub}
            if not args.no_cpu_baseline:
                px, py, vx, vy = A.generate_scene(A.scene_params(A.SCENE_REFERENCE_DEFAULT, size, size,
                                                                 cell_size=1.0))
                o = OracleSim(size, size, 1.0, props(A), threads=threads)
                o.set_particles(px, py, vx, vy)
                o.set_solver(solver, 1e-6, 500 if solver != A.SOLVER_REFERENCE else 100)
                for _ in range(warm):
                    o.update(A.DebugOptions(), dt)
                ct, csub, t_start = [], 0, time.perf_counter()
                for _ in range(args.steps):
                    t0 = time.perf_counter()
                    o.update(A.DebugOptions(), dt)
                    ct.append(time.perf_counter() - t0)
                    csub += o.stats().substeps
                    if time.perf_counter() - t_start > args.cpu_budget / 5:
                        break
                o.close()
                row.update({"cpu_ms_mean": 1e3 * float(np.mean(ct)), "cpu_updates": len(ct),
                            "cpu_particle_steps_per_s": n * csub / sum(ct),
                            "gpu_vs_cpu": (n * sub / sum(wall)) / (n * csub / sum(ct))})
            rows.append(row)
    last = rows[-1]
    line = {
        "metric": METRIC, "value": last["gpu_particle_steps_per_s"], "unit": METRIC, "workload": "criterion",
        "n_gpus": 1, "steps": args.steps, "warmup": warm, "higher_is_better": True, "data": "synthetic",
        "config": {"workload": "benches/fluid_benchmark.rs shape: Apic::new(size, size, 1.0) default particle "
                               "block, gravity -9.81, damping 0.1, cfl 5, 15 warm-up update(0.016), timed "
                               "update(0.016); value = the 1024x1024 case",
                   "solver": args.criterion_solver, "unit": UNIT_NOTE,
                   "cpu": f"C++ restatement, OpenMP {threads} threads" if not args.no_cpu_baseline else None,
                   "timing": "wall clock per apic_update call (returns when the update is done)"},
        "sizes": rows, "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def run_render(args):
    """The headless particle view (render_particles, src/main.rs:207-277) of the
    1024^2 bench scene after its warm-up updates: 1.13 M particles splatted
    into a 1920 x 1080 RGBA8 frame (the domain fills the frame's height)."""
    import apic_gb300 as A
    from apic_gb300 import build as gpu_build
    from oracle import oracle as O
    gpu_build.build()
    import torch
    torch.cuda.set_device(0)
    side = args.side
    sim = A.Apic(side, side, 1.0 / side, props(A))
    px, py, vx, vy = A.generate_scene(scene_params(A, side))
    sim.set_particles(px, py, vx, vy)
    sim.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
    for _ in range(args.warmup):
        sim.update(A.DebugOptions(), FRAME_DT)
    n = sim.num_particles
    rp = A.render_params(width=1920, height=1080, scale=1080.0)
    ext = torch.cuda.ExternalStream(ctypes_stream(sim))
    for _ in range(3):
        sim.render(rp, read=False)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    kernels = 0
    with ClockSampler(0) as clocks:
        for k in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ev[k][0].record(ext)
            _, st = sim.render(rp, read=False)
            ev[k][1].record(ext)
            kernels += st.kernels
        torch.cuda.synchronize()
    dev_ms = [a.elapsed_time(b) for a, b in ev]
    # end to end: render + frame to host memory, wall clock
    frame_h = torch.empty((1080, 1920, 4), dtype=torch.uint8).pin_memory()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sim.render(rp, read=False)
        A._check(A.load_library().apic_read_frame(sim._h, A.ctypes.c_void_p(frame_h.data_ptr()), frame_h.numel()),
                 "apic_read_frame")
    e2e_s = (time.perf_counter() - t0) / args.steps
    frame, st = sim.render(rp)
    cpu = None
    if not args.no_cpu_baseline:
        q = [sim.read_field(f)[:n] for f in ("pos_x", "pos_y", "vel_x", "vel_y")]
        t0 = time.perf_counter()
        ref, _ = O.render(*q, rp)
        cpu_s = time.perf_counter() - t0
        cpu = {"value": n / cpu_s, "unit": "particles splatted/s", "cores": 1, "kind": "port",
               "sample": "one frame of the same particles (oracle draw loop, 1 thread)",
               "frame_identical": bool(np.array_equal(ref, frame))}
    mean_ms = float(np.mean(dev_ms))
    line = {
        "metric": "particles splatted/s", "value": n / (mean_ms / 1e3), "unit": "particles/s", "workload": "render",
        "n_gpus": 1, "steps": args.steps, "warmup": 3, "higher_is_better": True, "data": "synthetic",
        "ms_per_frame": mean_ms, "frame_ms_p50": float(np.percentile(dev_ms, 50)),
        "config": {"workload": f"{workload_name(side)}, after {args.warmup} updates; 1920x1080 RGBA8 frame, "
                               f"1080 px per unit, 3 px discs", "particles": n,
                   "l2": "flushed (256 MB write) before each frame"},
        "stats": {"valid": st.valid, "nan": st.nan, "out_of_bounds": st.out_of_bounds, "kernels": st.kernels},
        "e2e": {"value": n / e2e_s, "unit": "particles/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(frame_h.numel()),
                "what": "apic_render + apic_read_frame to pinned host memory, wall clock"},
        "gpu_launches": kernels, "clocks": clocks.summary(), "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    sim.close()


def set_stress(args):
    """Switch the module to config 3 (scene, frame dt, default side)."""
    global STRESS, FRAME_DT, SIDE
    STRESS = True
    FRAME_DT = 1.0 / 1000.0
    SIDE = 4096
    if args.side == 1024:
        args.side = SIDE


def main():
    # Scenes run on one stream each; the driver maps streams onto this many
    # hardware work queues (default 8), and kernels of streams that share a
    # queue run one after another.  Read when CUDA initialises, so set here.
    if any(w in sys.argv for w in ("batched", "served")):
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--solver", default="mixed", choices=["mixed", "fp32", "reference"])
    ap.add_argument("--side", type=int, default=SIDE)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched-summary", action="store_true",
                    help="single: skip the brief config-4 batched run reported beside the headline")
    ap.add_argument("--no-solver-compare", action="store_true",
                    help="skip the plain-FP32-vs-mixed solve comparison of the default workload")
    ap.add_argument("--eager", action="store_true",
                    help="launch the stages one by one in the timed region (for ncu launch lists)")
    ap.add_argument("--no-dsm", action="store_true",
                    help="keep the middle multigrid levels in global memory instead of a cluster's shared memory")
    ap.add_argument("--no-pdl", action="store_true",
                    help="launch the PCG loop's kernels in plain stream order")
    ap.add_argument("--workload", default="single", choices=["single", "stress", "batched", "served", "criterion",
                                                             "render"],
                    help="single: the 1024^2 scene (default); stress: config 3 (4096^2 noise scene); "
                         "batched: config 4; served: config 5; criterion: the reference's own bench shape "
                         "(sizes 64..1024, cell 1.0, update(0.016)); render: the headless particle view")
    ap.add_argument("--criterion-solver", default="reference", choices=["reference", "fp32", "mixed"],
                    help="criterion: pressure solver (reference: the reference's exit rule)")
    ap.add_argument("--scenes", type=int, default=256, help="batched: number of scenes")
    ap.add_argument("--compare-steps", type=int, default=5, help="batched: updates compared with the plain path")
    ap.add_argument("--rate", type=float, default=200.0, help="served: arrivals per second")
    ap.add_argument("--seconds", type=float, default=2.0, help="served: length of the arrival stream")
    ap.add_argument("--budget-gb", type=float, default=120.0, help="served: device-memory budget")
    ap.add_argument("--max-active", type=int, default=256, help="served: active scenes at most")
    ap.add_argument("--max-active-cells", type=int, default=16 << 20,
                    help="served: grid cells of the admitted scenes at most (0: no limit)")
    ap.add_argument("--prepare-threads", type=int, default=8, help="served: scene preparation threads")
    ap.add_argument("--served-rounds", action="store_true", help="served: also run the lock-step rounds server")
    ap.add_argument("--no-plain", action="store_true", help="served: skip the plain one-scene-at-a-time arm")
    ap.add_argument("--served-max-side", type=int, default=1024, help="served: largest grid side of the requests")
    ap.add_argument("--scene-option", action="append",
                    help="served: NAME=VALUE[@[MIN_CELLS:]MAX_CELLS], Apic.set_option on the served scenes of that size")
    ap.add_argument("--time-limit", type=float, default=60.0, help="served: stop each run after this many seconds")
    ap.add_argument("--cpu-steps", type=int, default=0, help="CPU sample updates (default: --steps)")
    ap.add_argument("--cpu-budget", type=float, default=30.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "stress":
        set_stress(args)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
    elif args.workload == "batched":
        run_batched(args, world, rank, local)
    elif args.workload == "served":
        run_served(args)
    elif args.workload == "criterion":
        run_criterion(args)
    elif args.workload == "render":
        run_render(args)
    else:
        run_gpu_arm(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
