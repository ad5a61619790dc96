"""GPU-vs-oracle parity on the benchmark configurations (needs a GB300).

* The plain dam break (128^2 MAC grid, dx = 1/128, fluid x < 0.4, y < 0.6,
  4 particles per cell jittered from seed 0, dt = 1/240, 100 updates, Morton
  sort on): free-running, the GPU equals the oracle bit for bit after every
  update in the reference solver mode (src/apic.rs:2429-2474 with the
  reference's reduction orders).  Beside it the test prints the error of both
  against FP64 runs of the oracle (u, v, pressure, particle positions): one
  update from the same state (the FP64 oracle re-synchronised before every
  update) and a free-running FP64 run; with the two FP32 results identical,
  the GPU's error against FP64 is the reference arithmetic's own.  In the
  mixed-precision mode (FP32 PCG inside FP64 refinement to a true relative
  residual of 1e-6; no counterpart in the reference) the GPU's and the
  oracle's reductions round differently: one update from the same state
  agrees within 1e-5 in u and v, and the free-running drift after 100
  updates is printed.
* The single large scene (1024^2, dam break x < 0.5, y < 0.5 plus the
  falling disk, seed 1, dt = 1/480): two updates stage by stage in lock-step,
  every stage bit-exact.  At this cell size dx^2 t (1 - t) <= 1e-6 for every
  particle, so the APIC C terms are zero on both sides
  (src/apic.rs:2211-2221).
* The reference's own benchmark shape (benches/fluid_benchmark.rs:13-41:
  Apic::new's particle block, cell size 1.0, 15 warm-up update(0.016)), at
  64^2 and 256^2: free-running, bit-exact after every update.
* P2G on particles the scenes never produce: outside the grid, non-finite,
  and thousands in one cell (more than one tile of the ordered gather stages),
  bit-exact against the oracle.
"""
import numpy as np
import pytest

import apic_gb300 as A
from parity_helpers import eq, make_pair, run_lockstep

pytestmark = pytest.mark.gpu

PROPS = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
MIXED_STEP_RTOL = 1e-5    # one mixed-mode update from the same state: u, v relative to the field maximum


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(gpu_lib):
    if A.device_count() == 0:
        pytest.skip("no CUDA device")


def config1_scene(side=128):
    return A.scene_params(A.SCENE_DAM_BREAK, side, cell_size=1.0 / side, sub=2, seed=0, fluid_x=0.4, fluid_y=0.6)


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = float(np.max(np.abs(b))) if b.size else 0.0
    return float(np.max(np.abs(a - b))) / scale if scale > 0 else float(np.max(np.abs(a - b), initial=0.0))


def particle_state(sim, n):
    return {f: sim.read_field(f)[:n] for f in A.PARTICLE_FIELDS}


def copy_particles(dst, src, n):
    """Give dst the particle state of src (all nine fields; the padding lanes too)."""
    for f in A.PARTICLE_FIELDS:
        dst.write_field(f, src.read_field(f))


def step_errors(a, b, n, cs):
    """Per-field relative differences of a against b (b the reference)."""
    out = {f: rel_err(a.read_field(f), b.read_field(f)) for f in ("u", "v", "pressure")}
    d = np.hypot(a.read_field("pos_x")[:n].astype(np.float64) - b.read_field("pos_x")[:n],
                 a.read_field("pos_y")[:n].astype(np.float64) - b.read_field("pos_y")[:n]) / cs
    out["pos_max_cells"] = float(np.max(d)) if n else 0.0
    return out


def test_config1_100_updates_bit_exact_with_fp64_report(oracle_mod):
    side = 128
    cs = 1.0 / side
    px, py, vx, vy = A.generate_scene(config1_scene(side))
    g = A.Apic(side, side, cs, PROPS)
    o = oracle_mod.OracleSim(side, side, cs, PROPS)
    o64 = oracle_mod.OracleSim(side, side, cs, PROPS, fp64=True)       # re-synchronised before every update
    free64 = oracle_mod.OracleSim(side, side, cs, PROPS, fp64=True)    # free-running
    for sim in (g, o, o64, free64):
        sim.set_particles(px, py, vx, vy)
    n = len(px)
    opts = A.DebugOptions()
    report = {}
    for k in range(1, 101):
        copy_particles(o64, o, n)
        for sim in (g, o, o64, free64):
            sim.update(opts, 1.0 / 240)
        assert g.timestamp == o.info().timestamp, k
        for f in A.PARTICLE_FIELDS:
            eq(g.read_field(f)[:n], o.read_field(f)[:n], f"update {k} {f}")
        for f in ("u", "v", "pressure", "density"):
            eq(g.read_field(f), o.read_field(f), f"update {k} {f}")
        if o64.info().timestamp == o.info().timestamp:
            e = step_errors(g, o64, n, cs)
            for f, v in e.items():
                report[f] = max(report.get(f, 0.0), v)
        if k in (1, 10, 100):
            report[f"free_{k}"] = step_errors(g, free64, n, cs)
    print("\nconfig 1 (128^2 dam break, 100 updates of 1/240, sort on), reference solver: GPU == oracle FP32 bit "
          "for bit after every update (drift 0).  Error of both against FP64:")
    print("  one update from the same state, worst over 100 updates: u {u:.2e}  v {v:.2e}  pressure {pressure:.2e}"
          "  positions {pos_max_cells:.2e} cells".format(**report))
    for k in (1, 10, 100):
        e = report[f"free_{k}"]
        print(f"  free-running FP64 run, after update {k:3d}: u {e['u']:.2e}  v {e['v']:.2e}  "
              f"pressure {e['pressure']:.2e}  positions {e['pos_max_cells']:.2e} cells")
    assert report["u"] < 1e-4 and report["v"] < 1e-4 and report["pos_max_cells"] < 1e-2


def test_config1_mixed_solver_per_update_and_drift(oracle_mod):
    """Mixed solver (true relative residual <= 1e-6): from the same particle
    state, one update on the GPU and on the oracle agree within 1e-5 of the
    field maximum in u and v (their FP32 Krylov reductions round differently);
    the free-running drift after 100 updates is printed."""
    side = 128
    cs = 1.0 / side
    px, py, vx, vy = A.generate_scene(config1_scene(side))
    n = len(px)
    opts = A.DebugOptions()
    g = A.Apic(side, side, cs, PROPS)
    o = oracle_mod.OracleSim(side, side, cs, PROPS)
    for sim in (g, o):
        sim.set_particles(px, py, vx, vy)
        sim.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
    g.set_option(A.OPT_WARM_START, 0)
    o.set_warm_start(False)
    worst = {}
    for k in range(1, 101):
        copy_particles(o, g, n)
        g.update(opts, 1.0 / 240)
        o.update(opts, 1.0 / 240)
        assert g.stats().true_residual_rel <= 1e-6 and o.stats().true_residual_rel <= 1e-6
        assert g.timestamp == o.info().timestamp, k
        for f, v in step_errors(g, o, n, cs).items():
            worst[f] = max(worst.get(f, 0.0), v)
    # free-running, with the default warm start
    g2 = A.Apic(side, side, cs, PROPS)
    o2 = oracle_mod.OracleSim(side, side, cs, PROPS)
    for sim in (g2, o2):
        sim.set_particles(px, py, vx, vy)
        sim.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
    drift = {}
    for k in range(1, 101):
        g2.update(opts, 1.0 / 240)
        o2.update(opts, 1.0 / 240)
        if k in (1, 10, 100):
            drift[k] = step_errors(g2, o2, n, cs)
    print("\nconfig 1, mixed solver: one update from the same state, worst over 100 updates: "
          "u {u:.2e}  v {v:.2e}  pressure {pressure:.2e}  positions {pos_max_cells:.2e} cells".format(**worst))
    for k, e in drift.items():
        print(f"  free-running after update {k:3d}: u {e['u']:.2e}  v {e['v']:.2e}  pressure {e['pressure']:.2e}  "
              f"positions {e['pos_max_cells']:.2e} cells")
    assert worst["u"] <= MIXED_STEP_RTOL and worst["v"] <= MIXED_STEP_RTOL
    assert all(np.isfinite(g2.read_field(f)).all() for f in ("pos_x", "pos_y"))


def test_config2_lockstep_1024(oracle_mod):
    side = 1024
    cs = 1.0 / side
    scene = A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=cs, sub=2, seed=1, fluid_x=0.5, fluid_y=0.5,
                           disk=(0.7, 0.8, 0.08), disk_v=(0.0, -2.0))
    o, g = make_pair(oracle_mod, side, cs, PROPS, scene)
    run_lockstep(o, g, 2, 1.0 / 480, PROPS, cs)
    for f in ("cu_x", "cu_y", "cv_x", "cv_y"):
        a, b = g.read_field(f), o.read_field(f)
        eq(a, b, f)
        assert not np.any(a), f"{f}: APIC C should vanish at dx = 1/1024"


@pytest.mark.parametrize("side", [64, 256])
def test_criterion_shape_bit_exact(oracle_mod, side):
    o, g = make_pair(oracle_mod, side, 1.0, PROPS)
    n = o.info().num_particles
    assert g.num_particles == n
    opts = A.DebugOptions()
    for k in range(18):  # 15 warm-up updates, then timed ones
        o.update(opts, 0.016)
        g.update(opts, 0.016)
        assert g.timestamp == o.info().timestamp, k
        for f in A.PARTICLE_FIELDS:
            eq(g.read_field(f)[:n], o.read_field(f)[:n], f"update {k} {f}")
        for f in ("u", "v", "pressure"):
            eq(g.read_field(f), o.read_field(f), f"update {k} {f}")


def test_p2g_unusual_particles(oracle_mod):
    side = 64
    cs = 1.0 / side
    rng = np.random.default_rng(5)
    m = 6000  # all in one cell: more particles than one gather tile stages
    px = np.concatenate([np.full(m, 0.3, np.float32) + rng.uniform(0, 0.5 * cs, m).astype(np.float32),
                         rng.uniform(-0.5, 1.5, 500).astype(np.float32),
                         np.array([np.nan, np.inf, -np.inf, 1e10, -3e9, 0.0, 1.0, 1.0 - 1e-7], np.float32)])
    py = np.concatenate([np.full(m, 0.6, np.float32) + rng.uniform(0, 0.5 * cs, m).astype(np.float32),
                         rng.uniform(-0.5, 1.5, 500).astype(np.float32),
                         np.array([0.5, 0.5, 0.5, 0.5, 0.5, np.nan, 1.0, 0.0], np.float32)])
    vx = rng.normal(size=len(px)).astype(np.float32)
    vy = rng.normal(size=len(px)).astype(np.float32)
    o = oracle_mod.OracleSim(side, side, cs, PROPS)
    g = A.Apic(side, side, cs, PROPS)
    for sim in (o, g):
        sim.set_particles(px, py, vx, vy)
    for sort in (False, True):
        if sort:
            o.run_stage("sort", 1.0 / 240)
            g.run_stage("sort", 1.0 / 240)
        o.run_stage("p2g", 1.0 / 240)
        g.run_stage("p2g", 1.0 / 240)
        for f in ("u", "v", "density", "valid_u", "valid_v", "fluid_bits"):
            eq(g.read_field(f), o.read_field(f), f"p2g {f} (sorted {sort})")


def test_config3_lockstep_4096(oracle_mod):
    """The stress scene at its full size (4096^2, value-noise mask > 0.5 with
    lattice period 1/64, seed 2, 33.2 M particles, v ~ N(0, 0.5^2)): one
    substep stage by stage in the reference solver mode, every stage
    bit-identical to the oracle (serial, the reference's single-thread
    order), including the Morton sort of 33 M particles and every multigrid
    level."""
    side = 4096
    cs = 1.0 / side
    scene = A.scene_params(A.SCENE_NOISE, side, cell_size=cs, sub=2, seed=2, noise_period=1.0 / 64,
                           noise_threshold=0.5, vel_sigma=0.5)
    o, g = make_pair(oracle_mod, side, cs, PROPS, scene)
    assert g.num_particles == o.info().num_particles > 30_000_000
    stats = run_lockstep(o, g, 1, 1.0 / 8000, PROPS, cs)
    # the reference's exits stop this solve after a few iterations (gamma
    # falls below SAFTY at dx = 1/4096); the iterations run are the oracle's
    assert stats["pcg_iters"][0][0] == stats["pcg_iters"][0][1] > 0
