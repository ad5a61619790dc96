"""GPU-vs-oracle parity through the C-ABI (needs a GB300).

Lock-step test: the GPU library and the CPU oracle start from the same
particles and run each stage of every substep in the reference's order
(src/apic.rs:2429-2474).  After each stage the outputs are compared:

* bit-exact (== on values, so -0 == +0) for every stage whose arithmetic has
  one defined order: Morton keys and the stable sort permutation, the
  permuted particles, fluid masks and lists, valid flags, forces, density
  smoothing and the Laplacian, multigrid coarsening, the pressure gradient,
  extrapolation and G2P/advection;
* within a stated tolerance where the reference's own order is schedule
  dependent: P2G sums (float atomics, here and in the reference) and the PCG
  solve (FP64-accumulated reductions on the GPU, FP32 serial on the oracle).
  After those two stages the GPU state is re-synchronised from the oracle so
  the following stages start from identical inputs.
"""
import numpy as np
import pytest

import apic_gb300 as A

pytestmark = pytest.mark.gpu

P2G_RTOL = 2e-5      # relative to the field's max magnitude (order of float atomics)
PCG_RTOL = 2e-3      # pressure, relative to max |p| (FP64 vs FP32 reductions in the Krylov loop)
VCYCLE_RTOL = 1e-5   # z = M^-1 r: smoothing/transfers exact, coarsest CG reductions FP64 vs FP32


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(gpu_lib):
    if A.device_count() == 0:
        pytest.skip("no CUDA device")


def eq(a, b, name):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, f"{name}: shape {a.shape} vs {b.shape}"
    if a.dtype.kind == "f":
        bad = ~((a == b) | (np.isnan(a) & np.isnan(b)))
    else:
        bad = a != b
    if bad.any():
        i = int(np.argmax(bad))
        raise AssertionError(f"{name}: {int(bad.sum())}/{a.size} differ; first at {i}: gpu={a[i]!r} oracle={b[i]!r}")


def close(a, b, rtol, name):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    assert a.shape == b.shape, name
    scale = max(float(np.max(np.abs(b))) if b.size else 0.0, 1e-30)
    err = np.abs(a - b)
    worst = float(np.max(err)) if err.size else 0.0
    assert worst <= rtol * scale, f"{name}: max |diff| {worst:.3e} > {rtol:.1e} * max|ref| {scale:.3e}"
    return worst / scale


def iterations_close(a, b):
    """PCG iteration totals of two runs of the same updates.

    P2G's float atomics make two scenes differ in the last bits of the
    right-hand side; in the mixed solver that can move a refinement cycle's
    exit by an iteration or two, and a cycle more or less restarts PCG, so
    totals over two updates may differ by a few iterations."""
    return abs(int(a) - int(b)) <= max(3, int(0.1 * max(int(a), int(b))))


def fluid_padded(o):
    return o.read_field("fluid_list").astype(np.int64)


def host_dt(vmax, frame, t, cfl, cs):
    """Substep size exactly as src/apic.rs:2433-2441 computes it in f32."""
    f32 = np.float32
    safe = f32(f32(cfl) * f32(cs)) / f32(vmax) if f32(vmax) > f32(1e-5) else f32(frame)
    return float(min(safe, f32(f32(frame) - f32(t))))


def make_pair(oracle_mod, side, cs, props, scene=None):
    o = oracle_mod.OracleSim(side, side, cs, props)
    g = A.Apic(side, side, cs, props)
    if scene is not None:
        px, py, vx, vy = A.generate_scene(scene)
        o.set_particles(px, py, vx, vy)
        g.set_particles(px, py, vx, vy)
    return o, g


def lockstep_substep(o, g, dt, sort, stats):
    pf = A.PARTICLE_FIELDS
    if sort:
        o.run_stage("sort", dt)
        g.run_stage("sort", dt)
        eq(g.read_field("sort_keys"), o.read_field("sort_keys"), "sort keys")
        eq(g.read_field("sort_vals"), o.read_field("sort_vals"), "sort vals")
        for f in pf:
            eq(g.read_field(f), o.read_field(f), f"permuted {f}")
    # P2G (order-dependent sums): compare within tolerance, then re-sync
    o.run_stage("p2g", dt)
    g.run_stage("p2g", dt)
    eq(g.read_field("fluid_bits"), o.read_field("fluid_bits"), "fluid bits")
    eq(g.read_field("fluid_list"), o.read_field("fluid_list"), "fluid list")
    eq(g.read_field("valid_u"), o.read_field("valid_u"), "valid u")
    eq(g.read_field("valid_v"), o.read_field("valid_v"), "valid v")
    for f in ("u", "v", "density"):
        stats.setdefault("p2g_" + f, []).append(close(g.read_field(f), o.read_field(f), P2G_RTOL, "p2g " + f))
        g.write_field(f, o.read_field(f))
    o.run_stage("forces", dt)
    g.run_stage("forces", dt)
    eq(g.read_field("u"), o.read_field("u"), "forces u")
    eq(g.read_field("v"), o.read_field("v"), "forces v")
    o.run_stage("build", dt)
    g.run_stage("build", dt)
    eq(g.read_field("smoothed_density"), o.read_field("smoothed_density"), "smoothed density")
    fl = fluid_padded(o)
    for f in ("residual", "diag", "inv_diag", "plus_x", "plus_y"):
        eq(g.read_field(f)[fl], o.read_field(f)[fl], "build " + f)
    o.run_stage("mg", dt)
    g.run_stage("mg", dt)
    levels = o.info().mg_levels
    for lvl in range(levels):
        eq(g.read_field(A.mg_field("fluid_bits", lvl)), o.read_field(A.mg_field("fluid_bits", lvl)), f"mg{lvl} bits")
        bits = o.read_field(A.mg_field("fluid_bits", lvl))
        raw = np.nonzero(np.unpackbits(bits.view(np.uint8), bitorder="little"))[0]
        lw = lvl_width(o, lvl)
        idx = raw + lw
        for f in ("diag", "inv_diag", "plus_x", "plus_y"):
            eq(g.read_field(A.mg_field(f, lvl))[idx], o.read_field(A.mg_field(f, lvl))[idx], f"mg{lvl} {f}")
    # one V-cycle on the freshly built system (apply_preconditioner, src/apic.rs:1788-1821)
    o.run_stage("vcycle", dt)
    g.run_stage("vcycle", dt)
    stats.setdefault("vcycle", []).append(close(g.read_field("error")[fl], o.read_field("error")[fl], VCYCLE_RTOL,
                                                "vcycle z"))
    o.run_stage("pcg", dt)
    g.run_stage("pcg", dt)
    so, sg = o.stats(), g.stats()
    stats.setdefault("pcg_iters", []).append((sg.pcg_iterations, so.pcg_iterations))
    cells = fl - o.info().width
    p_o, p_g = o.read_field("pressure"), g.read_field("pressure")
    stats.setdefault("pcg_p", []).append(close(p_g[cells], p_o[cells], PCG_RTOL, "pressure"))
    # re-sync; writing the pressure also makes both sides project with this FP32 field
    g.write_field("pressure", p_o)
    o.write_field("pressure", p_o)
    o.run_stage("grad", dt)
    g.run_stage("grad", dt)
    for f in ("u", "v", "valid_u", "valid_v"):
        eq(g.read_field(f), o.read_field(f), "grad " + f)
    o.run_stage("post", dt)
    g.run_stage("post", dt)
    eq(g.read_field("u"), o.read_field("u"), "post u")
    o.run_stage("extrap", dt)
    g.run_stage("extrap", dt)
    for f in ("u", "v", "valid_u", "valid_v"):
        eq(g.read_field(f), o.read_field(f), "extrap " + f)
    o.run_stage("g2p", dt)
    g.run_stage("g2p", dt)
    for f in pf:
        eq(g.read_field(f), o.read_field(f), "g2p " + f)
    o.finish_substep(dt)
    g.finish_substep(dt)


def lvl_width(o, lvl):
    """Width of coarse level lvl (src/apic.rs:900-908 halves both sides)."""
    w = o.info().width
    for _ in range(lvl + 1):
        w //= 2
    return w


def run_lockstep(o, g, frames, frame_dt, props, cs, forces=None):
    stats = {}
    for k in range(frames):
        if forces and k in forces:
            for args in forces[k]:
                o.add_radial_force(*args)
                g.add_radial_force(*args)
            for f in ("ext_force_u", "ext_force_v", "post_force_u", "post_force_v"):
                eq(g.read_field(f), o.read_field(f), f)
        t = np.float32(0)
        first = True
        while t < np.float32(frame_dt):
            vo = o.get_max_particle_velocity()
            vg = g.get_max_particle_velocity()
            assert vg == vo, f"max velocity gpu {vg} oracle {vo}"
            dt = host_dt(vo, frame_dt, t, props.cfl, cs)
            lockstep_substep(o, g, dt, first, stats)
            first = False
            t = np.float32(t + np.float32(dt))
        # clear the frame's forces like Apic::update does (src/apic.rs:2470-2473)
        zu = np.zeros_like(o.read_field("ext_force_u"))
        zv = np.zeros_like(o.read_field("ext_force_v"))
        for name, z in (("ext_force_u", zu), ("ext_force_v", zv), ("post_force_u", zu), ("post_force_v", zv)):
            o.write_field(name, z)
            g.write_field(name, z)
    return stats


def test_lockstep_reference_default_scene(oracle_mod):
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    side = 64
    o, g = make_pair(oracle_mod, side, 1 / side, props)
    st = run_lockstep(o, g, 6, 1 / 60, props, 1 / side)
    assert len(st["pcg_p"]) >= 6


@pytest.mark.parametrize("mode", [A.SOLVER_REFERENCE, A.SOLVER_REL_MIXED])
def test_lockstep_dam_break_with_forces(oracle_mod, mode):
    props = A.WorldProperties(-9.81, 0.5, 5.0, 1e-5)
    side = 128
    cs = 1 / side
    scene = A.scene_params(A.SCENE_DAM_BREAK, side, cell_size=cs, sub=2, seed=0, fluid_x=0.4, fluid_y=0.6)
    o, g = make_pair(oracle_mod, side, cs, props, scene)
    for sim in (o, g):
        sim.set_solver(mode, 1e-6, 500)
    forces = {2: [(0.2, 0.3, 0.05, 150.0)], 3: [(0.25, 0.2, 0.06, -150.0)]}
    run_lockstep(o, g, 5, 1 / 240, props, cs, forces)


def test_lockstep_random_velocities_odd_count(oracle_mod):
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    side = 64
    cs = 1 / side
    scene = A.scene_params(A.SCENE_NOISE, side, cell_size=cs, sub=2, seed=2, noise_period=0.15,
                           noise_threshold=0.5, vel_sigma=0.5)
    px, py, vx, vy = A.generate_scene(scene)
    n = len(px) - (len(px) % 8) - 3  # force a ragged last chunk
    o = oracle_mod.OracleSim(side, side, cs, props)
    g = A.Apic(side, side, cs, props)
    o.set_particles(px[:n], py[:n], vx[:n], vy[:n])
    g.set_particles(px[:n], py[:n], vx[:n], vy[:n])
    run_lockstep(o, g, 4, 1 / 60, props, cs)


def test_full_update_drift(oracle_mod):
    """Whole updates with no re-sync: the drift from the oracle stays small.

    Sorting is disabled so that slot k holds the same particle on both sides
    (a sort reorders particles whose cells differ by last-bit rounding).
    """
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    side = 64
    o, g = make_pair(oracle_mod, side, 1 / side, props)
    opts = A.DebugOptions(disable_particle_sort=True)
    n = o.info().num_particles
    worst = 0.0
    for k in range(20):
        o.update(opts, 1 / 60)
        g.update(opts, 1 / 60)
        if g.timestamp != o.info().timestamp:
            break  # one side split a frame into one more CFL substep; stop comparing
        for f in ("pos_x", "pos_y"):
            d = np.abs(g.read_field(f)[:n].astype(np.float64) - o.read_field(f)[:n])
            worst = max(worst, float(np.max(d)))
    print(f"max position drift over {k + 1} updates: {worst:.3e} (cell {1 / side:.3e})")
    assert worst < 0.25 / side


@pytest.mark.parametrize("mode", [A.SOLVER_REFERENCE, A.SOLVER_REL_MIXED])
def test_graph_and_staged_paths_agree(gpu_lib, mode):
    """apic_update as one CUDA graph vs kernel-by-kernel launches (profiling)."""
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    side = 64
    a = A.Apic(side, side, 1 / side, props)
    b = A.Apic(side, side, 1 / side, props)
    for g in (a, b):
        g.set_solver(mode, 1e-6, 500)
    b.set_profiling(True)
    opts = A.DebugOptions(disable_particle_sort=True)
    for _ in range(3):
        a.update(opts, 1 / 60)
        b.update(opts, 1 / 60)
    assert a.timestamp == b.timestamp
    times = b.stage_times()
    assert times["pcg"][1] == b.timestamp and times["g2p"][1] == b.timestamp
    for f in ("pos_x", "pos_y", "vel_x", "vel_y"):
        d = np.max(np.abs(a.read_field(f).astype(np.float64) - b.read_field(f)))
        assert d < 1e-4, (f, d)


def test_disable_sort_keeps_order(oracle_mod):
    props = A.WorldProperties()
    side = 64
    o, g = make_pair(oracle_mod, side, 1 / side, props)
    opts = A.DebugOptions(disable_particle_sort=True)
    x0 = g.read_field("pos_x").copy()
    g.update(opts, 1 / 60)
    o.update(opts, 1 / 60)
    x1 = g.read_field("pos_x")
    n = o.info().num_particles
    # no permutation: every particle moved by at most a few cells
    assert np.max(np.abs(x1[:n] - x0[:n])) < 3 / side


def test_empty_and_tiny_grids(gpu_lib):
    props = A.WorldProperties()
    g = A.Apic(8, 8, 1 / 8, props)  # the reference seeds no particles on 8x8
    assert g.num_particles == 0
    g.update(A.DebugOptions(), 1 / 60)
    h = A.Apic(64, 64, 1 / 64, props)
    h.set_particles(np.zeros(0, np.float32), np.zeros(0, np.float32))
    h.update(A.DebugOptions(), 1 / 60)
    assert h.num_particles == 0


def test_odd_side_rejected(gpu_lib):
    # src/apic.rs:910 panics when no multigrid level exists; the C-ABI returns an error
    with pytest.raises(A.ApicError) as ei:
        A.Apic(66 + 1, 64, 1 / 64, A.WorldProperties())
    assert ei.value.code == A.ERR_INVALID_ARG


def test_nonfinite_particle_is_reported(gpu_lib):
    props = A.WorldProperties()
    g = A.Apic(64, 64, 1 / 64, props)
    x = g.read_field("pos_x")
    x[5] = np.nan
    g.write_field("pos_x", x)
    g.update(A.DebugOptions(), 1 / 60)
    assert g.stats().nonfinite_lanes > 0


@pytest.mark.parametrize("mode", [A.SOLVER_REL_FP32, A.SOLVER_REL_MIXED])
def test_relative_solver_modes(oracle_mod, mode):
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    side = 128
    cs = 1 / side
    scene = A.scene_params(A.SCENE_DAM_BREAK, side, cell_size=cs, sub=2, seed=0, fluid_x=0.4, fluid_y=0.6)
    o, g = make_pair(oracle_mod, side, cs, props, scene)
    for s in (o, g):
        s.set_solver(mode, 1e-6, 500)
    opts = A.DebugOptions()
    for _ in range(8):
        o.update(opts, 1 / 240)
        g.update(opts, 1 / 240)
    sg, so = g.stats(), o.stats()
    assert sg.pcg_iterations > 0
    if mode == A.SOLVER_REL_MIXED:
        assert sg.true_residual_rel <= 1e-6, sg.true_residual_rel
        assert so.true_residual_rel <= 1e-6, so.true_residual_rel
    else:
        assert sg.true_residual_rel <= 1e-4


@pytest.mark.parametrize("mode", [A.SOLVER_REFERENCE, A.SOLVER_REL_FP32, A.SOLVER_REL_MIXED])
def test_persistent_solver_matches_graph_solver(gpu_lib, mode):
    """The one-kernel persistent solve and the graph of per-phase kernels run
    the same iterations; only the reduction grouping differs."""
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    side = 256
    cs = 1 / side
    scene = A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=cs, sub=2, seed=1, fluid_x=0.5, fluid_y=0.5,
                           disk=(0.7, 0.8, 0.08), disk_v=(0.0, -2.0))
    px, py, vx, vy = A.generate_scene(scene)
    sims = []
    for persistent in (0, 1):
        g = A.Apic(side, side, cs, props)
        g.set_particles(px, py, vx, vy)
        g.set_solver(mode, 1e-6, 500)
        try:
            g.set_option(A.OPT_PERSISTENT_SOLVE, persistent)
        except A.ApicError as e:
            if e.code == 8:  # APIC_ERR_UNSUPPORTED: no cooperative launch on this device
                pytest.skip("cooperative launch unavailable")
            raise
        assert g.get_option(A.OPT_PERSISTENT_SOLVE) == persistent
        sims.append(g)
    opts = A.DebugOptions(disable_particle_sort=True)
    for k in range(6):
        for g in sims:
            g.update(opts, 1 / 480)
        a, b = sims[0].stats(), sims[1].stats()
        assert abs(int(a.pcg_iterations) - int(b.pcg_iterations)) <= 1, (k, a.pcg_iterations, b.pcg_iterations)
        if mode == A.SOLVER_REL_MIXED:
            assert b.true_residual_rel <= 1e-6 and a.true_residual_rel <= 1e-6
    pa, pb = sims[0].read_field("pressure"), sims[1].read_field("pressure")
    scale = float(np.max(np.abs(pa))) or 1.0
    assert float(np.max(np.abs(pa - pb))) <= 1e-3 * scale
    for f in ("pos_x", "pos_y"):
        assert float(np.max(np.abs(sims[0].read_field(f) - sims[1].read_field(f)))) < 1e-3 * cs


@pytest.mark.parametrize("side", [128, 256, 1024])
def test_fused_vcycle_equals_unfused(gpu_lib, side):
    """One kernel per level and direction gives the same z = M^-1 r, bit for bit."""
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    cs = 1 / side
    scene = A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=cs, sub=2, seed=1, fluid_x=0.5, fluid_y=0.5,
                           disk=(0.7, 0.8, 0.08), disk_v=(0.0, -2.0))
    g = A.Apic(side, side, cs, props)
    px, py, vx, vy = A.generate_scene(scene)
    g.set_particles(px, py, vx, vy)
    for _ in range(4):
        g.update(A.DebugOptions(), 1 / 480)
    g.run_stage("mg", 1 / 480)
    fl = g.read_field("fluid_list").astype(np.int64)
    out = []
    for fused in (1, 0):
        g.set_option(A.OPT_FUSED_VCYCLE, fused)
        g.run_stage("vcycle", 1 / 480)
        out.append(g.read_field("error")[fl])
    eq(out[0], out[1], "fused vs unfused V-cycle")


@pytest.mark.parametrize("side,cells", [(256, 65536), (1024, 65536), (1024, 1 << 20), (2048, 1 << 20)])
def test_cluster_vcycle_equals_unfused(gpu_lib, side, cells):
    """Middle levels inside one thread-block cluster give the same z = M^-1 r, bit for bit."""
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    cs = 1 / side
    scene = A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=cs, sub=2, seed=1, fluid_x=0.5, fluid_y=0.5,
                           disk=(0.7, 0.8, 0.08), disk_v=(0.0, -2.0))
    g = A.Apic(side, side, cs, props)
    if g.get_option(A.OPT_CLUSTER_VCYCLE) == 0:
        pytest.skip("thread-block clusters unavailable")
    g.set_option(A.OPT_DSM_VCYCLE, 0)  # the distributed form replaces this one when on
    px, py, vx, vy = A.generate_scene(scene)
    g.set_particles(px, py, vx, vy)
    for _ in range(3):
        g.update(A.DebugOptions(), 1 / 480)
    g.run_stage("mg", 1 / 480)
    fl = g.read_field("fluid_list").astype(np.int64)
    out = []
    for value in (cells, 0, cells):
        g.set_option(A.OPT_CLUSTER_VCYCLE, value)
        assert g.get_option(A.OPT_CLUSTER_VCYCLE) == value
        g.run_stage("vcycle", 1 / 480)
        out.append(g.read_field("error")[fl])
    eq(out[0], out[1], "cluster vs per-kernel V-cycle")
    eq(out[2], out[1], "cluster V-cycle, second run")
    # whole updates through the graph agree with the per-kernel form too
    sims = []
    for value in (cells, 0):
        h = A.Apic(side, side, cs, props)
        h.set_particles(px, py, vx, vy)
        h.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
        h.set_option(A.OPT_DSM_VCYCLE, 0)
        h.set_option(A.OPT_CLUSTER_VCYCLE, value)
        for _ in range(2):
            h.update(A.DebugOptions(disable_particle_sort=True), 1 / 480)
        sims.append(h)
    its = [h.stats().pcg_iterations_total for h in sims]
    assert iterations_close(*its), its
    for h in sims:
        assert float(h.stats().true_residual_rel) <= 1e-6


def test_cluster_option_rejected_without_middle_levels(gpu_lib):
    """A grid whose multigrid levels all fit the shared-memory tail has no cluster levels."""
    g = A.Apic(64, 64, 1 / 64, A.WorldProperties(-9.81, 0.1, 5.0, 1e-5))
    assert g.get_option(A.OPT_CLUSTER_VCYCLE) == 0
    with pytest.raises(A.ApicError) as ei:
        g.set_option(A.OPT_CLUSTER_VCYCLE, 65536)
    assert ei.value.code == A.ERR_UNSUPPORTED
    g.set_option(A.OPT_CLUSTER_VCYCLE, 0)


@pytest.mark.parametrize("side,kind", [(256, "dam"), (1024, "dam"), (2048, "dam"), (512, "noise"), (1024, "noise")])
def test_dsm_vcycle_equals_global(gpu_lib, side, kind):
    """Levels held in a cluster's distributed shared memory give the same z = M^-1 r, bit for bit.
    Noise masks put fluid in every row band and against every border."""
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    cs = 1 / side
    if kind == "noise":
        scene = A.scene_params(A.SCENE_NOISE, side, cell_size=cs, sub=2, seed=2, noise_period=1 / 64,
                               noise_threshold=0.5, vel_sigma=0.5)
    else:
        scene = A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=cs, sub=2, seed=1, fluid_x=0.5,
                               fluid_y=0.5, disk=(0.7, 0.8, 0.08), disk_v=(0.0, -2.0))
    g = A.Apic(side, side, cs, props)
    if g.get_option(A.OPT_DSM_VCYCLE) == 0:
        pytest.skip("no level qualifies for the distributed form on this GPU")
    px, py, vx, vy = A.generate_scene(scene)
    g.set_particles(px, py, vx, vy)
    for _ in range(3):
        g.update(A.DebugOptions(), 1 / 480)
    g.run_stage("mg", 1 / 480)
    fl = g.read_field("fluid_list").astype(np.int64)
    out = []
    for dsm, cluster in ((1, 65536), (0, 0), (1, 65536)):
        g.set_option(A.OPT_DSM_VCYCLE, dsm)
        g.set_option(A.OPT_CLUSTER_VCYCLE, cluster)
        g.run_stage("vcycle", 1 / 480)
        out.append(g.read_field("error")[fl])
    eq(out[0], out[1], "distributed vs per-kernel V-cycle")
    eq(out[2], out[1], "distributed V-cycle, second run")
    # whole updates through the graph, both solver families
    for mode in (A.SOLVER_REFERENCE, A.SOLVER_REL_MIXED):
        sims = []
        for dsm in (1, 0):
            h = A.Apic(side, side, cs, props)
            h.set_particles(px, py, vx, vy)
            h.set_solver(mode, 1e-6, 500)
            h.set_option(A.OPT_DSM_VCYCLE, dsm)
            for _ in range(2):
                h.update(A.DebugOptions(disable_particle_sort=True), 1 / 480)
            sims.append(h)
        its = [h.stats().pcg_iterations_total for h in sims]
        assert iterations_close(*its), (mode, its)
        if mode == A.SOLVER_REL_MIXED:
            for h in sims:
                assert float(h.stats().true_residual_rel) <= 1e-6
        pa, pb = sims[0].read_field("pressure"), sims[1].read_field("pressure")
        scale = float(np.max(np.abs(pa))) or 1.0
        assert float(np.max(np.abs(pa - pb))) <= 1e-3 * scale


def test_read_vec2x8_layout(gpu_lib):
    """apic_read_vec2x8 returns the reference's Vec2x8 chunks (8 x lanes, then 8 y lanes) of every field pair."""
    side = 64
    g = A.Apic(side, side, 1 / side, A.WorldProperties(-9.81, 0.1, 5.0, 1e-5))
    rng = np.random.default_rng(7)
    n = 1001  # ragged last chunk
    px = rng.uniform(0.1, 0.9, n).astype(np.float32)
    py = rng.uniform(0.1, 0.9, n).astype(np.float32)
    g.set_particles(px, py, rng.normal(size=n).astype(np.float32), rng.normal(size=n).astype(np.float32))
    g.update(A.DebugOptions(), 1 / 480)
    pairs = [("pos_x", "pos_y"), ("vel_x", "vel_y"), ("cu_x", "cu_y"), ("cv_x", "cv_y")]
    for which, (fx, fy) in enumerate(pairs):
        out = g.read_vec2x8(which)
        x, y = g.read_field(fx), g.read_field(fy)
        chunks = out.reshape(-1, 16)
        eq(chunks[:, :8].ravel(), x, f"Vec2x8 x lanes ({fx})")
        eq(chunks[:, 8:].ravel(), y, f"Vec2x8 y lanes ({fy})")


@pytest.mark.parametrize("mode", [A.SOLVER_REFERENCE, A.SOLVER_REL_FP32, A.SOLVER_REL_MIXED])
@pytest.mark.parametrize("side", [64, 176, 256])
def test_cluster_solve_matches_graph_solver(gpu_lib, mode, side):
    """A small scene's whole solve in one cluster launch runs the same iterations as the graph of per-phase kernels."""
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    cs = 1 / side
    scene = A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=cs, sub=2, seed=3, fluid_x=0.5, fluid_y=0.5,
                           disk=(0.7, 0.8, 0.08), disk_v=(0.0, -2.0))
    px, py, vx, vy = A.generate_scene(scene)
    sims = []
    for cells in (1 << 20, 0):
        g = A.Apic(side, side, cs, props)
        g.set_particles(px, py, vx, vy)
        g.set_solver(mode, 1e-6, 500)
        g.set_option(A.OPT_CLUSTER_SOLVE, cells)
        sims.append(g)
    if sims[0].get_option(A.OPT_CLUSTER_SOLVE) == 0:
        pytest.skip("cluster launch unavailable")
    assert sims[1].get_option(A.OPT_CLUSTER_SOLVE) == 0
    opts = A.DebugOptions(disable_particle_sort=True)
    for k in range(6):
        for g in sims:
            g.update(opts, 1 / 480)
        a, b = sims[0].stats(), sims[1].stats()
        # FP32 Krylov loops whose reductions are grouped differently cross a
        # relative threshold a few iterations apart
        slack = max(3, int(0.15 * b.pcg_iterations_total))
        assert abs(int(a.pcg_iterations_total) - int(b.pcg_iterations_total)) <= slack, (
            k, a.pcg_iterations_total, b.pcg_iterations_total)
        if mode == A.SOLVER_REL_MIXED:
            assert a.true_residual_rel <= 1e-6 and b.true_residual_rel <= 1e-6
    pa, pb = sims[0].read_field("pressure"), sims[1].read_field("pressure")
    scale = float(np.max(np.abs(pa))) or 1.0
    assert float(np.max(np.abs(pa - pb))) <= 1e-3 * scale
    for f in ("pos_x", "pos_y"):
        assert float(np.max(np.abs(sims[0].read_field(f) - sims[1].read_field(f)))) < 1e-3 * cs


def test_warm_start_option(oracle_mod):
    """APIC_OPT_WARM_START (default on): the mixed solve starts from the last
    solve's FP64 pressure, meets the same true-residual bound in fewer
    iterations than from zero, and follows the oracle's warm-started run."""
    side = 256
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    sc = A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=1.0 / side, sub=2, seed=7, fluid_x=0.5,
                        fluid_y=0.5, disk=(0.7, 0.8, 0.08), disk_v=(0.0, -2.0))
    px, py, vx, vy = A.generate_scene(sc)
    totals, pos = {}, {}
    for warm in (0, 1):
        g = A.Apic(side, side, 1.0 / side, props)
        assert g.get_option(A.OPT_WARM_START) == 1
        g.set_particles(px, py, vx, vy)
        g.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
        g.set_option(A.OPT_WARM_START, warm)
        assert g.get_option(A.OPT_WARM_START) == warm
        its = 0
        for _ in range(8):
            g.update(A.DebugOptions(), 1 / 240)
            st = g.stats()
            assert st.true_residual_rel <= 1e-6 and st.not_converged == 0
            its += st.pcg_iterations_total
        totals[warm], pos[warm] = its, g.read_vec2x8(0)
        g.close()
    assert totals[1] < totals[0], totals
    assert float(np.max(np.abs(pos[1] - pos[0]))) < 1e-3 / side
    o = oracle_mod.OracleSim(side, side, 1.0 / side, props, threads=4)
    o.set_particles(px, py, vx, vy)
    o.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
    its = 0
    for _ in range(8):
        o.update(A.DebugOptions(), 1 / 240)
        its += o.stats().pcg_iterations_total
    assert iterations_close(its, totals[1]), (its, totals[1])
