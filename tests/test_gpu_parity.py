"""GPU-vs-oracle parity through the C-ABI (needs a GB300).

Lock-step test: the GPU library and the CPU oracle start from the same
particles and run each stage of every substep in the reference's order
(src/apic.rs:2429-2474).  After each stage the outputs are compared bit for
bit (== on values, so -0 == +0): Morton keys and the stable sort
permutation, the permuted particles, the P2G sums (every face folds its
(chunk, corner) group sums in the oracle's single-thread order), fluid masks
and lists, valid flags, forces, density smoothing and the Laplacian,
multigrid coarsening, the pressure gradient, extrapolation and
G2P/advection.  In the reference solver mode the V-cycle and the PCG
pressure are bit-exact too: the GPU forms dot_product's eight lane sums,
apply_matrix_and_dot's 8192-cell chunk sums and the coarsest CG's serial
sums in the reference's order.  In the mixed-precision mode (no counterpart
in the reference) the GPU's Krylov reductions are double-float and the
oracle's FP64, so the V-cycle and the pressure are compared within a stated
tolerance and the GPU is then re-synchronised from the oracle.
"""
import numpy as np
import pytest

import apic_gb300 as A
from parity_helpers import eq, iterations_close, make_pair, run_lockstep

pytestmark = pytest.mark.gpu



@pytest.fixture(scope="module", autouse=True)
def _need_gpu(gpu_lib):
    if A.device_count() == 0:
        pytest.skip("no CUDA device")


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
    # the stage-by-stage comparison wants the oracle's P2G order in both modes
    g.set_option(A.OPT_P2G_ORDER, 1)
    forces = {2: [(0.2, 0.3, 0.05, 150.0)], 3: [(0.25, 0.2, 0.06, -150.0)]}
    run_lockstep(o, g, 5, 1 / 240, props, cs, forces, exact=mode == A.SOLVER_REFERENCE)


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


def test_full_updates_equal_oracle(oracle_mod):
    """Whole updates (one CUDA graph each, Morton sort on), no re-sync: after
    every one of 20 updates of the reference's default scene every particle
    field, the grid velocities and the pressure equal the oracle's bit for bit
    (reference solver mode)."""
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    side = 64
    o, g = make_pair(oracle_mod, side, 1 / side, props)
    opts = A.DebugOptions()
    n = o.info().num_particles
    for k in range(20):
        o.update(opts, 1 / 60)
        g.update(opts, 1 / 60)
        assert g.timestamp == o.info().timestamp, k
        for f in A.PARTICLE_FIELDS:
            eq(g.read_field(f)[:n], o.read_field(f)[:n], f"update {k} {f}")
        for f in ("u", "v", "pressure"):
            eq(g.read_field(f), o.read_field(f), f"update {k} {f}")


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
    for f in A.PARTICLE_FIELDS + ["pressure", "u", "v"]:
        eq(a.read_field(f), b.read_field(f), f"graph vs staged {f}")


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
    for dsm in (1, 0, 1):
        g.set_option(A.OPT_DSM_VCYCLE, dsm)
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
        assert its[0] == its[1], (mode, its)
        if mode == A.SOLVER_REL_MIXED:
            for h in sims:
                assert float(h.stats().true_residual_rel) <= 1e-6
        for f in ("pressure", "pos_x", "pos_y", "vel_x", "vel_y"):
            eq(sims[0].read_field(f), sims[1].read_field(f), f"dsm vs global {f}")


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


P2G_CELL_ORDER_RTOL = 4e-6  # the same <= 24 terms per face in another order, relative to the field maximum


def test_p2g_cell_order(oracle_mod):
    """APIC_OPT_P2G_ORDER 2 (the relative solver modes' default) adds each
    face's terms by cell, then by slot, instead of the reference's (chunk,
    corner) order: fluid bits, lists and valid flags equal the oracle's, the
    sums agree within a few float roundings, and the result is the same on
    every run."""
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    side = 128
    cs = 1 / side
    scene = A.scene_params(A.SCENE_DAM_BREAK, side, cell_size=cs, sub=2, seed=0, fluid_x=0.4, fluid_y=0.6)
    o, g = make_pair(oracle_mod, side, cs, props, scene)
    assert g.get_option(A.OPT_P2G_ORDER) == 1  # reference solver mode: the reference's order
    run_lockstep(o, g, 3, 1 / 240, props, cs)
    g.set_option(A.OPT_P2G_ORDER, 2)
    assert g.get_option(A.OPT_P2G_ORDER) == 2
    o.run_stage("p2g", 1 / 240)
    g.run_stage("p2g", 1 / 240)
    for f in ("fluid_bits", "fluid_list", "valid_u", "valid_v"):
        eq(g.read_field(f), o.read_field(f), "cell-order p2g " + f)
    first = {}
    for f in ("u", "v", "density"):
        a, b = g.read_field(f).astype(np.float64), o.read_field(f).astype(np.float64)
        scale = float(np.max(np.abs(b)))
        assert scale > 0
        err = float(np.max(np.abs(a - b))) / scale
        assert err <= P2G_CELL_ORDER_RTOL, (f, err)
        first[f] = g.read_field(f).copy()
    g.run_stage("p2g", 1 / 240)
    for f in ("u", "v", "density"):
        eq(g.read_field(f), first[f], "cell-order p2g, second run " + f)
    # the relative modes default to cell order, the reference mode to the reference's
    g.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
    g.set_option(A.OPT_P2G_ORDER, 0)
    assert g.get_option(A.OPT_P2G_ORDER) == 2
    g.set_solver(A.SOLVER_REFERENCE, 1e-6, 500)
    assert g.get_option(A.OPT_P2G_ORDER) == 1
    with pytest.raises(A.ApicError):
        g.set_option(A.OPT_P2G_ORDER, 3)
