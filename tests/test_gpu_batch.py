"""Batched and served scenes through the C-ABI (needs a GB300).

A scene updated inside a batch, or as one request among others in the
continuous-batching server, runs exactly the kernels it runs alone, and every
kernel's result is independent of scheduling (P2G folds each face in a fixed
order; reductions are summed in a fixed order), so its results equal the
scene's results alone bit for bit.
"""
import numpy as np
import pytest

import apic_gb300 as A

pytestmark = pytest.mark.gpu

PROPS = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(gpu_lib):
    if A.device_count() == 0:
        pytest.skip("no CUDA device")


def dam_break(side, seed, frac):
    f = float(np.sqrt(frac))
    return A.scene_params(A.SCENE_DAM_BREAK, side, cell_size=1.0 / side, sub=2, seed=seed, fluid_x=f, fluid_y=f)


def disk_drop(side, seed):
    return A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=1.0 / side, sub=2, seed=seed, fluid_x=0.3,
                          fluid_y=0.3, disk=(0.6, 0.7, 0.1), disk_v=(0.0, -2.0))


def alone(scene, steps, dt):
    """The scene through the plain single-scene path."""
    g = A.Apic(scene.width, scene.height, scene.cell_size, PROPS)
    px, py, vx, vy = A.generate_scene(scene)
    g.set_particles(px, py, vx, vy)
    g.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
    for _ in range(steps):
        g.update(A.DebugOptions(), dt)
    return g


def test_update_batch_matches_alone(gpu_lib):
    scenes = [dam_break(64, 11, 0.3), disk_drop(96, 12), dam_break(128, 13, 0.5), dam_break(256, 14, 0.25)]
    steps, dt = 6, 1 / 240
    sims = []
    for sc in scenes:
        g = A.Apic(sc.width, sc.height, sc.cell_size, PROPS)
        px, py, vx, vy = A.generate_scene(sc)
        g.set_particles(px, py, vx, vy)
        g.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
        sims.append(g)
    for _ in range(steps):
        status = A.update_batch(sims, A.DebugOptions(), dt)
        assert status == [A.OK] * len(sims)
        for g in sims:
            assert g.stats().substeps >= 1
            assert float(g.stats().true_residual_rel) <= 1e-6
    for sc, g in zip(scenes, sims):
        ref = alone(sc, steps, dt)
        assert np.array_equal(g.read_vec2x8(0), ref.read_vec2x8(0)), sc.width


FIELDS = tuple(A.PARTICLE_FIELDS)


def fast_disk(side, seed, vy):
    return A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=1.0 / side, sub=2, seed=seed, fluid_x=0.25,
                          fluid_y=0.25, disk=(0.6, 0.6, 0.12), disk_v=(0.0, vy))


def make(scene, mode):
    g = A.Apic(scene.width, scene.height, scene.cell_size, PROPS)
    px, py, vx, vy = A.generate_scene(scene)
    g.set_particles(px, py, vx, vy)
    g.set_solver(mode, 1e-6, 500)
    return g


def assert_same(a, b, what):
    for f in FIELDS + ("pressure", "u", "v"):
        x, y = a.read_field(f), b.read_field(f)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (what, f)


@pytest.mark.parametrize("mode", [A.SOLVER_REL_MIXED, A.SOLVER_REL_FP32], ids=["mixed", "fp32"])
def test_joint_batch_bit_exact(gpu_lib, mode):
    """The joint batch (the solves of all scenes as one launch per phase):
    uneven sides (powers of two and not, one without segment-kernel levels
    above its coarse tail), scenes with different substep counts in the same
    update, and a graph reused across updates; every scene equals itself run
    alone bit for bit, and the stream-per-scene batch too."""
    scenes = [dam_break(64, 31, 0.3), dam_break(88, 32, 0.5), fast_disk(120, 33, -25.0), dam_break(176, 34, 0.4),
              disk_drop(200, 35), fast_disk(256, 36, -6.0), dam_break(344, 37, 0.25), dam_break(512, 38, 0.2)]
    steps, dt = 4, 1 / 120
    joint = [make(sc, mode) for sc in scenes]
    streams = [make(sc, mode) for sc in scenes]
    subs = []
    for _ in range(steps):
        assert A.update_batch(joint, A.DebugOptions(), dt, joint=True) == [A.OK] * len(scenes)
        info = A.batch_last_info()
        assert info["joint"] == 1 and info["scenes"] == len(scenes), info
        assert info["batch_kernel_launches"] > 0 and info["pcg_rounds"] > 0, info
        subs.append([g.stats().substeps for g in joint])
        assert A.update_batch(streams, A.DebugOptions(), dt, streams=True) == [A.OK] * len(scenes)
        assert A.batch_last_info()["joint"] == 0
        for g, h in zip(joint, streams):
            assert g.stats().substeps == h.stats().substeps
            assert g.stats().pcg_iterations_total == h.stats().pcg_iterations_total
            assert g.stats().refinement_steps == h.stats().refinement_steps
    assert any(len(set(row)) > 1 for row in subs), subs  # the scenes' substep counts differed
    for sc, g, h in zip(scenes, joint, streams):
        ref = make(sc, mode)
        for _ in range(steps):
            ref.update(A.DebugOptions(), dt)
        assert_same(g, ref, ("joint", sc.width))
        assert_same(h, ref, ("streams", sc.width))
        assert g.stats().pcg_iterations_total == ref.stats().pcg_iterations_total
        if mode == A.SOLVER_REL_MIXED:
            assert float(g.stats().true_residual_rel) <= 1e-6


def test_joint_batch_rebuilds(gpu_lib):
    """The batch graph follows its scenes: a changed setting, a scene list in
    another order and a destroyed scene all rebuild it; the reference solver
    mode falls back to the stream-per-scene batch."""
    scenes = [dam_break(96, 41, 0.4), disk_drop(128, 42), dam_break(160, 43, 0.3)]
    dt = 1 / 240
    sims = [make(sc, A.SOLVER_REL_MIXED) for sc in scenes]
    refs = [make(sc, A.SOLVER_REL_MIXED) for sc in scenes]
    A.update_batch(sims, A.DebugOptions(), dt, joint=True)
    for r in refs:
        r.update(A.DebugOptions(), dt)
    sims[1].set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)  # invalidates its graphs
    refs[1].set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
    A.update_batch(sims[::-1], A.DebugOptions(), dt, joint=True)
    assert A.batch_last_info()["joint"] == 1
    for r in refs:
        r.update(A.DebugOptions(), dt)
    for g, r, sc in zip(sims, refs, scenes):
        assert_same(g, r, ("rebuilt", sc.width))
    sims[0].close()
    A.update_batch(sims[1:], A.DebugOptions(), dt, joint=True)
    assert A.batch_last_info()["joint"] == 1
    for r in refs[1:]:
        r.update(A.DebugOptions(), dt)
    for g, r, sc in zip(sims[1:], refs[1:], scenes[1:]):
        assert_same(g, r, ("after destroy", sc.width))
    ref_mode = [make(sc, A.SOLVER_REFERENCE) for sc in scenes[:2]]
    A.update_batch(ref_mode, A.DebugOptions(), dt)
    assert A.batch_last_info()["joint"] == 0


def test_batch_tuner(gpu_lib):
    """The tuner tries the stream-per-scene form and the joint form's shapes
    on the caller's updates, then keeps one; every form gives the bits the
    scenes give alone."""
    scenes = [dam_break(72, 51, 0.4), disk_drop(104, 52), dam_break(136, 53, 0.3), fast_disk(64, 54, -8.0)]
    dt = 1 / 240
    sims = [make(sc, A.SOLVER_REL_MIXED) for sc in scenes]
    seen, tuned_at = set(), None
    steps = 32
    for k in range(steps):
        assert A.update_batch(sims, A.DebugOptions(), dt) == [A.OK] * len(scenes)
        info = A.batch_last_info()
        seen.add((info["joint"], info["chunk_segs"], info["block_group"]))
        if info["tuned"] and tuned_at is None:
            tuned_at = k
    assert tuned_at is not None, "the tuner never settled"
    assert len(seen) >= 4, seen  # both forms and several shapes ran
    assert info["chunk_segs"] % 8 == 0 and info["block_group"] >= 1
    for sc, g in zip(scenes, sims):
        ref = make(sc, A.SOLVER_REL_MIXED)
        for _ in range(steps):
            ref.update(A.DebugOptions(), dt)
        assert_same(g, ref, ("tuned", sc.width))


def test_update_batch_rejects_bad_input(gpu_lib):
    with pytest.raises(A.ApicError) as ei:
        A.update_batch([A.Apic(64, 64, 1 / 64, PROPS), type("X", (), {"_h": None})()], None, 1 / 240)
    assert ei.value.code == A.ERR_INVALID_ARG


@pytest.mark.parametrize("mode,threads", [(A.SERVER_CONTINUOUS, 4), (A.SERVER_CONTINUOUS, 0), (A.SERVER_ROUNDS, 0)],
                         ids=["continuous", "continuous-inline", "rounds"])
def test_server_results_same_alone_and_in_mix(gpu_lib, mode, threads):
    reqs = [(dam_break(64, 21, 0.4), 5), (disk_drop(128, 22), 3), (dam_break(96, 23, 0.2), 7),
            (dam_break(128, 24, 0.5), 4), (disk_drop(64, 25), 6), (dam_break(192, 26, 0.3), 2)]
    dt = 1 / 240
    # room for about two of these scenes at a time: admission must queue the rest
    budget = 2 * max(A.scene_bytes(sc.width, sc.height, len(A.generate_scene(sc)[0])) for sc, _ in reqs)
    sv = A.Server(budget, max_active=4, keep_results=True, mode=mode, prepare_threads=threads)
    if mode == A.SERVER_CONTINUOUS and threads:
        # per-size rules change how a scene runs, never what it computes
        sv.scene_option(A.OPT_STREAM_PRIORITY, 5, 0, 64 * 64)
        sv.scene_option(A.OPT_DSM_VCYCLE, 0, 96 * 96, 128 * 128)
    ids = [sv.submit(sc, PROPS, steps, dt) for sc, steps in reqs]
    max_stepped, rounds, waited = 0, 0, False
    while True:
        rd = sv.step()
        rounds += 1
        max_stepped = max(max_stepped, rd.stepped)
        waited = waited or (rd.queued > 0 and rd.active > 0)
        assert rd.memory_used <= budget
        if rd.active == 0 and rd.queued == 0:
            break
        assert rounds < 200
    st = sv.stats()
    assert st.completed == len(reqs) and st.failed == 0
    assert st.memory_peak <= budget
    assert max_stepped <= 4  # max_active
    assert waited  # the budget held requests back while others ran
    assert st.step_p99_ms >= st.step_p50_ms > 0.0
    assert st.request_p99_ms >= st.request_p50_ms > 0.0
    total = 0
    for rid, (sc, steps) in zip(ids, reqs):
        info = sv.request(rid)
        assert info.status == A.OK and info.finished and info.steps_done == steps
        assert info.admit_ms >= info.submit_ms and info.done_ms >= info.admit_ms
        assert info.max_true_residual <= 1e-6
        total += info.particles * info.substeps
        ref = alone(sc, steps, dt)
        assert np.array_equal(sv.result_positions(rid), ref.read_vec2x8(0)), rid
    assert st.particle_substeps == total
    assert st.updates == sum(steps for _, steps in reqs) and st.mode == mode
    sv.close()


def test_server_continuous_keeps_small_scenes_moving(gpu_lib):
    """In continuous mode a small scene's updates do not wait for a large
    scene's: the small request finishes while the large one still runs."""
    sv = A.Server(1 << 40, max_active=4, mode=A.SERVER_CONTINUOUS)
    big = sv.submit(dam_break(512, 31, 0.5), PROPS, 6, 1 / 240)
    small = sv.submit(dam_break(64, 32, 0.3), PROPS, 6, 1 / 240)
    small_done_first = False
    for _ in range(200):
        rd = sv.step()
        ib, is_ = sv.request(big), sv.request(small)
        if is_.finished and not ib.finished:
            small_done_first = True
        if rd.active == 0 and rd.queued == 0:
            break
    assert sv.request(big).finished and sv.request(small).finished
    assert sv.request(big).status == A.OK and sv.request(small).status == A.OK
    assert small_done_first
    sv.close()


def test_server_rejects_scene_over_budget(gpu_lib):
    sv = A.Server(1 << 20, max_active=2)
    with pytest.raises(A.ApicError) as ei:
        sv.submit(dam_break(256, 1, 0.5), PROPS, 3, 1 / 240)
    assert ei.value.code == A.ERR_OOM
    sv.close()


def test_scene_bytes_bounds_server_scenes(gpu_lib):
    """The admission estimate bounds what an admitted scene holds on the device."""
    import torch
    sv = A.Server(1 << 40, max_active=1, keep_results=True)
    # a first request loads the library's kernels and module data, which are
    # not part of a scene's footprint
    sv.submit(dam_break(128, 5, 0.3), PROPS, 1, 1 / 240)
    sv.step()
    for side, frac in ((128, 0.3), (512, 0.6), (1024, 0.6)):
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        rid = sv.submit(dam_break(side, 5, frac), PROPS, 2, 1 / 240)
        sv.step()  # admits the scene and runs its first update
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        used, est = free0 - free1, sv.request(rid).bytes
        assert used <= est, (side, used, est)
        sv.step()  # last update: positions kept, device memory released
    sv.close()


def test_stream_priority_option(gpu_lib):
    """The scene's stream priority is clamped to the device's range and does
    not change results."""
    sc = dam_break(64, 41, 0.4)
    runs = []
    for prio in (0, 3, 100):
        g = A.Apic(sc.width, sc.height, sc.cell_size, PROPS)
        g.set_particles(*A.generate_scene(sc))
        g.set_option(A.OPT_STREAM_PRIORITY, prio)
        got = g.get_option(A.OPT_STREAM_PRIORITY)
        assert 0 <= got <= prio
        if prio == 0:
            assert got == 0
        g.update(A.DebugOptions(disable_particle_sort=True), 1 / 240)
        runs.append(g.read_field("pos_x"))
        g.close()
    with pytest.raises(A.ApicError):
        A.Apic(64, 64, 1 / 64, PROPS).set_option(A.OPT_STREAM_PRIORITY, -1)
    assert np.array_equal(runs[1], runs[0])
    assert np.array_equal(runs[2], runs[0])


def test_server_work_limit_bounds_admitted_cells(gpu_lib):
    """With a work limit of one scene's cells, the server runs one scene at a
    time (each still completes); without it, all are admitted at once."""
    for limit, expect_max in ((96 * 96, 1), (0, 3)):
        sv = A.Server(1 << 40, max_active=8, mode=A.SERVER_CONTINUOUS, prepare_threads=2)
        sv.set_work_limit(limit)
        ids = [sv.submit(dam_break(96, 51 + k, 0.3), PROPS, 2, 1 / 240) for k in range(3)]
        most = 0
        for _ in range(100):
            rd = sv.step()
            most = max(most, rd.active)
            if rd.active == 0 and rd.queued == 0:
                break
        assert most == expect_max, (limit, most)
        assert all(sv.request(i).status == A.OK and sv.request(i).finished for i in ids)
        sv.close()
