"""Headless particle view on the GPU against the oracle (needs a GB300).

The GPU frame is compared byte for byte with the oracle's sequential draw loop
on the same particles (read back from the device), together with the
RenderStats counters, the pick and the volume.
"""
import numpy as np
import pytest

import apic_gb300 as A

pytestmark = pytest.mark.gpu

# the GUI's world (src/main.rs:355-363) and grid (:29-31)
GUI_PROPS = A.WorldProperties(-9.8, 0.5, 5.0, 1e-5)


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(gpu_lib):
    if A.device_count() == 0:
        pytest.skip("no CUDA device")


def particles(g):
    n = g.info().num_particles
    return [g.read_field(f)[:n] for f in ("pos_x", "pos_y", "vel_x", "vel_y")]


def check_frame(oracle_mod, g, params):
    frame, st = g.render(params)
    px, py, vx, vy = particles(g)
    info = g.info()
    ref, rst = oracle_mod.render(px, py, vx, vy, params, fluid_cells=info.fluid_cells, cell_size=info.cell_size)
    assert (st.valid, st.nan, st.out_of_bounds, st.picked) == (rst.valid, rst.nan, rst.out_of_bounds, rst.picked)
    assert st.fluid_cells == rst.fluid_cells and st.volume == rst.volume
    diff = np.argwhere(np.any(frame != ref, axis=2))
    assert len(diff) == 0, (len(diff), diff[:5].tolist())
    assert st.kernels > 0
    return frame, st


def test_gui_scene_frames(oracle_mod):
    """The GUI's own scene: Apic::new's default block on a 256 x 128 grid with
    cell 0.075, drawn at 1920 x 1080 after each of three 1/60 s updates."""
    g = A.Apic(256, 128, 0.075, GUI_PROPS)
    sc = A.scene_params(A.SCENE_REFERENCE_DEFAULT, 256, 128, cell_size=0.075)
    g.set_particles(*A.generate_scene(sc))
    p = A.render_params()
    frame, st = check_frame(oracle_mod, g, p)
    assert st.valid == g.info().num_particles and st.nan == 0
    for _ in range(3):
        g.update(A.DebugOptions(), 1 / 60)
        frame, st = check_frame(oracle_mod, g, p)
    assert np.count_nonzero(frame[:, :, 2]) > 1000  # particles were drawn
    g.close()


def test_planted_nonfinite_far_and_pick(oracle_mod):
    rng = np.random.default_rng(5)
    n = 5000
    px = rng.uniform(0.5, 18.0, n).astype(np.float32)
    py = rng.uniform(0.5, 9.0, n).astype(np.float32)
    vx = rng.normal(0, 6, n).astype(np.float32)
    vy = rng.normal(0, 6, n).astype(np.float32)
    px[::97] = np.nan
    py[5::131] = np.inf
    px[7::113] = -3.0   # 300 px left of the frame
    py[11::89] = 30.0   # far above
    vx[13::101] = np.nan
    g = A.Apic(256, 128, 0.075, GUI_PROPS)
    g.set_particles(px, py, vx, vy)
    target = 1234
    tx, ty = float(px[target]) * 100.0, 1080.0 - float(py[target]) * 100.0
    _, st = check_frame(oracle_mod, g, A.render_params(pick=(tx, ty), pick_radius=12.0))
    assert st.nan > 0 and st.out_of_bounds > 0
    assert st.picked >= 0
    _, st = check_frame(oracle_mod, g, A.render_params(pick=(-500.0, -500.0), pick_radius=12.0))
    assert st.picked == -1
    g.close()


def test_odd_frame_radius_and_background(oracle_mod):
    g = A.Apic(128, 128, 1.0 / 128, GUI_PROPS)
    sc = A.scene_params(A.SCENE_DAM_BREAK_DISK, 128, cell_size=1.0 / 128, sub=2, seed=4, fluid_x=0.5,
                        fluid_y=0.5, disk=(0.7, 0.8, 0.1), disk_v=(0.0, -2.0))
    g.set_particles(*A.generate_scene(sc))
    g.update(A.DebugOptions(), 1 / 120)
    for w, h, scale, radius, bg in ((333, 77, 300.0, 7.0, (10, 20, 30)), (17, 1, 16.0, 0.5, (0, 0, 0)),
                                    (1000, 1000, 1000.0, 2.25, (255, 255, 255)), (64, 48, 40.0, 3.0, (1, 2, 3))):
        check_frame(oracle_mod, g, A.render_params(width=w, height=h, scale=scale, draw_radius=radius,
                                                   background=bg, margin=10.0))
    g.close()


def test_large_scene_frame(oracle_mod):
    """1.1 M particles of the 1024^2 dam break + disk, the domain filling a
    1080-pixel square of a 1920 x 1080 frame (about 260 overlapping quads per
    tile)."""
    side = 1024
    g = A.Apic(side, side, 1.0 / side, GUI_PROPS)
    sc = A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=1.0 / side, sub=2, seed=1, fluid_x=0.5,
                        fluid_y=0.5, disk=(0.7, 0.8, 0.08), disk_v=(0.0, -2.0))
    g.set_particles(*A.generate_scene(sc))
    g.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
    for _ in range(2):
        g.update(A.DebugOptions(), 1 / 480)
    _, st = check_frame(oracle_mod, g, A.render_params(scale=1080.0, pick=(540.0, 540.0), pick_radius=12.0))
    assert st.valid == g.info().num_particles
    g.close()


def test_empty_scene_and_device_pointer(oracle_mod):
    g = A.Apic(64, 64, 1.0 / 64, GUI_PROPS)
    e = np.zeros(0, np.float32)
    g.set_particles(e, e, e, e)  # Apic::new's default block removed
    frame, st = g.render(A.render_params(width=40, height=30, scale=30.0, background=(7, 8, 9)))
    assert np.all(frame == np.array([7, 8, 9, 255], dtype=np.uint8))
    assert (st.valid, st.nan, st.out_of_bounds, st.picked) == (0, 0, 0, -1)
    ptr, w, h = g.frame_device_ptr()
    assert ptr and (w, h) == (40, 30)
    g.close()


def test_render_rejects_bad_params(gpu_lib):
    g = A.Apic(64, 64, 1.0 / 64, GUI_PROPS)
    for kw in ({"width": 0}, {"height": 20000}, {"scale": 0.0}, {"draw_radius": 0.0}, {"draw_radius": 7.5},
               {"margin": -1.0}):
        with pytest.raises(A.ApicError) as ei:
            g.render(A.render_params(**{"scale": 10.0, **kw}))
        assert ei.value.code == A.ERR_INVALID_ARG, kw
    with pytest.raises(A.ApicError):
        g.frame_device_ptr()  # nothing rendered yet
    g.close()
