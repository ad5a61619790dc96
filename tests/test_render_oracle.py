"""Known answers of the oracle's headless particle view (no GPU).

The answers follow from the GUI's drawing code by hand: make_circle_texture
(src/main.rs:73-101), the speed tint and the RenderStats counters of
render_particles (:207-277).
"""
import numpy as np
import pytest

import apic_gb300 as A

BG = (0, 0, 0, 255)


def params(w=200, h=200, scale=100.0, **kw):
    return A.render_params(width=w, height=h, scale=scale, **kw)


def one(oracle_mod, x, y, vx=0.0, vy=0.0, **kw):
    f32 = lambda v: np.array([v], dtype=np.float32)  # noqa: E731
    return oracle_mod.render(f32(x), f32(y), f32(vx), f32(vy), params(**kw))


def test_particle_at_rest_centre_and_extent(oracle_mod):
    # draw_x = 1.0 * 100 = 100, draw_y = 200 - 100 = 100: quad [97, 103)^2,
    # pixels 97..102; the disc's inner texels have alpha 255, so the centre
    # pixels take the tint exactly: r = 0, g = 0.5 -> 128, b = 1 -> 255
    frame, st = one(oracle_mod, 1.0, 1.0)
    assert (st.valid, st.nan, st.out_of_bounds, st.picked) == (1, 0, 0, -1)
    for p in ((99, 99), (99, 100), (100, 99), (100, 100), (98, 100), (101, 99)):
        assert tuple(frame[p[1], p[0]]) == (0, 128, 255, 255), p
    # the quad's corners lie outside the disc: untouched
    for p in ((97, 97), (102, 97), (97, 102), (102, 102)):
        assert tuple(frame[p[1], p[0]]) == BG, p
    # nothing outside the quad changes
    touched = np.argwhere(np.any(frame[:, :, :3] != 0, axis=2))
    assert touched[:, 0].min() >= 97 and touched[:, 0].max() <= 102
    assert touched[:, 1].min() >= 97 and touched[:, 1].max() <= 102
    # the disc's rim is partly covered (anti-aliased): pixel (98, 97) samples
    # the texture between texels 7 and 8 of row 2, inside the alpha ramp
    edge = frame[97, 98]
    assert 0 < edge[2] < 255
    # the 6 x 6 footprint is symmetric under the four flips
    blk = frame[97:103, 97:103, 2]
    assert np.array_equal(blk, blk[::-1, :]) and np.array_equal(blk, blk[:, ::-1]) and np.array_equal(blk, blk.T)


def test_speed_tint(oracle_mod):
    # |v|^2 = 50: r = min(0.5, 1) = 0.5 -> 128, b = 1 - 0.25 -> 191 (190.75 + 0.5)
    frame, _ = one(oracle_mod, 1.0, 1.0, vx=5.0, vy=5.0)
    assert tuple(frame[100, 100]) == (128, 128, 191, 255)
    # |v|^2 >= 100 saturates r at 1: b = 0.5 -> 128
    frame, _ = one(oracle_mod, 1.0, 1.0, vx=30.0, vy=0.0)
    assert tuple(frame[100, 100]) == (255, 128, 128, 255)
    # a NaN velocity: f32::min(NaN, 1.0) is 1.0
    frame, _ = one(oracle_mod, 1.0, 1.0, vx=float("nan"), vy=0.0)
    assert tuple(frame[100, 100]) == (255, 128, 128, 255)


def test_counters_and_margin(oracle_mod):
    nan, inf = float("nan"), float("inf")
    # frame 200 x 200 at 100 px/unit, margin 50: x in [-0.5, 2.5] is drawn
    xs = np.array([1.0, nan, 1.0, inf, -0.49, -0.51, 2.49, 2.51, 1.0, 1.0], dtype=np.float32)
    ys = np.array([1.0, 1.0, nan, 1.0, 1.0, 1.0, 1.0, 1.0, -0.51, 2.51], dtype=np.float32)
    z = np.zeros_like(xs)
    _, st = oracle_mod.render(xs, ys, z, z, params())
    # drawn: x = 1, -0.49, 2.49; NaN/inf: 3; beyond the margin: x = -0.51,
    # 2.51 and y = -0.51 (draw_y 251), 2.51 (draw_y -51)
    assert (st.valid, st.nan, st.out_of_bounds) == (3, 3, 4)


def test_pick_nearest_first_on_ties(oracle_mod):
    # draw_x = 100, 106.25, 93.75, 150 (binary fractions: distances are exact)
    xs = np.array([1.0, 1.0625, 0.9375, 1.5], dtype=np.float32)
    ys = np.array([1.0, 1.0, 1.0, 1.0], dtype=np.float32)
    z = np.zeros_like(xs)
    # pick at pixel (100, 100): particle 0 at distance 0
    _, st = oracle_mod.render(xs, ys, z, z, params(pick=(100.0, 100.0), pick_radius=12.0))
    assert st.picked == 0
    # at 105: particle 1 (1.25 px) is nearer than particle 0 (5 px)
    _, st = oracle_mod.render(xs, ys, z, z, params(pick=(105.0, 100.0), pick_radius=12.0))
    assert st.picked == 1
    # at 103.125 particles 0 and 1 tie at 3.125 px: the first wins
    _, st = oracle_mod.render(xs, ys, z, z, params(pick=(103.125, 100.0), pick_radius=12.0))
    assert st.picked == 0
    # at 96.875 particles 0 and 2 tie: particle 0 again
    _, st = oracle_mod.render(xs, ys, z, z, params(pick=(96.875, 100.0), pick_radius=12.0))
    assert st.picked == 0
    # nothing within the radius
    _, st = oracle_mod.render(xs, ys, z, z, params(pick=(10.0, 10.0), pick_radius=12.0))
    assert st.picked == -1


def test_blend_order_matters(oracle_mod):
    # two overlapping particles of different tint: the later one is on top
    xs = np.array([1.0, 1.0], dtype=np.float32)
    ys = np.array([1.0, 1.0], dtype=np.float32)
    slow, fast = np.array([0.0, 30.0], dtype=np.float32), np.array([30.0, 0.0], dtype=np.float32)
    z = np.zeros(2, dtype=np.float32)
    a, _ = oracle_mod.render(xs, ys, slow, z, params())
    b, _ = oracle_mod.render(xs, ys, fast, z, params())
    assert tuple(a[100, 100]) == (255, 128, 128, 255)  # fast particle drawn last
    assert tuple(b[100, 100]) == (0, 128, 255, 255)
    # on the anti-aliased rim the blend of both shows, and differs by order
    assert not np.array_equal(a, b)


def test_background_and_empty(oracle_mod):
    e = np.zeros(0, dtype=np.float32)
    frame, st = oracle_mod.render(e, e, e, e, params(w=33, h=17, background=(10, 20, 30)))
    assert frame.shape == (17, 33, 4)
    assert np.all(frame == np.array([10, 20, 30, 255], dtype=np.uint8))
    assert (st.valid, st.nan, st.out_of_bounds, st.picked) == (0, 0, 0, -1)


def test_volume_stat(oracle_mod):
    e = np.zeros(0, dtype=np.float32)
    _, st = oracle_mod.render(e, e, e, e, params(), fluid_cells=1000, cell_size=0.075)
    # active_fluid_cells as f32 * (CELL_SIZE * CELL_SIZE), src/main.rs:466-468
    assert st.volume == pytest.approx(float(np.float32(1000) * (np.float32(0.075) * np.float32(0.075))), rel=0)


def test_gui_default_scale():
    # SIM_SCALE = WIDTH / (GRID_WIDTH * CELL_SIZE) = 1920 / 19.2 (src/main.rs:34)
    p = A.render_params()
    assert (p.width, p.height, p.draw_radius, p.margin) == (1920, 1080, 3.0, 50.0)
    assert p.scale == pytest.approx(100.0, rel=1e-6)
