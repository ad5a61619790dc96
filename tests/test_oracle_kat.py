"""Known-answer and invariant tests of the CPU oracle (no GPU).

The reference ships no tests or golden vectors, so these known answers are
derived by hand from the reference's formulas (src/apic.rs line cited per
test) and from an independent Python restatement of its integer hash.
"""
import math
import struct

import numpy as np
import pytest


def py_random_lane(slot: int, seed: int) -> float:
    """Apic::random_simd for one lane (src/apic.rs:946-975), in Python ints."""
    m = (slot ^ seed) & 0xFFFFFFFF
    m ^= m >> 16
    m = (m * 0x7FEB352D) & 0xFFFFFFFF
    m ^= m >> 15
    m = (m * 0x846CA68B) & 0xFFFFFFFF
    m ^= m >> 16
    f = struct.unpack("<f", struct.pack("<I", (m & 0x007FFFFF) | 0x3F800000))[0]
    return float(np.float32(f) - np.float32(1.5))


def test_morton_known_answers(oracle_mod):
    # expand_bits / morton_code, src/apic.rs:185-203
    cases = {(0, 0): 0, (1, 0): 1, (0, 1): 2, (1, 1): 3, (2, 0): 4, (3, 3): 15, (5, 9): 0b10010011,
             (0xFFFF, 0): 0x55555555, (0, 0xFFFF): 0xAAAAAAAA, (0xFFFF, 0xFFFF): 0xFFFFFFFF,
             (0x10000, 0): 0, (127, 127): 0x3FFF}
    for (x, y), k in cases.items():
        assert oracle_mod.morton(x, y) == k, (x, y)


def test_random_lane_matches_independent_restatement(oracle_mod):
    rng = np.random.default_rng(0)
    for slot, seed in [(0, 0), (1, 0), (7, 3), (123456, 99), (2**31 + 5, 2**32 - 1)] + \
            [(int(a), int(b)) for a, b in rng.integers(0, 2**32, size=(64, 2))]:
        v = oracle_mod.random_lane(slot, seed)
        assert v == py_random_lane(slot, seed)
        assert -0.5 <= v < 0.5


def test_temporal_weight_known_answers(oracle_mod):
    # temporal_kernel_w_t, src/apic.rs:31-46
    assert oracle_mod.temporal_weight(0.5) == 2.1875
    assert oracle_mod.temporal_weight(0.0) == 0.9228515625
    assert oracle_mod.temporal_weight(1.5) == pytest.approx(1e-5, rel=1e-6)
    assert oracle_mod.temporal_weight(-3.0) == pytest.approx(1e-5, rel=1e-6)


@pytest.mark.parametrize("side,count", [(128, 63189), (64, 13365), (8, 0)])
def test_reference_default_scene_count(oracle_mod, side, count):
    # Apic::new seeds 3x3 particles per cell for 4 < x < W-4, 4 < y < H/2 (src/apic.rs:838-846)
    from apic_gb300 import WorldProperties
    o = oracle_mod.OracleSim(side, side, 1.0 / side, WorldProperties())
    info = o.info()
    assert info.num_particles == count
    assert info.num_chunks == (count + 7) // 8
    if count:
        assert info.mg_levels == int(math.log2(side)) - 2


def test_padding_lanes_copy_last_particle(oracle_mod):
    # src/apic.rs:887-898: the last chunk is padded with the last position
    from apic_gb300 import WorldProperties
    o = oracle_mod.OracleSim(32, 32, 1 / 32, WorldProperties())
    px = np.array([0.3, 0.4, 0.5], np.float32)
    py = np.array([0.2, 0.2, 0.25], np.float32)
    o.set_particles(px, py)
    x = o.read_field("pos_x")
    assert len(x) == 8
    assert np.all(x[3:] == px[-1])
    assert np.all(o.read_field("vel_x") == 0)


def _run(o, steps, dt=1 / 60):
    from apic_gb300 import DebugOptions
    for _ in range(steps):
        o.update(DebugOptions(), dt)


def test_oracle_invariants_reference_scene(oracle_mod):
    from apic_gb300 import WorldProperties
    side = 64
    o = oracle_mod.OracleSim(side, side, 1.0 / side, WorldProperties())
    n0 = o.info().num_particles
    ts = 0
    for _ in range(6):
        _run(o, 1)
        st = o.stats()
        ts += st.substeps
        assert o.info().timestamp == ts
    info = o.info()
    assert info.num_particles == n0
    x, y = o.read_field("pos_x")[:n0], o.read_field("pos_y")[:n0]
    dx = 1.0 / side
    assert np.all(np.isfinite(x)) and np.all(np.isfinite(y))
    lo, hi = np.float32(1.001) * np.float32(dx), (np.float32(side) - np.float32(1.001)) * np.float32(dx)
    assert x.min() >= lo and x.max() <= hi and y.min() >= lo and y.max() <= hi
    fl = o.read_field("fluid_list")
    assert len(fl) == info.fluid_cells
    assert np.all(np.diff(fl.astype(np.int64)) > 0)
    bits = o.read_field("fluid_bits")
    assert sum(bin(int(w)).count("1") for w in bits) == info.fluid_cells
    obst = o.read_field("obstacle_bits")
    assert all((int(a) & int(b)) == 0 for a, b in zip(bits, obst))


def test_sort_is_stable_and_matches_keys(oracle_mod):
    from apic_gb300 import WorldProperties
    side = 64
    o = oracle_mod.OracleSim(side, side, 1.0 / side, WorldProperties())
    _run(o, 3)
    o.run_stage("sort", 0.0)
    keys = o.read_field("sort_keys").astype(np.int64)
    vals = o.read_field("sort_vals").astype(np.int64)
    assert np.all(np.diff(keys) >= 0)
    same = np.diff(keys) == 0
    assert np.all(np.diff(vals)[same] > 0)
    assert sorted(vals.tolist()) == list(range(len(vals)))


def test_fp64_shadow_close_to_fp32(oracle_mod):
    from apic_gb300 import WorldProperties
    side = 64
    a = oracle_mod.OracleSim(side, side, 1.0 / side, WorldProperties())
    b = oracle_mod.OracleSim(side, side, 1.0 / side, WorldProperties(), fp64=True)
    _run(a, 2)
    _run(b, 2)
    xa, xb = a.read_field("pos_y"), b.read_field("pos_y")
    assert xb.dtype == np.float64
    assert np.max(np.abs(xa - xb)) < 1e-4


def test_openmp_mode_matches_serial(oracle_mod):
    from apic_gb300 import WorldProperties
    side = 128
    a = oracle_mod.OracleSim(side, side, 1.0 / side, WorldProperties(), threads=1)
    b = oracle_mod.OracleSim(side, side, 1.0 / side, WorldProperties(), threads=4)
    _run(a, 3)
    _run(b, 3)
    for f in ("pos_x", "pos_y", "vel_x", "vel_y"):
        va, vb = a.read_field(f), b.read_field(f)
        scale = max(1e-6, float(np.max(np.abs(va))))
        assert np.max(np.abs(va - vb)) <= 1e-4 * scale, f


def test_mixed_warm_start_same_tolerance_fewer_iterations(oracle_mod):
    """The mixed solve started from the previous solve's FP64 pressure meets
    the same true-residual bound in fewer iterations and gives the same flow
    (the pressures differ only within that bound)."""
    import apic_gb300 as A
    side = 128
    sc = A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=1.0 / side, sub=2, seed=7, fluid_x=0.5,
                        fluid_y=0.5, disk=(0.7, 0.8, 0.08), disk_v=(0.0, -2.0))
    px, py, vx, vy = A.generate_scene(sc)
    runs = []
    for warm in (False, True):
        o = oracle_mod.OracleSim(side, side, 1.0 / side, A.WorldProperties(-9.81, 0.1, 5.0, 1e-5), threads=4)
        o.set_particles(px, py, vx, vy)
        o.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
        o.set_warm_start(warm)
        its = 0
        for _ in range(8):
            o.update(A.DebugOptions(), 1 / 240)
            st = o.stats()
            assert st.true_residual_rel <= 1e-6 and st.not_converged == 0
            its += st.pcg_iterations_total
        runs.append((its, o.read_field("pos_x"), o.read_field("pos_y")))
    (cold, cx, cy), (warm, wx, wy) = runs
    assert warm < cold, (warm, cold)
    assert float(np.max(np.abs(cx - wx))) < 1e-3 / side
    assert float(np.max(np.abs(cy - wy))) < 1e-3 / side
