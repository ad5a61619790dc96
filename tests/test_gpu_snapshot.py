"""Snapshot / restore through the C-ABI (needs a GB300).

A restored handle holds exactly the saved state (compared field by field and
by re-snapshotting), and its next updates compute what the original's do, bit
for bit (every kernel's result is independent of scheduling).
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


def scene(side, seed):
    g = A.Apic(side, side, 1.0 / side, PROPS)
    sc = A.scene_params(A.SCENE_DAM_BREAK_DISK, side, cell_size=1.0 / side, sub=2, seed=seed, fluid_x=0.4,
                        fluid_y=0.5, disk=(0.7, 0.7, 0.1), disk_v=(0.5, -2.0))
    g.set_particles(*A.generate_scene(sc))
    g.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
    return g


def test_restore_then_continue():
    side = 256
    a = scene(side, 3)
    for _ in range(3):
        a.update(A.DebugOptions(), 1 / 240)
    a.add_radial_force(0.5, 0.3, 0.1, 40.0)   # pending post force
    a.add_radial_force(0.3, 0.3, 0.1, -40.0)  # pending external force
    blob = a.snapshot()
    b = A.Apic(side, side, 1.0 / side, PROPS)
    b.restore(blob)
    for f in A.PARTICLE_FIELDS + ["obstacle_bits", "ext_force_u", "ext_force_v", "post_force_u", "post_force_v"]:
        assert np.array_equal(a.read_field(f), b.read_field(f), equal_nan=True), f
    ia, ib = a.info(), b.info()
    assert (ia.num_particles, ia.timestamp, ia.prev_deltatime) == (ib.num_particles, ib.timestamp, ib.prev_deltatime)
    assert b.snapshot() == blob
    for _ in range(3):
        a.update(A.DebugOptions(), 1 / 240)
        b.update(A.DebugOptions(), 1 / 240)
        assert a.stats().substeps == b.stats().substeps
    # (the pressure outside the current fluid cells is stale history, src/apic.rs:1872-1883, and not compared)
    for f in A.PARTICLE_FIELDS + ["u", "v"]:
        assert np.array_equal(a.read_field(f), b.read_field(f), equal_nan=True), f
    assert a.info().timestamp == b.info().timestamp
    a.close()
    b.close()


def test_empty_scene_round_trip():
    a = A.Apic(64, 64, 1.0 / 64, PROPS)
    e = np.zeros(0, np.float32)
    a.set_particles(e, e, e, e)  # Apic::new's default block removed
    blob = a.snapshot()
    b = A.Apic(64, 64, 1.0 / 64, PROPS)
    b.set_particles(np.full(10, 0.5, np.float32), np.full(10, 0.5, np.float32))
    b.restore(blob)
    assert b.info().num_particles == 0
    assert b.snapshot() == blob
    a.close()
    b.close()


def test_restore_rejects_other_scenes():
    a = scene(128, 1)
    blob = a.snapshot()
    for other in (A.Apic(256, 256, 1.0 / 256, PROPS), A.Apic(128, 128, 1.0 / 128, A.WorldProperties(-1.0, 0.1, 5.0, 1e-5)),
                  A.Apic(128, 128, 1.0 / 100, PROPS)):
        with pytest.raises(A.ApicError) as ei:
            other.restore(blob)
        assert ei.value.code == A.ERR_INVALID_ARG
        other.close()
    b = A.Apic(128, 128, 1.0 / 128, PROPS)
    bad = bytearray(blob)
    bad[0] ^= 0xFF
    for broken in (bytes(bad), blob[:-4], blob + b"\0" * 8, b""):
        with pytest.raises(A.ApicError) as ei:
            b.restore(broken)
        assert ei.value.code == A.ERR_INVALID_ARG
    a.close()
    b.close()
