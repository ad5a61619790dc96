"""Pipelined host I/O (apic_stage_field, apic_update_async / apic_update_wait,
apic_read_vec2x8_async / apic_read_wait): the same results, bit for bit, as
apic_write_field + apic_update + apic_read_vec2x8, with the next update's
forces uploaded and the last update's particles read back while an update
runs."""
import numpy as np
import pytest

import apic_gb300 as A
from parity_helpers import eq

pytestmark = pytest.mark.gpu


def test_pipelined_io_matches_synchronous(gpu_lib):
    torch = pytest.importorskip("torch")
    side = 128
    cs = 1.0 / side
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    sc = A.scene_params(A.SCENE_DAM_BREAK, side, cell_size=cs, sub=2, seed=0, fluid_x=0.4, fluid_y=0.6)
    px, py, vx, vy = A.generate_scene(sc)
    sims = []
    for _ in range(2):
        g = A.Apic(side, side, cs, props)
        g.set_particles(px, py, vx, vy)
        g.set_solver(A.SOLVER_REL_MIXED, 1e-6, 500)
        sims.append(g)
    sync, pipe = sims
    nu = sync.field_shape(A.FIELDS["ext_force_u"])[0]
    nv = sync.field_shape(A.FIELDS["ext_force_v"])[0]
    rng = np.random.default_rng(5)
    steps = 6
    forces = [(rng.normal(0, 20, nu).astype(np.float32), rng.normal(0, 20, nv).astype(np.float32))
              for _ in range(steps)]
    opts = A.DebugOptions()
    # synchronous reference run
    ref = []
    for fu, fv in forces:
        sync.write_field("ext_force_u", fu)
        sync.write_field("ext_force_v", fv)
        sync.update(opts, 1 / 240)
        ref.append((sync.read_vec2x8(0).copy(), sync.read_vec2x8(1).copy(), sync.stats().substeps))
    # pipelined: forces of step k+1 staged and step k's particles read back while updates run
    nc = pipe.num_chunks
    fu_h = [torch.from_numpy(f[0]).pin_memory() for f in forces]
    fv_h = [torch.from_numpy(f[1]).pin_memory() for f in forces]
    pos_h = [torch.empty(nc * 16, dtype=torch.float32).pin_memory() for _ in range(steps)]
    vel_h = [torch.empty(nc * 16, dtype=torch.float32).pin_memory() for _ in range(steps)]
    subs = []
    pipe.stage_field("ext_force_u", fu_h[0].data_ptr(), nu * 4)
    pipe.stage_field("ext_force_v", fv_h[0].data_ptr(), nv * 4)
    for k in range(steps):
        pipe.update_async(opts, 1 / 240)
        pipe.read_vec2x8_async(0, pos_h[k].data_ptr(), nc * 16)
        pipe.read_vec2x8_async(1, vel_h[k].data_ptr(), nc * 16)
        if k + 1 < steps:
            pipe.stage_field("ext_force_u", fu_h[k + 1].data_ptr(), nu * 4)
            pipe.stage_field("ext_force_v", fv_h[k + 1].data_ptr(), nv * 4)
        pipe.update_wait()
        subs.append(pipe.stats().substeps)
    pipe.read_wait()
    for k in range(steps):
        assert subs[k] == ref[k][2], (k, subs[k], ref[k][2])
        eq(pos_h[k].numpy(), ref[k][0].ravel(), f"pipelined positions, step {k}")
        eq(vel_h[k].numpy(), ref[k][1].ravel(), f"pipelined velocities, step {k}")
    # a staged field is applied once, by the next update only (then cleared like a written one)
    for g in (sync, pipe):
        g.update(opts, 1 / 240)
    eq(pipe.read_vec2x8(0), sync.read_vec2x8(0), "after the pipeline")
    with pytest.raises(A.ApicError):
        pipe.stage_field("pressure", fu_h[0].data_ptr(), nu * 4)
    with pytest.raises(A.ApicError):
        pipe.stage_field("ext_force_u", fu_h[0].data_ptr(), nu * 4 - 4)
