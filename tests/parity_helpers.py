"""Lock-step helpers shared by the GPU-vs-oracle parity tests.

The GPU library (apic_gb300.Apic) and the CPU oracle (oracle.oracle.OracleSim)
run each stage of every substep in the reference's order
(src/apic.rs:2429-2474) from the same state, and each stage's outputs are
compared.
"""
import numpy as np

import apic_gb300 as A

# mixed-precision mode only (the reference mode is compared with ==)
PCG_RTOL = 2e-3      # pressure, relative to max |p| (inner FP32 solves reduced in different orders)
VCYCLE_RTOL = 1e-5   # z = M^-1 r: smoothing/transfers exact, coarsest CG reductions FP64 vs FP32


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
    """PCG iteration totals of the GPU and the oracle over the same updates in
    the mixed solver: their Krylov reductions round differently, which can
    move a refinement cycle's exit by an iteration or two, and a cycle more or
    less restarts PCG, so totals may differ by a few iterations."""
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


def lockstep_substep(o, g, dt, sort, stats, exact=True):
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
    # P2G folds each face's (chunk, corner) group sums in the oracle's order
    for f in ("u", "v", "density"):
        eq(g.read_field(f), o.read_field(f), "p2g " + f)
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
    if exact:
        eq(g.read_field("error")[fl], o.read_field("error")[fl], "vcycle z")
    else:
        stats.setdefault("vcycle", []).append(close(g.read_field("error")[fl], o.read_field("error")[fl],
                                                    VCYCLE_RTOL, "vcycle z"))
    o.run_stage("pcg", dt)
    g.run_stage("pcg", dt)
    so, sg = o.stats(), g.stats()
    stats.setdefault("pcg_iters", []).append((sg.pcg_iterations, so.pcg_iterations))
    cells = fl - o.info().width
    p_o, p_g = o.read_field("pressure"), g.read_field("pressure")
    if exact:
        assert sg.pcg_iterations == so.pcg_iterations, (sg.pcg_iterations, so.pcg_iterations)
        eq(p_g[cells], p_o[cells], "pressure")
        stats.setdefault("pcg_p", []).append(0.0)
    else:
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


def run_lockstep(o, g, frames, frame_dt, props, cs, forces=None, exact=True):
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
            lockstep_substep(o, g, dt, first, stats, exact)
            first = False
            t = np.float32(t + np.float32(dt))
        # clear the frame's forces like Apic::update does (src/apic.rs:2470-2473)
        zu = np.zeros_like(o.read_field("ext_force_u"))
        zv = np.zeros_like(o.read_field("ext_force_v"))
        for name, z in (("ext_force_u", zu), ("ext_force_v", zv), ("post_force_u", zu), ("post_force_v", zv)):
            o.write_field(name, z)
            g.write_field(name, z)
    return stats
