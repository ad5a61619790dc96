"""Scenarios run through a given build of the library (the default one, or
the bounds-checked one in a child process): returns every result array."""
import numpy as np

import apic_gb300 as A


def run_all():
    out = {}
    props = A.WorldProperties(-9.81, 0.1, 5.0, 1e-5)
    side = 128
    cs = 1.0 / side
    sc = A.scene_params(A.SCENE_DAM_BREAK, side, cell_size=cs, sub=2, seed=0, fluid_x=0.4, fluid_y=0.6)
    px, py, vx, vy = A.generate_scene(sc)
    for name, mode, opts in (("mixed", A.SOLVER_REL_MIXED, A.DebugOptions()),
                             ("reference", A.SOLVER_REFERENCE, A.DebugOptions()),
                             ("nosort", A.SOLVER_REL_MIXED, A.DebugOptions(disable_particle_sort=True))):
        g = A.Apic(side, side, cs, props)
        g.set_particles(px, py, vx, vy)
        g.set_solver(mode, 1e-6, 500)
        g.add_radial_force(0.3, 0.3, 0.05, 100.0)
        for _ in range(3):
            g.update(opts, 1 / 240)
        for f in A.PARTICLE_FIELDS + ["u", "v", "pressure", "density"]:
            out[f"{name}_{f}"] = g.read_field(f).copy()
        g.close()
    # dense and degenerate particles: the banded and the global-memory P2G paths
    rng = np.random.default_rng(5)
    side = 64
    cs = 1.0 / side
    m = 6000
    qx = np.concatenate([np.full(m, 0.3, np.float32) + rng.uniform(0, 0.5 * cs, m).astype(np.float32),
                         rng.uniform(-0.5, 1.5, 500).astype(np.float32),
                         np.array([np.inf, -np.inf, 1e10, -3e9, 0.0, 1.0], np.float32)])
    qy = np.concatenate([np.full(m, 0.6, np.float32) + rng.uniform(0, 0.5 * cs, m).astype(np.float32),
                         rng.uniform(-0.5, 1.5, 500).astype(np.float32),
                         np.array([0.5, 0.5, 0.5, 0.5, 1.0, 0.0], np.float32)])
    for name, mode in (("dense_ref", A.SOLVER_REFERENCE), ("dense_mixed", A.SOLVER_REL_MIXED)):
        g = A.Apic(side, side, cs, props)
        g.set_particles(qx, qy)
        g.set_solver(mode, 1e-6, 500)
        g.run_stage("p2g", 1 / 240)
        for f in ("u", "v", "density", "valid_u", "valid_v", "fluid_bits"):
            out[f"{name}_{f}"] = g.read_field(f).copy()
        g.close()
    return out


if __name__ == "__main__":
    import sys
    A.load_library(sys.argv[1])
    np.savez(sys.argv[2], **run_all())
