"""Independent scenes on several GPUs: placement by apic_place_scenes (a
memory-budget bin packer) and a run with no collective on the data path.

The packer is host code of the C-ABI and runs here on the CPU.  The two-rank
test runs the host-side multi-GPU path as two gloo ranks on the CPU: both
ranks compute the same placement, each steps only its own scenes (with the
oracle, as no GPU is present), and rank 0 gathers the results, which equal a
single-process run of every scene."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_place_scenes_budgets_balance_and_rejects(gpu_lib):
    import apic_gb300 as A
    rng = np.random.default_rng(3)
    sizes = [int(x) for x in rng.integers(1 << 20, 1 << 26, 200)]
    work = [int(x) for x in rng.integers(1000, 200000, 200)]
    budgets = [1 << 31, 1 << 31, 3 << 29, 1 << 32]
    where = A.place_scenes(sizes, work, budgets)
    assert where == A.place_scenes(sizes, work, budgets)  # deterministic
    used = [0] * len(budgets)
    for b, d in zip(sizes, where):
        assert d >= 0
        used[d] += b
    assert all(u <= cap for u, cap in zip(used, budgets))
    # ample memory: largest-first onto the least-loaded device keeps the loads
    # within one scene's work of each other
    where = A.place_scenes(sizes, work, [1 << 40] * 4)
    load = [sum(w for w, d in zip(work, where) if d == k) for k in range(4)]
    assert max(load) - min(load) <= max(work)
    # a scene larger than every budget is not placed; the others still are
    where = A.place_scenes([5, 100, 5], [1, 1, 1], [50, 60])
    assert where[1] == -1 and where[0] >= 0 and where[2] >= 0
    assert A.place_scenes([], [], [10]) == []
    with pytest.raises(A.ApicError):
        A.place_scenes([1], [1], [])


def _scenes(A):
    out = []
    for i, side in enumerate((16, 24, 32, 16, 32, 24, 16)):
        out.append(A.scene_params(A.SCENE_DAM_BREAK, side, cell_size=1.0 / side, sub=2, seed=50 + i,
                                  fluid_x=0.5, fluid_y=0.6))
    return out


def _run_scene(A, oracle, sc, updates=2):
    px, py, vx, vy = oracle.generate_scene(sc)
    o = oracle.OracleSim(sc.width, sc.height, sc.cell_size, A.WorldProperties(-9.81, 0.1, 5.0, 1e-5))
    o.set_particles(px, py, vx, vy)
    for _ in range(updates):
        o.update(A.DebugOptions(), 1.0 / 240)
    n = len(px)
    return float(np.sum(o.read_field("pos_x")[:n], dtype=np.float64) +
                 np.sum(o.read_field("pos_y")[:n], dtype=np.float64))


def _rank_main(rank, world, port, out_dir):
    os.environ["CUDA_VISIBLE_DEVICES"] = ""
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "apic-fluid-simulation_gb300"))
    import bench
    import apic_gb300 as A
    from oracle import oracle
    w, r, _ = bench.dist_setup()
    scenes = _scenes(A)
    where = bench.place_on_ranks(A, scenes, w, 1 << 40)
    mine = {i: _run_scene(A, oracle, sc) for i, sc in enumerate(scenes) if where[i] == r}
    import torch.distributed as dist
    got = [None] * w if r == 0 else None
    dist.gather_object((r, mine, where), got, dst=0)
    if r == 0:
        with open(os.path.join(out_dir, "gathered.txt"), "w") as f:
            f.write(repr(got))
    dist.destroy_process_group()


def test_two_gloo_ranks_place_run_and_gather(tmp_path, gpu_lib, oracle_mod):
    mp = pytest.importorskip("torch.multiprocessing")
    import apic_gb300 as A
    world, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True, start_method="spawn")
    got = eval((tmp_path / "gathered.txt").read_text())
    scenes = _scenes(A)
    results, placements = {}, []
    for r, mine, where in got:
        placements.append(where)
        for i in mine:
            assert where[i] == r and i not in results
        results.update(mine)
    assert placements[0] == placements[1]  # the same placement on every rank, no exchange needed
    assert set(placements[0]) == {0, 1}  # both ranks got work
    assert sorted(results) == list(range(len(scenes)))
    for i, sc in enumerate(scenes):
        assert results[i] == _run_scene(A, oracle_mod, sc)
