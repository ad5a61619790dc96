"""The multi-GPU form of the bench is N independent replicas: one process per
GPU, no collective on the data path, a barrier around the timed region and
the maximum of the ranks' times.  These tests run that host-side path as two
gloo ranks on the CPU (no GPU, no kernels)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    # CPU ranks on gloo wherever the test runs (CUDA reads this at first use)
    os.environ["CUDA_VISIBLE_DEVICES"] = ""
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.dist_barrier(w)
    # each replica's device seconds differ; every rank sees the slowest
    got = bench.dist_max(1.5 + rank, w)
    # the reference arm runs on rank 0 only: the other ranks return at once
    class Args:
        steps, warmup, gpus = 1, 0, world
    if rank != 0:
        assert bench.run_reference_arm(Args(), w, r) is None
    bench.dist_barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(repr(got))


def test_two_gloo_replicas_take_the_max(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True, start_method="spawn")
    for rank in range(world):
        assert float((tmp_path / f"rank{rank}.txt").read_text()) == 2.5


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        assert bench.dist_setup() == (1, 0, 0)
        assert bench.dist_max(3.25, 1) == 3.25
        bench.dist_barrier(1)
    finally:
        os.environ.update(env)
