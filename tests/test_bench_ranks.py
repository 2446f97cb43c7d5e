"""bench.py's multi-rank path on the CPU.  Under torchrun every rank runs an independent
replica of the workload (the lattice is not sharded); the job's time is the slowest
rank's, and the whole-job rate counts every rank's fluid-node updates over that time.
Two gloo ranks stand in for the GPUs here; the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")

import bench  # noqa: E402


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(times[rank], dist, "cpu")
        with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
            f.write(repr(t))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_agree_on_the_slowest_time(tmp_path):
    import torch.multiprocessing as mp
    world, times = 2, [1.25, 2.5]
    mp.spawn(_rank_main, args=(world, _free_port(), times, str(tmp_path)), nprocs=world, join=True)
    got = [float((tmp_path / f"rank{r}.txt").read_text()) for r in range(world)]
    assert got == [2.5, 2.5]
    # 2 replicas x 1 M fluid nodes x 20 steps over the slowest rank's 2.5 s
    assert bench.whole_job_mlups(1_000_000, 20, world, got[0]) == pytest.approx(16.0)


def test_single_process_keeps_its_own_time():
    assert bench.max_over_ranks(3.0) == 3.0
    assert bench.whole_job_mlups(3_689_484, 20, 1, 0.023) == pytest.approx(3_689_484 * 20 / 0.023 / 1e6)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    args = bench.parse()
    assert bench.run_reference(args) == 0     # returns before building any workload
