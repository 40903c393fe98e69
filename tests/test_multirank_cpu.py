"""The bench's multi-rank plumbing on CPU: two gloo ranks (127.0.0.1), each a
replica of the workload; the job time is the max over ranks and the job rate is
all replicas' units over that time.  The hot path itself does not shard (one
GPU per replica, no data-path collective)."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    local_time = 1.5 + rank  # rank 1 is the slow replica
    t = bench.max_over_ranks(local_time, world, device="cpu")
    rate = bench.job_rate(1024 * 20, world, t)
    dist.barrier()
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as fh:
        fh.write(f"{t} {rate}")
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_max_over_ranks_and_job_rate_gloo(tmp_path):
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    vals = [tuple(map(float, (tmp_path / f"r{r}.txt").read_text().split())) for r in range(world)]
    for t, rate in vals:
        assert t == 2.5
        assert rate == pytest.approx(1024 * 20 * world / 2.5)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.25, 1) == 3.25
    assert bench.job_rate(100, 1, 2.0) == 50.0
