"""The multi-rank path of bench.py on CPU: two gloo ranks, each timing its own
replica; the job time is the slowest rank's and the throughput counts every
rank's bytes (weak scaling, no data-path collective)."""
import os
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    local_ms = [4.0, 5.0][rank]
    ms = bench.max_over_ranks(local_ms, dist, "cpu")
    q.put((rank, ms, bench.whole_job_gbs(32_214_089_728, world, ms)))
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_take_max_and_sum_bytes():
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=100) for _ in range(2)]
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    for _, ms, gbs in res:
        assert ms == 5.0
        assert abs(gbs - 32_214_089_728 * 2 / 5e-3 / 1e9) < 1e-6


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert torch.tensor(bench.whole_job_gbs(1e9, 1, 1.0)).item() == pytest.approx(1000.0)
