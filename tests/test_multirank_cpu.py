"""bench.py's multi-rank logic on CPU: two gloo ranks (one per process), each a replica.

The BVE path does not shard (solves are independent), so N GPUs run N replicas; the job's
time is the slowest rank's and its rate is N x per-rank units over that time.
"""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    elapsed = 100.0 + 50.0 * rank           # rank 1 is the slow replica
    m = bench.max_over_ranks(elapsed, world)
    rate = bench.whole_job_rate(world, 10, m)
    q.put((rank, m, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_take_the_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, m, rate in res:
        assert m == 150.0
        assert rate == pytest.approx(2 * 10 / 0.150)


def test_reference_arm_nonzero_ranks_do_nothing(capsys, monkeypatch):
    import bench
    monkeypatch.setattr("sys.argv", ["bench.py", "--impl", "reference"])
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    bench.main()
    assert capsys.readouterr().out == ""
