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


def test_reference_arm_json_line(capsys, monkeypatch):
    """The reference arm's line (CPU oracle, small mesh): the GPU arm's metric, unit and workload,
    a cpu_baseline describing the run and an e2e block with no host-device traffic."""
    import json

    import bench
    monkeypatch.setattr("sys.argv", ["bench.py", "--impl", "reference", "--level", "3", "--steps", "1",
                                     "--warmup", "0"])
    monkeypatch.delenv("RANK", raising=False)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    bench.main()
    lines = [line for line in capsys.readouterr().out.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "RK4 steps/s" and d["unit"] == "steps/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 0
    assert d["value"] > 0 and d["ms_per_step"] == pytest.approx(1000.0 / d["value"])
    # the same config object as the GPU arm's line (level 3 instead of the default 8)
    assert d["config"] == bench.bench_config(bench.workload("c5", 3), 1)
    assert d["steps_kind"].startswith("sampled evaluations")
    fc = d["full_evaluation_check"]
    assert fc["level"] == 3 and fc["pairs_per_s"] > 0 and fc["sample_over_full"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
