"""The multi-rank rules of bench.py (replicas: every rank times its own copy of the workload,
the job takes the slowest rank's time, rank 0 reports; the reference arm runs on rank 0 only),
exercised with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, loc = bench.dist_env()
    t = bench.max_over_ranks(1.0 + rank, dist)      # rank 1 is the slower replica
    rate = bench.job_rate(10_000 * 5, w, t)
    dist.barrier()
    out.put((r, w, loc, t, rate))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[:3] for r in res] == [(0, 2, 0), (1, 2, 1)]
    assert all(r[3] == 2.0 for r in res)                      # both ranks see the max
    assert all(r[4] == pytest.approx(2 * 50_000 / 2.0) for r in res)


def test_single_rank_helpers():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.job_rate(100, 1, 0.5) == 200


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    called = []
    monkeypatch.setattr(bench, "make_data", lambda: called.append(1))
    assert bench.run_reference(None) is None and not called   # rank 1 exits without work
