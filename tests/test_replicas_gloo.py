"""Multi-GPU runs are independent replicas (hmpano/replicas.py): barriers around the timed region,
the per-step time is the maximum over ranks, the job's rate counts every rank's units. The
multi-rank path runs here as two gloo processes on the CPU (127.0.0.1 rendezvous)."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank: int, world: int, port: int, out) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from hmpano import replicas

    r = replicas.init("gloo")
    r.barrier()
    slowest = r.max_over_ranks(1.5 + rank)  # rank 1 is the slow replica
    rate = r.job_rate(10.0, 2.0)
    r.barrier()
    out.put((rank, r.world, slowest, rate))
    r.close()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(rank, 2, port, q)) for rank in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in results] == [0, 1]
    for _, world, slowest, rate in results:
        assert world == 2
        assert slowest == pytest.approx(2.5)  # the maximum over both ranks, on every rank
        assert rate == pytest.approx(10.0)    # 2 ranks x 10 units / 2 s


def test_single_process_is_local(monkeypatch):
    from hmpano import replicas

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    r = replicas.init("gloo")
    assert (r.rank, r.world) == (0, 1)
    r.barrier()
    assert r.max_over_ranks(3.25) == 3.25
    assert r.job_rate(8.0, 2.0) == 4.0
    r.close()
