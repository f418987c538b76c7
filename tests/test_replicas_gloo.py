"""Replica aggregation (dgc_gb300.replicas) over a world_size-2 gloo process
group on the CPU: the max over ranks and the job throughput bench.py reports
under torchrun."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as tdist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from dgc_gb300 import replicas  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    tdist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        my_ms = [3.0, 5.0][rank]                     # the second rank is slower
        slow = replicas.max_over_ranks(my_ms, device="cpu")
        q.put((rank, replicas.world(), slow,
               replicas.job_throughput(units_per_rank=1e9, seconds_slowest=slow * 1e-3, world_size=ws)))
        tdist.barrier()
    finally:
        tdist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time_and_job_throughput():
    ws, port = 2, free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=10) for _ in range(ws))
    for rank, (w, r), slow, thr in got:
        assert (w, r) == (ws, rank)
        assert slow == 5.0
        assert thr == pytest.approx(2 * 1e9 / 5e-3)


def test_single_process_is_identity():
    assert replicas.world() == (1, 0)
    assert replicas.max_over_ranks(7.5) == 7.5
    assert replicas.job_throughput(10.0, 2.0, 1) == 5.0
    with pytest.raises(ValueError):
        replicas.job_throughput(1.0, 0.0, 1)
