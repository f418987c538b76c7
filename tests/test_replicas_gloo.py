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


def test_gpu_local_cpus_from_sysfs(tmp_path):
    from dgc_gb300 import replicas
    dev = tmp_path / "bus" / "pci" / "devices" / "0009:01:00.0"
    dev.mkdir(parents=True)
    (dev / "numa_node").write_text("1\n")
    node = tmp_path / "devices" / "system" / "node" / "node1"
    node.mkdir(parents=True)
    (node / "cpulist").write_text("72-75,80,90-91\n")
    assert replicas.gpu_local_cpus("00000009:01:00.0", sysfs=str(tmp_path)) == {72, 73, 74, 75, 80, 90, 91}
    (dev / "numa_node").write_text("-1\n")
    assert replicas.gpu_local_cpus("00000009:01:00.0", sysfs=str(tmp_path)) == set()
    assert replicas.gpu_local_cpus("00000001:02:00.0", sysfs=str(tmp_path)) == set()


def test_bind_local_cpus_without_gpu_changes_nothing():
    import os
    from dgc_gb300 import replicas
    before = os.sched_getaffinity(0)
    assert replicas.bind_local_cpus(0) == [] or set(replicas.bind_local_cpus(0)) <= before
    assert os.sched_getaffinity(0) <= before
