"""The N > 1 path of bench.py on CPU: two gloo ranks (127.0.0.1), the slowest
rank's time decides, the job rate counts every rank's units (replicas, weak
scaling), and the reference arm does its work on rank 0 only."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        t = bench.max_over_ranks(1.0 + rank)  # rank 1 is the slow one
        rate = bench.whole_job_rate(1000.0, ws, t)
        ref = bench.run_reference(type("A", (), {"steps": 1, "warmup": 0})()) if rank == 1 else "skipped"
        q.put((rank, t, rate, ref))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t, rate, ref in res:
        assert t == 2.0  # max over ranks
        assert rate == pytest.approx(1000.0 * 2 / 2.0)
    assert res[1][3] is None  # rank 1 of the reference arm returns without work


def test_single_process_identity():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(10.0, 1, 2.0) == 5.0
