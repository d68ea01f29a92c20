"""bench.py's sharded mode on the CPU: two gloo ranks (127.0.0.1) split one
series' doSplit blocks with rfba_gb300.shard, the FP64 oracle standing in for
the GPU (tests/test_shard_cpu.OracleBackend). Rank 0 prints the JSON line of
the strong-scaling run and the map it gathered (tensor gather) equals one
process's block forward bit for bit."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

KW = dict(mag=2, method=3, itc=0, trac_order=2, gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)
SHAPE = (4, 11, 10, 12)  # T, D, H, W


def _series():
    from rfba_gb300 import synth
    T, D, H, W = SHAPE
    scene = synth.make_scene(13, T, (W, H, D), 8)
    return synth.render(scene, (W, H, D), 13, np.float32)


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
    from tests.test_shard_cpu import OracleBackend
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        args = type("A", (), {"steps": 1, "warmup": 1})()
        line, out = bench.run_sharded(args, make_backend=lambda: OracleBackend(KW), series=_series(), cfg_kw=KW,
                                      block=(6, 1))
        q.put((rank, line, out))
    finally:
        dist.destroy_process_group()


def test_sharded_bench_line_and_map():
    from rfba_gb300 import srrf
    from tests.test_shard_cpu import OracleBackend
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=600) for _ in range(2)), key=lambda r: r[0])
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    line, out = res[0][1], res[0][2]
    assert res[1][1] is None and res[1][2] is None
    assert line["n_gpus"] == 2 and line["config"]["parallelism"] == "sharded" and line["scaling"] == "strong"
    assert line["value"] > 0 and line["config"]["blocks"] >= 4
    cfg = srrf.Config.make(**KW)
    x = _series()
    blocks, n, oe = srrf.blocks_dosplit(cfg, x.shape, 6, 1)
    one = OracleBackend(KW).forward_blocks(cfg, x, blocks, n, oe)
    assert np.array_equal(out.view(np.uint32), one.view(np.uint32))  # bit for bit, NaN included
