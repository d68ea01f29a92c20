"""rfba_gb300.shard on the CPU: the block partition and its put-back, and the
z-slab drift refinement over two gloo ranks (127.0.0.1), with the FP64 oracle
standing in for the GPU (an `OracleBackend` with the Context methods the shard
code calls). The sharded results must equal one process's: the same map
bit for bit, the same shifts up to the order of the partial sums."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

KW = dict(mag=2, method=3, itc=0, trac_order=2, gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1,
          block_size=(7, 7, 7))
SHAPE = (4, 9, 8, 8)  # T, D, H, W


class OracleBackend:
    """The Context methods used by rfba_gb300.shard, computed by the oracle
    (FP64, results returned as float32 tensors)."""

    def __init__(self, kw):
        from oracle import oracle as O
        self.O = O
        self.conf = O.make_conf(**kw)

    def _np(self, t):
        return None if t is None else t.detach().cpu().numpy()

    def forward_shifted(self, cfg, x, sh, out=None, stream=None):
        import torch
        return torch.from_numpy(self.O.forward_shifted(self._np(x), self.conf, self._np(sh)).astype(np.float32))

    def backward(self, cfg, x, sh, g, stream=None):
        import torch
        _, din, dsh = self.O.adjoint(self._np(x), self.conf, self._np(g), self._np(sh))
        return torch.from_numpy(din.astype(np.float32)), torch.from_numpy(dsh.astype(np.float32))

    def forward_shifted_region(self, cfg, x, sh, lo, hi, out=None, stream=None):
        full = self.forward_shifted(cfg, x, sh)
        return full[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]].contiguous()

    def backward_region(self, cfg, x, sh, lo, hi, g, stream=None):
        import torch
        T, D, H, W = x.shape
        m = self.conf.mag
        G = torch.zeros((D * m[2], H * m[1], W * m[0]), dtype=torch.float32)
        G[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] = g
        return self.backward(cfg, x, sh, G)

    def forward_blocks(self, cfg, x, blocks, n, out_elems, out=None, stream=None):
        x = self._np(x) if not isinstance(x, np.ndarray) else x
        out = np.zeros(out_elems, np.float32) if out is None else out
        for k in range(n):
            b = blocks[k]
            o, s = list(b.origin), list(b.size)
            sub = x[:, o[2]:o[2] + s[2], o[1]:o[1] + s[1], o[0]:o[0] + s[0]]
            r = self.O.srrf_region(sub, self.conf, list(b.lo), list(b.hi)).astype(np.float32)
            nz, ny, nx = r.shape
            idx = (b.out_offset + np.arange(nz)[:, None, None] * b.out_stride[2] +
                   np.arange(ny)[None, :, None] * b.out_stride[1] + np.arange(nx)[None, None, :] * b.out_stride[0])
            out[idx.reshape(-1)] = r.reshape(-1)
        return out


def _series(seed=5):
    from rfba_gb300 import synth
    T, D, H, W = SHAPE
    scene = synth.make_scene(seed, T, (W, H, D), 8)
    x = synth.render(scene, (W, H, D), seed, np.float32)
    sh = np.random.default_rng(seed).normal(0, 0.3, size=(T, 3)).astype(np.float32)
    return x, sh


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_balance_and_slabs():
    from rfba_gb300 import shard
    costs = [7, 3, 9, 1, 4, 4, 8, 2]
    parts = shard.balance(costs, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    # longest-first greedy is within max(cost) of the mean load
    assert max(loads) - sum(costs) / 3 <= max(costs)
    assert shard.balance(costs, 1) == [list(range(len(costs)))]
    assert shard.balance([], 2) == [[], []]
    with pytest.raises(ValueError):
        shard.balance(costs, 0)
    assert shard.z_slabs(10, 3) == [(0, 4), (4, 7), (7, 10)]
    assert shard.z_slabs(2, 4) == [(0, 1), (1, 2), (2, 2), (2, 2)]


@pytest.mark.parametrize("split", ["gradientcalc", "dosplit"])
def test_repack_put_back_identity(split):
    """Packing any subset of blocks and putting it back reproduces the writes
    of the original block list: GradientCalc's blocks put back into the whole
    map, doSplit's written one after another."""
    from rfba_gb300 import shard, srrf
    cfg = srrf.Config.make(**KW)
    if split == "gradientcalc":
        blocks, n = srrf.blocks_gradientcalc(cfg, SHAPE)
        total = SHAPE[1] * SHAPE[2] * SHAPE[3] * 8
    else:
        blocks, n, total = srrf.blocks_dosplit(cfg, SHAPE, 5, 1)
    assert n >= 4
    ref = np.zeros(total, np.float32)
    rng = np.random.default_rng(0)
    vals = []
    for k in range(n):  # a distinct value per block region, written by stride
        b = blocks[k]
        nx, ny, nz = (b.hi[a] - b.lo[a] for a in range(3))
        v = rng.standard_normal(nx * ny * nz).astype(np.float32)
        vals.append(v)
        shard.put_back(ref, blocks, [k], v)
    for world in (2, 3):
        out = np.zeros(total, np.float32)
        for idx in shard.balance([shard.block_cost(blocks[k], 4) for k in range(n)], world):
            sub, m, elems = shard.repack(blocks, idx)
            assert elems == sum(len(vals[k]) for k in idx)
            packed = np.concatenate([vals[k] for k in idx]) if idx else np.zeros(0, np.float32)
            for j in range(m):  # the packed layout: offsets in order, [z][y][x]
                assert sub[j].out_stride[0] == 1
            shard.put_back(out, blocks, idx, packed)
        np.testing.assert_array_equal(out, ref)


@pytest.mark.parametrize("world", [2, 3, 5])
def test_rank_input_box(world):
    """Each rank's share computed from its cropped input box equals the same
    blocks computed from the whole series, and the box is smaller than the
    series once the blocks are spread over ranks."""
    from rfba_gb300 import shard, srrf
    be = OracleBackend(KW)
    cfg = srrf.Config.make(**KW)
    x, _ = _series()
    blocks, n = srrf.blocks_gradientcalc(cfg, SHAPE)
    T = SHAPE[0]
    boxes = 0
    for r in range(world):
        idx, packed = shard.forward_local(be, cfg, x, blocks, n, r, world)
        if not idx:
            continue
        sub, m, elems = shard.repack(blocks, idx)
        np.testing.assert_array_equal(packed, be.forward_blocks(cfg, x, sub, m, elems))
        lo, hi = shard.input_box(blocks, idx)
        xs, sub2, _, _ = shard.crop(x, blocks, idx)
        assert xs.shape == (T, hi[2] - lo[2], hi[1] - lo[1], hi[0] - lo[0])
        for k in range(m):
            for a in range(3):
                assert 0 <= sub2[k].origin[a] and sub2[k].origin[a] + sub2[k].size[a] <= xs.shape[3 - a]
        boxes += xs.size
    assert boxes > 0


def _rank(rank, ws, port, ckpt, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch
    import torch.distributed as dist
    from rfba_gb300 import shard, srrf
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        be = OracleBackend(KW)
        cfg = srrf.Config.make(**KW)
        x, sh = _series()
        blocks, n = srrf.blocks_gradientcalc(cfg, SHAPE)
        T, D, H, W = SHAPE
        full = shard.forward_sharded(be, cfg, x, blocks, n, D * H * W * 8)
        st, m, zr = shard.refine_drift_sharded(be, cfg, torch.from_numpy(x), iters=3, start=sh, checkpoint=ckpt)
        q.put((rank, full, st.shifts, st.it, m.numpy(), zr))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_match_one_process(tmp_path):
    import torch
    from rfba_gb300 import drift, srrf
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ckpt = str(tmp_path / "drift.npz")
    procs = [ctx.Process(target=_rank, args=(r, 2, port, ckpt, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=300) for _ in range(2)], key=lambda r: r[0])
    for p in procs:
        p.join(60)
        assert p.exitcode == 0

    be = OracleBackend(KW)
    cfg = srrf.Config.make(**KW)
    x, sh = _series()
    blocks, n = srrf.blocks_gradientcalc(cfg, SHAPE)
    T, D, H, W = SHAPE
    one = be.forward_blocks(cfg, x, blocks, n, D * H * W * 8)
    np.testing.assert_array_equal(res[0][1], one)  # the gathered map, bit for bit
    assert res[1][1] is None

    st1, m1 = drift.refine_drift(be, cfg, torch.from_numpy(x), iters=3, start=sh, stream=0)
    np.testing.assert_array_equal(res[0][2], res[1][2])  # every rank took the same steps
    np.testing.assert_allclose(res[0][2], st1.shifts, rtol=0, atol=1e-5)
    assert res[0][3] == 3
    slabs = [r[4] for r in res]
    assert [r[5] for r in res] == [(0, 9), (9, 18)]
    np.testing.assert_allclose(np.concatenate(slabs, 0), m1.numpy(), rtol=1e-4, atol=1e-4)
    saved = drift.DriftState.load(ckpt)
    np.testing.assert_array_equal(saved.shifts, res[0][2])
    assert saved.it == 3
