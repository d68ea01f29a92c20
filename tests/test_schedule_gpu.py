"""Autotuned schedules and CUDA-graph replay of the extended forward give the
same maps, bit for bit, as the eager default schedule and the plain per-block
path (tile shape and tile order change which CTA computes a subvoxel, never
the arithmetic of a subvoxel)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHIPPED = dict(gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(np.nan_to_num(a), np.nan_to_num(b))


@pytest.fixture
def env(monkeypatch):
    monkeypatch.setenv("RFBA_TUNE_MIN", "0")
    return monkeypatch


def _volume(T, shape, seed=3):
    from rfba_gb300 import synth
    scene = synth.make_scene(seed, T, shape, 60)
    return synth.render(scene, shape, seed, np.uint16)


@pytest.mark.parametrize("kw", [dict(mag=2, method=1), dict(mag=(3, 3, 3), method=3, itc=0, trac_order=2),
                                dict(mag=(4, 4, 2), method=3, itc=1, trac_order=2)],
                         ids=["tra_mag2", "trac2_mag3", "trac2_itc1_mag442"])
def test_tuned_graph_forward_matches_eager(ctx, env, kw):
    import torch
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(**kw, **SHIPPED)
    x = _volume(6, (24, 20, 18))
    xd = torch.from_numpy(x.view(np.int16)).cuda()
    env.setenv("RFBA_TUNE", "0")
    env.setenv("RFBA_GRAPH", "0")
    ref = ctx.forward(cfg, xd).cpu().numpy()
    assert not ctx.schedule()["graph"]
    env.delenv("RFBA_TUNE")
    env.delenv("RFBA_GRAPH")
    out = torch.empty_like(torch.from_numpy(ref)).cuda()
    ctx.forward(cfg, xd, out=out)
    s1 = ctx.schedule()
    assert s1["tuned"] and s1["graph"]
    assert _same(out.cpu().numpy(), ref)
    out.fill_(0)
    ctx.forward(cfg, xd, out=out)          # replay of the captured graph
    s2 = ctx.schedule()
    assert s2["graph"] and not s2["tuned"]
    assert _same(out.cpu().numpy(), ref)


def test_block_list_graph_matches_plain_and_pinned(ctx, env):
    import torch
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=3, method=1, **SHIPPED)
    x = _volume(5, (40, 36, 30))
    blocks, n, oe = srrf.blocks_dosplit(cfg, x.shape, 17, 1)
    plain = np.zeros(oe, np.float32)
    ctx.forward_blocks_plain(cfg, x, blocks, n, oe, out=plain)
    xd = torch.from_numpy(x.view(np.int16)).cuda()
    outd = torch.empty(oe, dtype=torch.float32, device="cuda")
    for _ in range(2):
        ctx.forward_blocks(cfg, xd, blocks, n, oe, out=outd)
        assert ctx.schedule()["graph"]
        assert _same(outd.cpu().numpy(), plain)
    pin_in = torch.empty(x.nbytes, dtype=torch.uint8).pin_memory().numpy().view(np.uint16).reshape(x.shape)
    pin_in[...] = x
    pin_out = torch.empty(oe, dtype=torch.float32).pin_memory().numpy()
    for _ in range(2):
        pin_out[:] = 0
        ctx.forward_blocks(cfg, pin_in, blocks, n, oe, out=pin_out)
        assert ctx.schedule()["graph"]
        assert _same(pin_out, plain)
    # pageable host buffers run eagerly
    page_out = np.zeros(oe, np.float32)
    ctx.forward_blocks(cfg, x, blocks, n, oe, out=page_out)
    assert not ctx.schedule()["graph"]
    assert _same(page_out, plain)


def test_graph_rebuilt_after_scratch_grows(ctx, env):
    """A larger call reallocates the scratch the first graph was captured on;
    replaying the first call again must not use the stale graph."""
    import torch
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=2, method=1, **SHIPPED)
    small = _volume(4, (16, 16, 12))
    big = _volume(8, (32, 28, 24), seed=4)
    sd = torch.from_numpy(small.view(np.int16)).cuda()
    bd = torch.from_numpy(big.view(np.int16)).cuda()
    env.setenv("RFBA_GRAPH", "0")
    ref_small = ctx.forward(cfg, sd).cpu().numpy()
    env.delenv("RFBA_GRAPH")
    o1 = ctx.forward(cfg, sd)
    assert _same(o1.cpu().numpy(), ref_small)
    ctx.forward(cfg, bd)
    o1.fill_(0)
    ctx.forward(cfg, sd, out=o1)
    assert _same(o1.cpu().numpy(), ref_small)


def test_graph_replay_reports_kernel_times(ctx, env):
    """Kernel times of a replayed graph come from event nodes inside it."""
    import torch
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=2, method=1, **SHIPPED)
    x = _volume(4, (24, 24, 16))
    xd = torch.from_numpy(x.view(np.int16)).cuda()
    ctx.set_timing(True)
    try:
        for _ in range(3):
            ctx.forward(cfg, xd)
            t = ctx.timing()
            assert ctx.schedule()["graph"]
            assert t.radiality_ms > 0 and t.temporal_ms > 0
    finally:
        ctx.set_timing(False)


@pytest.mark.parametrize("T", [1, 2, 13])
def test_pinned_forward_with_windowed_input_copy(ctx, env, T):
    """With pinned host buffers the captured forward copies the first tenth of
    the volumes, then the rest on a second stream while the first window's
    radiality runs; the map equals the one from a single input copy
    (RFBA_OVERLAP=0) and from device buffers, bit for bit."""
    import torch
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=(4, 4, 2), method=3, itc=0, trac_order=2, intensity_w=1, **SHIPPED)
    x = _volume(T, (20, 18, 14), seed=9)
    xd = torch.from_numpy(x.view(np.int16)).cuda()
    ref = ctx.forward(cfg, xd).cpu().numpy()
    pin_in = torch.empty(x.nbytes, dtype=torch.uint8).pin_memory().numpy().view(np.uint16).reshape(x.shape)
    pin_in[...] = x
    pin_out = torch.empty(ref.size, dtype=torch.float32).pin_memory().numpy().reshape(ref.shape)
    for overlap in ("1", "0", "1"):
        env.setenv("RFBA_OVERLAP", overlap)
        for _ in range(2):  # capture, then replay
            pin_out[...] = 0
            ctx.forward(cfg, pin_in, out=pin_out)
            assert ctx.schedule()["graph"]
            assert _same(pin_out, ref), (T, overlap)
