"""Region entry points and the shard partition on one GPU, through the C-ABI.

- rfba_srrf_forward_shifted_region equals the same region of the whole-map
  forward; rfba_srrf_backward_region is linear in the map: the contributions of
  z slabs that tile the map sum to rfba_srrf_backward's dL/din and dL/dshifts.
- rfba_gb300.shard's block partition, run rank by rank on this GPU (the ranks'
  launches are independent, none waits on another), puts back the same map as
  one rfba_srrf_forward_blocks over all blocks.
- The sharded drift loop with one process equals rfba_gb300.drift's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHIPPED = dict(gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)
CASES = [
    ("trac2_mag2", dict(mag=2, method=3, itc=0, trac_order=2, **SHIPPED), (7, 9, 10, 11)),
    ("tra_mag442", dict(mag=(4, 4, 2), method=1, **SHIPPED), (5, 9, 7, 8)),
]


def _case(seed, T, D, H, W):
    from rfba_gb300 import synth
    scene = synth.make_scene(seed, T, (W, H, D), 10)
    x = synth.render(scene, (W, H, D), seed, np.float32)
    sh = np.random.default_rng(seed).normal(0, 0.3, size=(T, 3)).astype(np.float32)
    return x, sh


@pytest.mark.parametrize("name,kw,shape", CASES, ids=[c[0] for c in CASES])
def test_regions_tile_the_pair(ctx, name, kw, shape):
    import torch
    from rfba_gb300 import shard, srrf
    cfg = srrf.Config.make(**kw)
    x, sh = _case(3 + len(name), *shape)
    xd, sd = torch.from_numpy(x).cuda(), torch.from_numpy(sh).cuda()
    T, D, H, W = shape
    m = ctx.forward_shifted(cfg, xd, sd).clone()
    g = torch.randn(m.shape, generator=torch.Generator().manual_seed(1)).cuda()
    din, dsh = ctx.backward(cfg, xd, sd, g)
    din, dsh = din.clone(), dsh.clone()
    Wf, Hf, Zf = W * cfg.mag[0], H * cfg.mag[1], D * cfg.mag[2]
    sin = torch.zeros_like(din)
    ssh = torch.zeros_like(dsh)
    for z0, z1 in shard.z_slabs(Zf, 3):
        lo, hi = (0, 0, z0), (Wf, Hf, z1)
        r = ctx.forward_shifted_region(cfg, xd, sd, lo, hi)
        torch.testing.assert_close(r, m[z0:z1], rtol=1e-6, atol=1e-6, equal_nan=True)
        a, b = ctx.backward_region(cfg, xd, sd, lo, hi, g[z0:z1].contiguous())
        sin += a
        ssh += b
    # an interior box: the forward region only
    lo, hi = (3, 2, 1), (Wf - 2, Hf - 3, Zf - 1)
    r = ctx.forward_shifted_region(cfg, xd, sd, lo, hi)
    torch.testing.assert_close(r, m[1:Zf - 1, 2:Hf - 3, 3:Wf - 2], rtol=1e-6, atol=1e-6, equal_nan=True)
    torch.cuda.synchronize()
    scale_in = din.abs().max().item()
    assert (sin - din).abs().max().item() <= 1e-4 * scale_in
    scale_sh = dsh.abs().max().item()
    assert (ssh - dsh).abs().max().item() <= 1e-4 * scale_sh, (ssh, dsh)


def test_region_rejects_bad_boxes(ctx):
    import torch
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=2, method=1, **SHIPPED)
    x, sh = _case(1, 3, 6, 6, 6)
    xd = torch.from_numpy(x).cuda()
    for lo, hi in [((0, 0, 0), (13, 12, 12)), ((0, 0, 5), (12, 12, 5)), ((-1, 0, 0), (4, 4, 4))]:
        with pytest.raises(srrf.RfbaError, match="region"):
            ctx.forward_shifted_region(cfg, xd, None, lo, hi,
                                       out=torch.empty(1024, device="cuda"))


@pytest.mark.parametrize("world", [2, 3, 8])
def test_block_partition_puts_back_the_map(ctx, world):
    """Each rank computes its blocks from its own input box (shard.crop: the
    union of its blocks' sub-volumes with their halos, origins rebased to the
    box). With 8 ranks one rank's box starts off the origin on every axis."""
    import torch
    from rfba_gb300 import shard, srrf
    cfg = srrf.Config.make(mag=2, method=3, itc=0, trac_order=2, block_size=(12, 12, 12), **SHIPPED)
    T, D, H, W = 6, 20, 18, 22
    x, _ = _case(9, T, D, H, W)
    xd = torch.from_numpy(x).cuda()
    blocks, n = srrf.blocks_gradientcalc(cfg, x.shape)
    total = D * H * W * 8
    one = ctx.forward_blocks(cfg, xd, blocks, n, total).cpu().numpy()
    out = np.zeros(total, np.float32)
    box_lo = []
    for r in range(world):
        idx, packed = shard.forward_local(ctx, cfg, xd, blocks, n, r, world)
        if idx:
            box_lo.append(shard.input_box(blocks, idx)[0])
        shard.put_back(out, blocks, idx, packed)
    np.testing.assert_array_equal(out, one)
    if world == 8:
        assert any(all(v > 0 for v in lo) for lo in box_lo), box_lo


def test_sharded_drift_one_process_equals_drift(ctx):
    import torch
    from rfba_gb300 import drift, shard, srrf
    cfg = srrf.Config.make(mag=2, method=3, itc=0, trac_order=2, **SHIPPED)
    x, sh = _case(4, 6, 8, 9, 10)
    xd = torch.from_numpy(x).cuda()
    a, ma = drift.refine_drift(ctx, cfg, xd, iters=3, start=sh)
    b, mb, zr = shard.refine_drift_sharded(ctx, cfg, xd, iters=3, start=sh)
    assert zr == (0, 16)
    np.testing.assert_allclose(b.shifts, a.shifts, rtol=0, atol=1e-5)
    torch.testing.assert_close(mb, ma, rtol=1e-4, atol=1e-4, equal_nan=True)
