"""Bounds and determinism checks that need no sanitizer: canary-filled output
arrays (a block list written with gaps between its rows and planes and guard
regions around it must leave every gap and guard untouched and write every
target element), and repeated calls (the forward is bit-for-bit repeatable; the
adjoint's scatter adds in float atomics, so repeated backwards agree to
rounding)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SMOOTH = dict(gradient_smooth=1, x_range=1, y_range=1, z_range=1)
CANARY = np.frombuffer(np.uint32(0x7FC0DEAD).tobytes(), np.float32)[0]  # a NaN payload no kernel writes


def _series(seed, T, D, H, W, dtype=np.uint16):
    from rfba_gb300 import synth
    scene = synth.make_scene(seed, T, (W, H, D), 10)
    return synth.render(scene, (W, H, D), seed, dtype)


def test_block_outputs_touch_only_their_elements(ctx):
    import torch
    from rfba_gb300.srrf import Block, Config
    cfg = Config.make(mag=2, method=3, itc=0, trac_order=2, **SMOOTH)
    x = _series(3, 5, 12, 13, 14)
    regions = [((0, 0, 0), (14, 13, 12), (2, 3, 1), (22, 21, 17)),
               ((3, 2, 4), (9, 10, 7), (0, 0, 0), (18, 20, 14))]
    b = (Block * 2)()
    guard, off, targets = 1000, 1000, []
    for i, (org, size, lo, hi) in enumerate(regions):
        nx, ny, nz = hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]
        sx, sy = nx + 3, (nx + 3) * (ny + 2)  # gaps after every row and plane
        b[i].origin[:], b[i].size[:], b[i].lo[:], b[i].hi[:] = org, size, lo, hi
        b[i].out_offset = off
        b[i].out_stride[:] = [1, sx, sy]
        zz, yy, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        targets.append(off + xx + yy * sx + zz * sy)
        off += nz * sy + guard
    total = off + guard
    out = torch.full((total,), float(CANARY), dtype=torch.float32, device="cuda")
    out.view(torch.int32).fill_(0x7FC0DEAD)
    ctx.forward_blocks(cfg, torch.from_numpy(x.view(np.int16)).cuda(), b, 2, total, out=out)
    torch.cuda.synchronize()
    bits = out.view(torch.int32).cpu().numpy()
    written = np.zeros(total, bool)
    for t in targets:
        written[t.ravel()] = True
    assert (bits[~written] == 0x7FC0DEAD).all(), "an element outside the block regions was written"
    assert (bits[written] != 0x7FC0DEAD).all(), "a target element was not written"
    # and the regions hold the whole-block maps
    for i, (org, size, lo, hi) in enumerate(regions):
        xs = np.ascontiguousarray(x[:, org[2]:org[2] + size[2], org[1]:org[1] + size[1], org[0]:org[0] + size[0]])
        whole = ctx.forward(cfg, xs)[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
        got = out.cpu().numpy()[targets[i]]
        assert np.array_equal(np.isnan(got), np.isnan(whole))
        assert np.array_equal(np.nan_to_num(got), np.nan_to_num(whole))


def test_forward_repeatable_and_backward_to_rounding(ctx):
    import torch
    from rfba_gb300 import drift
    from rfba_gb300.srrf import Config
    cfg = Config.make(mag=2, method=3, itc=0, trac_order=2, **SMOOTH)
    x = torch.from_numpy(_series(4, 6, 11, 12, 13, np.float32)).cuda()
    sh = torch.from_numpy(np.random.default_rng(4).normal(0, 0.3, (6, 3)).astype(np.float32)).cuda()
    m1 = ctx.forward_shifted(cfg, x, sh).clone()
    m2 = ctx.forward_shifted(cfg, x, sh).clone()
    assert torch.equal(torch.isnan(m1), torch.isnan(m2))
    assert torch.equal(torch.nan_to_num(m1), torch.nan_to_num(m2))
    g = drift.grad_map(m2)
    a_in, a_sh = ctx.backward(cfg, x, sh, g)
    a_in, a_sh = a_in.clone(), a_sh.clone()
    b_in, b_sh = ctx.backward(cfg, x, sh, g)
    torch.cuda.synchronize()
    scale_in = float(a_in.abs().max())
    scale_sh = float(a_sh.abs().max())
    assert scale_in > 0 and scale_sh > 0
    assert float((a_in - b_in).abs().max()) <= 1e-6 * scale_in
    assert float((a_sh - b_sh).abs().max()) <= 1e-6 * scale_sh
