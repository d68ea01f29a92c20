"""The forward's TMA-staged input tile (tensor-map box rounded to a 16-byte x
boundary, zero-filled outside the volume, block-edge clamp applied when the
staging area is converted) gives the same maps, bit for bit, as plain loads:
whole volumes, doSplit block lists (odd block origins, edge blocks) and the
reference's GradientCalc split, for uint16 and float input."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHIPPED = dict(gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(np.nan_to_num(a), np.nan_to_num(b))


def _run(monkeypatch, tma, fn):
    monkeypatch.setenv("RFBA_GRAPH", "0")
    monkeypatch.setenv("RFBA_TUNE", "0")
    monkeypatch.setenv("RFBA_TMA", "1" if tma else "0")
    return fn()


@pytest.mark.parametrize("dtype,shape,kw", [
    (np.uint16, (40, 36, 30), dict(mag=3, method=1)),
    (np.uint16, (48, 24, 20), dict(mag=(4, 4, 2), method=3, itc=0, trac_order=2)),
    (np.float32, (32, 28, 24), dict(mag=2, method=3, itc=1, trac_order=3)),
    (np.float32, (36, 20, 16), dict(mag=(2, 2, 1), method=0, gradient_smooth=0)),
], ids=["u16_mag3", "u16_mag442", "f32_mag2_itc1", "f32_aniso_nosmooth"])
def test_tma_matches_plain_loads(ctx, monkeypatch, dtype, shape, kw):
    import torch
    from rfba_gb300 import srrf, synth
    k = dict(SHIPPED)
    k.update(kw)
    cfg = srrf.Config.make(**k)
    scene = synth.make_scene(9, 5, shape, 50)
    x = synth.render(scene, shape, 9, dtype)
    xd = torch.from_numpy(x.view(np.int16) if dtype == np.uint16 else x).cuda()
    whole = [_run(monkeypatch, t, lambda: ctx.forward(cfg, xd).cpu().numpy()) for t in (False, True)]
    assert _same(whole[0], whole[1])
    blocks, n, oe = srrf.blocks_dosplit(cfg, x.shape, 13, 1)
    bl = [_run(monkeypatch, t, lambda: ctx.forward_blocks(cfg, xd, blocks, n, oe).cpu().numpy())
          for t in (False, True)]
    assert _same(bl[0], bl[1])
    if cfg.mag[0] == cfg.mag[1] == cfg.mag[2]:
        gb, gn = srrf.blocks_gradientcalc(cfg, x.shape)
        goe = int(np.prod(x.shape[1:])) * cfg.mag[0] ** 3
        gc = [_run(monkeypatch, t, lambda: ctx.forward_blocks(cfg, xd, gb, gn, goe).cpu().numpy())
              for t in (False, True)]
        assert _same(gc[0], gc[1])
