"""Block lists on the GPU: the batched persistent path against the plain
per-block path and the oracle, the reference's block split/put-back on
synthetic data, and scratch-budget splitting into several passes."""
import os

import numpy as np
import pytest

from tests.parity import assert_parity

pytestmark = pytest.mark.gpu

SHIPPED = dict(gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)


def _series(seed, T, D, H, W, emitters=30):
    from rfba_gb300 import synth
    scene = synth.make_scene(seed, T, (W, H, D), emitters)
    return synth.render(scene, (W, H, D), seed, np.uint16)


def test_dosplit_batched_equals_plain_and_oracle(ctx, oracle_mod):
    from rfba_gb300 import srrf
    kw = dict(mag=3, method=3, itc=0, trac_order=2, **SHIPPED)
    cfg = srrf.Config.make(**kw)
    x = _series(41, 6, 20, 30, 34)
    blocks, n, oe = srrf.blocks_dosplit(cfg, x.shape, (15, 15, 11), 1)
    assert n > 4
    batched = ctx.forward_blocks(cfg, x, blocks, n, oe)
    plain = ctx.forward_blocks_plain(cfg, x, blocks, n, oe)
    assert np.array_equal(np.isnan(batched), np.isnan(plain))
    assert np.array_equal(np.nan_to_num(batched), np.nan_to_num(plain))
    oc = oracle_mod.make_conf(**kw)
    for b in range(n):
        B = blocks[b]
        sub = x[:, B.origin[2]:B.origin[2] + B.size[2], B.origin[1]:B.origin[1] + B.size[1],
                B.origin[0]:B.origin[0] + B.size[0]].astype(np.float32)
        ref = oracle_mod.srrf_region(sub, oc)
        nz, ny, nx = ref.shape
        got = batched[B.out_offset: B.out_offset + nx * ny * nz].reshape(nz, ny, nx)
        assert_parity(got, ref, 1e-4, f"block {b}")


def test_legacy_split_on_synthetic(tmp_path, oracle_mod):
    from rfba_gb300 import srrf
    kw = dict(mag=2, method=1, block_size=(12, 10, 9), **SHIPPED)
    x = _series(42, 5, 15, 19, 23).astype(np.float32)
    ini = ("[SRRF]\nMagnification=2\nMainRange=1\nXRange=1\nYRange=1\nZRange=1\n[Temproal]\nMethod=1\n"
           "[Radiality]\nGradient_Smoothing=1\n[Split]\nBlockSizeX=12\nBlockSizeY=10\nBlockSizeZ=9\n")
    (tmp_path / "SRRF.ini").write_text(ini)
    cwd = os.getcwd()
    try:
        os.chdir(tmp_path)
        got = srrf.SRRFGradientCalc(x)
    finally:
        os.chdir(cwd)
    ref = oracle_mod.legacy(x, oracle_mod.make_conf(**kw), fill=0.0)
    assert_parity(got, ref, 1e-5, "legacy split")


def test_small_scratch_budget_splits_into_passes(oracle_mod):
    """A budget far below one stack forces z slabs and several passes; the map
    must not change."""
    from rfba_gb300 import srrf
    kw = dict(mag=2, method=3, itc=1, trac_order=2, **SHIPPED)
    cfg = srrf.Config.make(**kw)
    x = _series(43, 10, 12, 14, 16)
    big = srrf.Context(0)
    small = srrf.Context(0, scratch_budget_bytes=256 * 1024)
    try:
        a = big.forward(cfg, x)
        b = small.forward(cfg, x)
    finally:
        big.close()
        small.close()
    assert np.array_equal(np.isnan(a), np.isnan(b))
    assert np.array_equal(np.nan_to_num(a), np.nan_to_num(b))
    assert_parity(b, oracle_mod.srrf_region(x.astype(np.float32), oracle_mod.make_conf(**kw)), 1e-4, "passes")


def test_edge_shapes(ctx, oracle_mod):
    """Tiny and ragged volumes, T = 1..3, volumes smaller than the window."""
    from rfba_gb300 import srrf
    for (T, D, H, W), kw in [((1, 5, 6, 7), dict(mag=2, method=1)),
                             ((2, 4, 4, 4), dict(mag=3, method=3, itc=1, trac_order=2)),
                             ((3, 3, 9, 2), dict(mag=2, method=0)),
                             ((3, 1, 1, 1), dict(mag=2, method=1)),
                             ((4, 6, 5, 17), dict(mag=(3, 1, 2), method=2))]:
        x = _series(44 + T, T, D, H, W, emitters=3)
        cfg = srrf.Config.make(**kw, **SHIPPED)
        got = ctx.forward(cfg, x)
        ref = oracle_mod.srrf_region(x.astype(np.float32), oracle_mod.make_conf(**kw, **SHIPPED))
        assert_parity(got, ref, 1e-4, f"edge {(T, D, H, W)} {kw}")
