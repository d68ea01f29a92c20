"""Parity of the CUDA path (through the C-ABI) against the FP64 oracle."""
import numpy as np
import pytest

from tests.parity import assert_parity, tol_for

pytestmark = pytest.mark.gpu


def _series(seed, T, D, H, W, dtype=np.uint16, emitters=12):
    from rfba_gb300 import synth
    scene = synth.make_scene(seed, T, (W, H, D), emitters)
    return synth.render(scene, (W, H, D), seed, dtype)


def _cfg_pair(**kw):
    from rfba_gb300.srrf import Config
    from oracle import oracle as O
    return Config.make(**kw), O.make_conf(**kw)


CASES = [
    # (name, T, D, H, W, config)
    ("tra_mag2_smooth", 6, 10, 11, 12, dict(mag=2, method=1, gradient_smooth=1, x_range=1, y_range=1, z_range=1)),
    ("tra_mag2_nosmooth", 5, 9, 9, 10, dict(mag=2, method=1, gradient_smooth=0)),
    ("tra_noiw", 5, 9, 9, 9, dict(mag=2, method=1, intensity_w=0, gradient_smooth=1, x_range=1, y_range=1, z_range=1)),
    ("trm", 6, 9, 10, 9, dict(mag=2, method=0, gradient_smooth=1, x_range=1, y_range=1, z_range=1)),
    ("trppm", 6, 9, 9, 10, dict(mag=2, method=2, gradient_smooth=1, x_range=1, y_range=1, z_range=1)),
    ("trac2_itc0", 10, 9, 9, 9, dict(mag=2, method=3, itc=0, trac_order=2, gradient_smooth=1, x_range=1, y_range=1,
                                     z_range=1)),
    ("trac2_itc1", 12, 9, 9, 9, dict(mag=2, method=3, itc=1, trac_order=2, gradient_smooth=1, x_range=1, y_range=1,
                                     z_range=1)),
    ("trac3_itc1_odd", 13, 8, 9, 9, dict(mag=2, method=3, itc=1, trac_order=3, gradient_smooth=1, x_range=1,
                                         y_range=1, z_range=1)),
    ("trac4_itc0", 11, 8, 9, 9, dict(mag=2, method=3, itc=0, trac_order=4, gradient_smooth=1, x_range=1, y_range=1,
                                     z_range=1)),
    ("trac4_itc1", 16, 8, 8, 9, dict(mag=2, method=3, itc=1, trac_order=4, gradient_smooth=1, x_range=1, y_range=1,
                                     z_range=1)),
    ("mag3", 5, 8, 9, 8, dict(mag=3, method=1, gradient_smooth=1, x_range=1, y_range=1, z_range=1)),
    ("mag442", 6, 8, 8, 9, dict(mag=(4, 4, 2), method=3, itc=0, trac_order=2, gradient_smooth=1, x_range=1,
                                y_range=1, z_range=1)),
    ("mag5", 4, 7, 7, 8, dict(mag=5, method=1, gradient_smooth=1, x_range=1, y_range=1, z_range=1)),
    ("mag1", 5, 9, 12, 10, dict(mag=1, method=1, gradient_smooth=1, x_range=1, y_range=1, z_range=1)),
    ("renorm_poscon", 5, 9, 9, 9, dict(mag=2, method=1, renormalize=1, remove_con=1, gradient_smooth=1)),
    ("ranges_main2", 5, 10, 10, 10, dict(mag=2, method=1, gradient_smooth=1, main_range=2, x_range=1, y_range=0,
                                         z_range=2)),
    ("axes4", 5, 9, 9, 9, dict(mag=2, method=1, axes_in_ring=4, gradient_smooth=1, x_range=1, y_range=1, z_range=1)),
    ("radius_03", 5, 9, 9, 9, dict(mag=2, method=1, ring_radius=0.3, gradient_smooth=1, x_range=1, y_range=1,
                                   z_range=1)),
    # 12-row tiles (mag_y 6), the 224-thread 28-row tile (mag_y 7), mag 8
    ("mag6", 3, 6, 6, 7, dict(mag=6, method=1, gradient_smooth=1, x_range=1, y_range=1, z_range=1)),
    ("mag7", 3, 5, 6, 5, dict(mag=7, method=3, itc=0, trac_order=2, gradient_smooth=1, x_range=1, y_range=1,
                              z_range=1)),
    ("mag8", 2, 5, 5, 6, dict(mag=8, method=1, gradient_smooth=1, x_range=1, y_range=1, z_range=1)),
    # short series: one volume; TRAC with no full lag window; ITC 1 binning of 3 volumes
    ("t1_tra", 1, 8, 8, 9, dict(mag=2, method=1, gradient_smooth=1, x_range=1, y_range=1, z_range=1)),
    ("t2_trac2", 2, 8, 9, 8, dict(mag=2, method=3, itc=0, trac_order=2, gradient_smooth=1, x_range=1, y_range=1,
                                  z_range=1)),
    ("t3_trac2_itc1", 3, 8, 8, 8, dict(mag=2, method=3, itc=1, trac_order=2, gradient_smooth=1, x_range=1,
                                       y_range=1, z_range=1)),
]


@pytest.mark.parametrize("name,T,D,H,W,kw", CASES, ids=[c[0] for c in CASES])
def test_forward_matches_oracle(ctx, oracle_mod, name, T, D, H, W, kw):
    cfg, oc = _cfg_pair(**kw)
    x = _series(100 + len(name), T, D, H, W)
    got = ctx.forward(cfg, x)
    ref = oracle_mod.srrf_region(x.astype(np.float32), oc)
    err = assert_parity(got, ref, tol_for(cfg.method), name)
    print(f"[parity] {name}: rel L-inf {err:.2e}")


def test_float_input_matches_u16(ctx):
    from rfba_gb300.srrf import Config
    cfg = Config.make(mag=2, method=1, gradient_smooth=1, x_range=1, y_range=1, z_range=1)
    x = _series(7, 5, 9, 9, 9)
    a = ctx.forward(cfg, x)
    b = ctx.forward(cfg, x.astype(np.float32))
    assert np.array_equal(np.isnan(a), np.isnan(b))
    assert np.allclose(np.nan_to_num(a), np.nan_to_num(b), rtol=0, atol=0)


def test_device_pointers_match_host(ctx):
    import torch
    from rfba_gb300.srrf import Config
    cfg = Config.make(mag=2, method=3, itc=0, trac_order=2, gradient_smooth=1, x_range=1, y_range=1, z_range=1)
    x = _series(8, 8, 9, 10, 11, dtype=np.float32)
    a = ctx.forward(cfg, x)
    xd = torch.from_numpy(x).cuda()
    b = ctx.forward(cfg, xd)
    torch.cuda.synchronize()
    b = b.cpu().numpy()
    assert np.array_equal(np.isnan(a), np.isnan(b))
    assert np.array_equal(np.nan_to_num(a), np.nan_to_num(b))


def test_sub_regions_match_whole(ctx, oracle_mod):
    """A block restricted to a sub-region computes exactly that part of the
    whole-block map."""
    from rfba_gb300.srrf import Block, Config
    cfg = Config.make(mag=2, method=1, gradient_smooth=1, x_range=1, y_range=1, z_range=1)
    x = _series(9, 5, 10, 10, 12)
    whole = ctx.forward(cfg, x)
    b = (Block * 1)()
    b[0].origin[:] = [0, 0, 0]
    b[0].size[:] = [12, 10, 10]
    b[0].lo[:] = [3, 5, 7]
    b[0].hi[:] = [21, 17, 13]
    nx, ny, nz = 18, 12, 6
    b[0].out_offset = 0
    b[0].out_stride[:] = [1, nx, nx * ny]
    out = ctx.forward_blocks(cfg, x, b, 1, nx * ny * nz)
    sub = out.reshape(nz, ny, nx)
    ref = whole[7:13, 5:17, 3:21]
    assert np.array_equal(np.isnan(sub), np.isnan(ref))
    assert np.array_equal(np.nan_to_num(sub), np.nan_to_num(ref))
