"""Parity at the benchmark configurations' full sizes: the CUDA path computes
each configuration's whole map (synthetic series of the configuration's
shape and model, rfba_gb300/synth.py), and regions of it near the low corner,
in the middle and near the high corner are compared with the FP64 oracle
computed on the same full-size input. Tolerances, relative L-inf with identical
NaN masks: 1e-5 for the temporal mean, 1e-4 for TRAC maps. The large series
runs in full (200 volumes, TRAC-4) with its map cut into 16-plane z slices, the
checked regions straddling slice boundaries; the batching series is the 160^3
variant with 216 blocks."""
import numpy as np
import pytest

from tests.parity import assert_parity

pytestmark = pytest.mark.gpu

SMOOTH = dict(gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)


def _workload(name, n_vol=None, shape=None):
    from rfba_gb300 import synth
    w = dict(synth.WORKLOADS[name])
    if n_vol is not None:
        w["n_vol"] = n_vol
    if shape is not None:
        w["shape"] = tuple(shape)
    seed = 1234 + w["index"]
    scene = synth.make_scene(seed, w["n_vol"], w["shape"], w["n_emitters"], w["curves"], w["drift"])
    return synth.render_parallel(scene, w["shape"], seed, w["dtype"]), scene


def _check_regions(got, img, oracle_mod, kw, regions, tol, label, also=()):
    """Regions of `got` (and of every map in `also`) against the oracle."""
    conf = oracle_mod.make_conf(**kw)
    worst = 0.0
    for lo, hi in regions:
        ref = oracle_mod.srrf_region(img, conf, lo, hi)
        assert np.isfinite(ref).any(), f"{label}: region {lo}-{hi} lies outside the window"
        for i, m in enumerate((got,) + tuple(also)):
            sub = m[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
            worst = max(worst, assert_parity(sub, ref, tol, f"{label} map {i} region {lo}-{hi}"))
    print(f"[config] {label}: rel L-inf {worst:.2e} over {len(regions)} regions (tolerance {tol:.0e})")
    return worst


def test_small_tra(ctx, oracle_mod):
    from rfba_gb300.srrf import Config
    x, _ = _workload("small")
    kw = dict(mag=2, method=1, **SMOOTH)
    got = ctx.forward(Config.make(**kw), x)
    _check_regions(got, x.astype(np.float32), oracle_mod, kw,
                   [((4, 4, 4), (12, 12, 12)), ((28, 28, 28), (36, 36, 36)), ((52, 50, 54), (60, 58, 60))], 1e-5,
                   "small 30 x 32^3, mag 2, TRA")


def test_mid_trac2(ctx, oracle_mod):
    from rfba_gb300.srrf import Config
    x, _ = _workload("mid")
    kw = dict(mag=(4, 4, 2), method=3, itc=0, trac_order=2, **SMOOTH)
    got = ctx.forward(Config.make(**kw), x)
    _check_regions(got, x.astype(np.float32), oracle_mod, kw,
                   [((8, 8, 4), (20, 20, 10)), ((250, 250, 60), (262, 262, 66)), ((490, 495, 118), (502, 507, 124))],
                   1e-4, "mid 100 x 128x128x64, mag 4x4x2, TRAC-2")


@pytest.mark.parametrize("method", [1, 3], ids=["TRA", "TRAC-2"])
def test_batching_blocks(ctx, oracle_mod, method):
    from rfba_gb300 import srrf
    x, _ = _workload("batching", shape=(160, 160, 160))
    kw = dict(mag=3, method=method, itc=0, trac_order=2, **SMOOTH)
    cfg = srrf.Config.make(**kw)
    blocks, n, oe = srrf.blocks_dosplit(cfg, x.shape, 29, 1)
    assert n == 216
    got = ctx.forward_blocks(cfg, x, blocks, n, oe)
    conf = oracle_mod.make_conf(**kw)
    worst = 0.0
    for i in (0, 107, 215):
        b = blocks[i]
        (ox, oy, oz), (sx, sy, sz) = tuple(b.origin), tuple(b.size)
        nx, ny, nz = b.hi[0] - b.lo[0], b.hi[1] - b.lo[1], b.hi[2] - b.lo[2]
        bm = got[b.out_offset:b.out_offset + nx * ny * nz].reshape(nz, ny, nx)
        sub = np.ascontiguousarray(x[:, oz:oz + sz, oy:oy + sy, ox:ox + sx], dtype=np.float32)
        for lo, hi in [((6, 6, 6), (14, 14, 14)), ((nx - 14, ny - 14, nz - 12), (nx - 6, ny - 6, nz - 6))]:
            ref = oracle_mod.srrf_region(sub, conf, lo, hi)
            assert np.isfinite(ref).any()
            rb = bm[lo[2] - b.lo[2]:hi[2] - b.lo[2], lo[1] - b.lo[1]:hi[1] - b.lo[1], lo[0] - b.lo[0]:hi[0] - b.lo[0]]
            worst = max(worst, assert_parity(rb, ref, 1e-5 if method == 1 else 1e-4, f"block {i} {lo}-{hi}"))
    print(f"[config] batching 216 blocks of 50 x 160^3, mag 3, method {method}: rel L-inf {worst:.2e}")


def test_diff_drift_corrected_trac2(ctx, oracle_mod):
    import torch
    from rfba_gb300.srrf import Config
    x, scene = _workload("diff")
    shifts = (-scene.drift).astype(np.float32)
    kw = dict(mag=2, method=3, itc=0, trac_order=2, **SMOOTH)
    got = ctx.forward_shifted(Config.make(**kw), torch.from_numpy(x).cuda(), torch.from_numpy(shifts).cuda())
    torch.cuda.synchronize()
    got = got.cpu().numpy()
    xp = np.ascontiguousarray(oracle_mod.shift(x, shifts), dtype=np.float32)
    _check_regions(got, xp, oracle_mod, kw,
                   [((6, 6, 6), (14, 14, 14)), ((60, 60, 60), (68, 68, 68)), ((112, 110, 114), (120, 118, 122))],
                   1e-4, "diff 60 x 64^3 drift-corrected, mag 2, TRAC-2")


def test_large_trac4_20_volumes(ctx, oracle_mod):
    from rfba_gb300.srrf import Config
    x, _ = _workload("large", n_vol=20)
    kw = dict(mag=(4, 4, 2), method=3, itc=0, trac_order=4, **SMOOTH)
    got = ctx.forward(Config.make(**kw), x)
    _check_regions(got, x.astype(np.float32), oracle_mod, kw,
                   [((16, 16, 8), (24, 24, 14)), ((510, 510, 126), (518, 518, 132)),
                    ((1000, 1004, 240), (1008, 1012, 246))], 1e-4, "large 20 x 256x256x128, mag 4x4x2, TRAC-4")


def test_large_trac4_all_200_volumes(oracle_mod):
    """The large configuration in full: 200 x 256x256x128 u16, mag 4x4x2, TRAC-4
    ITC 0 (kernel.cu:469-500 with order 4). The radiality + intensity stacks of
    the whole map would take 430 GB, so the forward cuts the map into z slices
    under the context's scratch budget, each slice computed for all 200
    volumes. The budget here, 16 planes x 1024 x 1024 subvoxels x 200 volumes x
    8 bytes, fixes the slices at z = 16 k; every checked region below straddles a
    slice boundary (z 16, 128, 240) and together they cover the low corner, the
    middle and the high corner of the map plus seeded interior boxes.

    The same budget with the series in time batches (the automatic choice: 25
    volumes a batch, the TRAC-4 window sums carried between batches) holds the
    stacks of 25 volumes and the carried state for 64 planes at a time; that map
    is checked on the same regions and against the sliced one."""
    from rfba_gb300 import srrf
    from tests.parity import assert_parity
    x, _ = _workload("large")
    assert x.shape == (200, 128, 256, 256)
    kw = dict(mag=(4, 4, 2), method=3, itc=0, trac_order=4, **SMOOTH)
    budget = 16 * 1024 * 1024 * 200 * 8
    c = srrf.Context(0, budget)
    try:
        c.set_time_batch(-1)
        got = c.forward(srrf.Config.make(**kw), x)
        assert c.last_time_batches() == (0, 0)
        c.set_time_batch(0)
        streamed = c.forward(srrf.Config.make(**kw), x)
        assert c.last_time_batches() == (25, 8)
    finally:
        c.close()
    assert_parity(streamed, got, 1e-4, "large TRAC-4: time batches vs z slices")
    rng = np.random.default_rng(2026)
    regions = [((16, 16, 12), (24, 24, 20)), ((508, 510, 124), (516, 518, 132)),
               ((1000, 1004, 236), (1008, 1012, 244))]
    for _ in range(5):  # interior boxes, each across one of the 15 inner slice boundaries
        x0, y0 = (int(v) for v in rng.integers(12, 1004, size=2))
        zb = 16 * int(rng.integers(1, 16))
        regions.append(((x0, y0, zb - 4), (x0 + 8, y0 + 8, zb + 4)))
    xf = x.astype(np.float32)
    del x
    _check_regions(got, xf, oracle_mod, kw, regions, 1e-4,
                   "large 200 x 256x256x128, mag 4x4x2, TRAC-4 (z slices; time batches)", also=(streamed,))


def test_mid_trac2_itc1_reduced_t(ctx, oracle_mod):
    """The shipped INI's temporal setting (TRAC-2 with integrated lag times) at
    the mid configuration's spatial size, 24 volumes."""
    from rfba_gb300.srrf import Config
    x, _ = _workload("mid", n_vol=24)
    kw = dict(mag=(4, 4, 2), method=3, itc=1, trac_order=2, **SMOOTH)
    got = ctx.forward(Config.make(**kw), x)
    _check_regions(got, x.astype(np.float32), oracle_mod, kw,
                   [((8, 8, 4), (20, 20, 10)), ((250, 250, 60), (262, 262, 66)), ((490, 495, 118), (502, 507, 124))],
                   1e-4, "mid 24 x 128x128x64, mag 4x4x2, TRAC-2 ITC 1")
