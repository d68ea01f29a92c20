"""CombineBlock (Matlab Scripts/CombineBlock.m, genpsf.m, loadResult.m): the
library's PSF table and result-file parser against the numpy restatement (CPU),
and the GPU reconstruction (histogram, noise mask, convn 'same', uint16 scaling)
bit for bit against it (GPU)."""
import numpy as np
import pytest

from oracle import combine_oracle as C


@pytest.mark.parametrize("sigma,thr", [(3.5, 1000.0), (2.0, 500.0), (1.2, 3000.0)])
def test_psf_matches_genpsf(built_lib, sigma, thr):
    from rfba_gb300 import srrf
    a = srrf.combine_psf(sigma, thr)
    b = C.genpsf(sigma, thr)
    assert a.shape == b.shape and np.array_equal(a, b)
    assert a.max() == 65535


def _write_res(path, spots, passes=2, junk=True):
    with open(path, "w") as f:
        if junk:
            f.write("MAIN: 1 2 3\nIterations: 10\n")
        for p in range(passes):
            sel = spots[p::passes]
            f.write(f"PASS{p}: " + " ".join(f"{v:.20e}" for v in sel.ravel()) + "\n")


def _spots(rng, n, img):
    s = np.empty((n, 5))
    s[:, 0] = rng.uniform(100, 1000, n)
    s[:, 1] = rng.uniform(1, 2, n)
    for a in range(3):
        s[:, 2 + a] = rng.uniform(0, img[a] - 1, n)
    return s


def test_load_result_matches(built_lib, tmp_path):
    from rfba_gb300 import srrf
    rng = np.random.default_rng(2)
    sp = _spots(rng, 300, (30, 25, 20))
    p = tmp_path / "res_1_1_1.txt"
    _write_res(p, sp, passes=3)
    for start, size, border in [((1, 1, 1), (30, 25, 20), 2), ((9, 5, 3), (14, 12, 10), 1), ((1, 1, 1), (6, 6, 6), 0)]:
        got = srrf.combine_load_result(p, border, start, size)
        exp = C.load_result(p, border, start, size)
        assert got.shape == exp.shape and np.array_equal(got, exp)


@pytest.mark.gpu
@pytest.mark.parametrize("img,zoom,r,rz,thr", [((8, 7, 5), 4, 3, 1, 5), ((6, 6, 4), 5, 2, 1, 2),
                                              ((5, 4, 3), 3, 20, 3, 70)],
                         ids=["masked", "small_window", "window_larger_than_grid"])
def test_render_matches_oracle(ctx, img, zoom, r, rz, thr):
    rng = np.random.default_rng(7)
    sp = _spots(rng, 400, img)
    sp[:40, 2:] = sp[40:80, 2:] + rng.normal(0, 0.02, (40, 3))  # clusters
    sp[0, 2] = img[0] - 0.01  # rounds onto the cropped margin
    psf = C.genpsf(1.5, 1000.0)
    got, dropped = ctx.combine_render(sp, img, zoom, psf, r, rz, thr)
    exp = C.render(sp, img, zoom, psf, r, rz, thr)
    assert dropped >= 1
    assert got.shape == exp.shape
    assert np.array_equal(got, exp), f"{np.count_nonzero(got != exp)} voxels differ"


@pytest.mark.gpu
def test_combine_blocks_pipeline(ctx, tmp_path):
    from rfba_gb300 import srrf
    rng = np.random.default_rng(4)
    img, block, border = (20, 16, 12), (9, 9, 8), 1
    xs, ys, zs = (srrf.dosplit(img[a], block[a], border) for a in range(3))
    allsp = []
    for i, (sx, nx) in enumerate(xs, 1):
        for j, (sy, ny) in enumerate(ys, 1):
            for k, (sz, nz) in enumerate(zs, 1):
                sp = _spots(rng, 60, img)
                _write_res(tmp_path / f"res_{i}_{j}_{k}.txt", sp)
                allsp.append(C.load_result(tmp_path / f"res_{i}_{j}_{k}.txt", border, (sx, sy, sz), (nx, ny, nz)))
    got, _ = ctx.combine_blocks(tmp_path, img, block, border, zoom=3, sigma=1.5, noise_r=2, noise_rz=1,
                                noise_threshold=3)
    exp = C.render(np.concatenate(allsp), img, 3, C.genpsf(1.5, 1000.0), 2, 1, 3)
    assert np.array_equal(got, exp)


@pytest.mark.gpu
def test_combine_cli_writes_tiff(tmp_path):
    import subprocess
    import sys
    from pathlib import Path
    from rfba_gb300 import srrf
    rng = np.random.default_rng(9)
    img, block, border = (12, 10, 8), (7, 6, 6), 1
    xs, ys, zs = (srrf.dosplit(img[a], block[a], border) for a in range(3))
    allsp = []
    for i, (sx, nx) in enumerate(xs, 1):
        for j, (sy, ny) in enumerate(ys, 1):
            for k, (sz, nz) in enumerate(zs, 1):
                sp = _spots(rng, 40, img)
                _write_res(tmp_path / f"res_{i}_{j}_{k}.txt", sp)
                allsp.append(C.load_result(tmp_path / f"res_{i}_{j}_{k}.txt", border, (sx, sy, sz), (nx, ny, nz)))
    out = tmp_path / "reconstruction.tif"
    root = Path(__file__).resolve().parents[1]
    subprocess.run([sys.executable, "-m", "rfba_gb300.combine_cli", "--dims", *map(str, img), "--block",
                    *map(str, block), "--border", str(border), "--zoom", "3", "--sigma", "1.5", "--noise-r", "2",
                    "--noise-rz", "1", "--noise-threshold", "3", str(tmp_path), str(out)], check=True, cwd=root)
    exp = C.render(np.concatenate(allsp), img, 3, C.genpsf(1.5, 1000.0), 2, 1, 3)
    # read back the pages (little-endian, one strip per page as written)
    import struct
    b = out.read_bytes()
    pages = []
    off = struct.unpack("<I", b[4:8])[0]
    while off:
        n = struct.unpack("<H", b[off:off + 2])[0]
        tags = {}
        for e in range(n):
            tag, typ, cnt, val = struct.unpack("<HHII", b[off + 2 + 12 * e: off + 14 + 12 * e])
            tags[tag] = val & 0xFFFF if typ == 3 else val
        W, H, so = tags[256], tags[257], tags[273]
        pages.append(np.frombuffer(b[so:so + W * H * 2], "<u2").reshape(H, W))
        off = struct.unpack("<I", b[off + 2 + 12 * n: off + 6 + 12 * n])[0]
    assert np.array_equal(np.stack(pages), exp)


# ---- known answers derived from CombineBlock.m by hand (no oracle) -----------
# A hand-made PSF makes placement and scaling exact: convn(..., 'same') puts
# kernel element floor(K/2) (0-based) on the spot's voxel (CombineBlock.m:148),
# the result is divided by its maximum and scaled to 65535 (:151-153), and
# uint16() rounds half away from zero (:157). Spots land on
# round(p * zoom) (+1 in MATLAB's 1-based indices, :43-45).

def _hand_psf():
    psf = np.zeros((3, 4, 5), np.uint16)  # [z][y][x]; even y extent: centre element index 2
    psf[1, 2, 2] = 60000
    psf[1, 2, 3] = 30000
    psf[0, 1, 2] = 15000
    psf[2, 3, 4] = 7
    return psf


def _place(shape, psf, at, scale=1.0):
    Z, Y, X = shape
    out = np.zeros(shape, np.float64)
    Kz, Ky, Kx = psf.shape
    az, ay, ax = at
    for z in range(Kz):
        for y in range(Ky):
            for x in range(Kx):
                oz, oy, ox = az + z - Kz // 2, ay + y - Ky // 2, ax + x - Kx // 2
                if 0 <= oz < Z and 0 <= oy < Y and 0 <= ox < X:
                    out[oz, oy, ox] += scale * psf[z, y, x]
    return out


def _scaled(v):
    """result ./ max .* 65535, then uint16() (round half away from zero)."""
    v = np.asarray(v, np.float64)
    return np.floor(v / v.max() * 65535.0 + 0.5).astype(np.uint16)


@pytest.mark.gpu
def test_render_known_answers(ctx):
    psf = _hand_psf()
    img, zoom = (4, 3, 2), 5  # grid 20 x 15 x 10
    shape = (10, 15, 20)
    # one spot, window larger than the grid (mask all ones): the PSF itself,
    # scaled by 65535 / 60000
    sp = np.array([[500.0, 1.5, 2.0, 1.0, 0.4]])  # -> voxel (x, y, z) = (10, 5, 2)
    got, dropped = ctx.combine_render(sp, img, zoom, psf, 30, 3, 1)
    assert dropped == 0
    np.testing.assert_array_equal(got, _scaled(_place(shape, psf, (2, 5, 10))))
    # two spots on one voxel count twice; scaling by the maximum cancels it
    got2, _ = ctx.combine_render(np.vstack([sp, sp]), img, zoom, psf, 30, 3, 1)
    np.testing.assert_array_equal(got2, got)
    # two spots apart: the copies add before the scaling
    sp2 = np.array([[1.0, 1.0, 2.0, 1.0, 0.4], [1.0, 1.0, 2.2, 1.0, 0.4]])  # x voxels 10 and 11
    got3, _ = ctx.combine_render(sp2, img, zoom, psf, 30, 3, 1)
    acc = _place(shape, psf, (2, 5, 10)) + _place(shape, psf, (2, 5, 11))
    np.testing.assert_array_equal(got3, _scaled(acc))
    # rounding half away from zero: 0.125 * 4 = 0.5 -> voxel 1; -0.125 * 4 = -0.5 -> -1, outside (dropped);
    # a spot on the upper margin (round(p * zoom) = grid size) is dropped too
    img4, zoom4 = (3, 3, 3), 4
    sp3 = np.array([[1, 1, 0.125, 1.0, 1.0], [1, 1, -0.125, 1.0, 1.0], [1, 1, 3.0, 1.0, 1.0]])
    got4, dropped4 = ctx.combine_render(sp3, img4, zoom4, psf, 30, 3, 1)
    assert dropped4 == 2
    np.testing.assert_array_equal(got4, _scaled(_place((12, 12, 12), psf, (4, 4, 1))))
    # no spots: all zeros
    got5, _ = ctx.combine_render(np.zeros((0, 5)), img, zoom, psf, 30, 3, 1)
    assert not got5.any()


@pytest.mark.gpu
def test_render_noise_mask_threshold_edge(ctx):
    """The mask keeps an interior voxel when the occupied voxels in its
    (2r+1)^2 x (2rz+1) box number more than the threshold (CombineBlock.m:
    133-136), and keeps every voxel of the border band."""
    psf = _hand_psf()
    img, zoom, r, rz, thr = (6, 6, 4), 4, 2, 1, 2  # grid 24 x 24 x 16, interior [2, 22) x [2, 22) x [1, 15)
    shape = (16, 24, 24)
    pts = [(10, 10, 8), (11, 10, 8), (10, 11, 8)]  # three occupied voxels within one box
    sp = np.array([[1.0, 1.0, x / zoom, y / zoom, z / zoom] for x, y, z in pts])
    # 3 > 2: kept
    got, _ = ctx.combine_render(sp, img, zoom, psf, r, rz, thr)
    acc = sum(_place(shape, psf, (z, y, x)) for x, y, z in pts)
    np.testing.assert_array_equal(got, _scaled(acc))
    # 2 occupied voxels, not more than 2: masked, nothing left
    got2, _ = ctx.combine_render(sp[:2], img, zoom, psf, r, rz, thr)
    assert not got2.any()
    # a lone voxel in the border band (y = 1 < r) is kept whatever the threshold
    lone = np.array([[1.0, 1.0, 10 / zoom, 1 / zoom, 8 / zoom]])
    got3, _ = ctx.combine_render(lone, img, zoom, psf, r, rz, thr)
    np.testing.assert_array_equal(got3, _scaled(_place(shape, psf, (8, 1, 10))))
