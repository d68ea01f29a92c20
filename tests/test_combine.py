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
