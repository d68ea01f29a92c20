"""ctypes front end of the CPU oracle (oracle/srrf_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, never by the product package. Functions mirror the
reference's GradientCalc entry points (RFBA Main/GradientCalc/kernel.cu:560,
GradientCalc.cpp:120) on host arrays.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libsrrf_oracle.so"
REF_LIB_PATH = HERE / "_ref" / "libsrrf_ref_host.so"


class OConf(ctypes.Structure):
    """Field layout shared with the product's rfba_srrf_config."""

    _fields_ = [
        ("ring_radius", ctypes.c_float),
        ("mag", ctypes.c_int * 3),
        ("axes_in_ring", ctypes.c_int),
        ("main_range", ctypes.c_int),
        ("x_range", ctypes.c_int),
        ("y_range", ctypes.c_int),
        ("z_range", ctypes.c_int),
        ("method", ctypes.c_int),
        ("itc", ctypes.c_int),
        ("trac_order", ctypes.c_int),
        ("remove_con", ctypes.c_int),
        ("renormalize", ctypes.c_int),
        ("gradient_smooth", ctypes.c_int),
        ("intensity_w", ctypes.c_int),
        ("block_size", ctypes.c_int * 3),
    ]


class RefSRRFConf(ctypes.Structure):
    """The reference's SRRFConf (RFBA Main/GradientCalc/kernel.cuh:3-24)."""

    _fields_ = [
        ("RingRadius", ctypes.c_float),
        ("Magnification", ctypes.c_int),
        ("AxesinRing", ctypes.c_int),
        ("MainRange", ctypes.c_int),
        ("XRange", ctypes.c_int),
        ("YRange", ctypes.c_int),
        ("ZRange", ctypes.c_int),
        ("Method", ctypes.c_int),
        ("ITC", ctypes.c_int),
        ("TRACOrder", ctypes.c_int),
        ("RemoveCon", ctypes.c_int),
        ("Renormalize", ctypes.c_int),
        ("GradientSmooth", ctypes.c_int),
        ("IntensityW", ctypes.c_int),
        ("blockSizeX", ctypes.c_int),
        ("blockSizeY", ctypes.c_int),
        ("blockSizeZ", ctypes.c_int),
    ]


def make_conf(**kw) -> OConf:
    """Configuration with the reference's GradientCalc.cpp:19-41 defaults,
    overridden by keyword (``mag`` may be an int or a 3-sequence)."""
    c = OConf()
    c.ring_radius = kw.get("ring_radius", 0.5)
    mag = kw.get("mag", 5)
    if isinstance(mag, int):
        mag = (mag, mag, mag)
    for i in range(3):
        c.mag[i] = int(mag[i])
    c.axes_in_ring = kw.get("axes_in_ring", 6)
    c.main_range = kw.get("main_range", 1)
    c.x_range = kw.get("x_range", 0)
    c.y_range = kw.get("y_range", 0)
    c.z_range = kw.get("z_range", 0)
    c.method = kw.get("method", 1)
    c.itc = kw.get("itc", 1)
    c.trac_order = kw.get("trac_order", 2)
    c.remove_con = kw.get("remove_con", 0)
    c.renormalize = kw.get("renormalize", 0)
    c.gradient_smooth = kw.get("gradient_smooth", 0)
    c.intensity_w = kw.get("intensity_w", 1)
    bs = kw.get("block_size", (16, 16, 16))
    for i in range(3):
        c.block_size[i] = int(bs[i])
    return c


def build(force: bool = False) -> Path:
    """Compile the oracle shared library (g++, OpenMP, no FP contraction so that
    the FP32 port gives the same bits on x86 and Arm)."""
    if LIB_PATH.exists() and not force and LIB_PATH.stat().st_mtime >= (HERE / "srrf_oracle.cpp").stat().st_mtime:
        return LIB_PATH
    LIB_PATH.parent.mkdir(parents=True, exist_ok=True)
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           str(HERE / "srrf_oracle.cpp"), "-o", str(LIB_PATH)]
    subprocess.run(cmd, check=True)
    return LIB_PATH


def build_ref(reference_root: str | None = None) -> Path | None:
    """Compile the reference's own sources as host code (oracle/build_ref.sh);
    returns None when the reference tree is absent. The tree is found by
    oracle.refroot.reference_root (RFBA_REFERENCE_ROOT, then the argument)."""
    from oracle.refroot import reference_root as _root
    reference_root = _root(reference_root)
    if not os.path.isdir(reference_root):
        return None
    subprocess.run(["bash", str(HERE / "build_ref.sh"), reference_root], check=True)
    return REF_LIB_PATH if REF_LIB_PATH.exists() else None


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        f32p = ctypes.POINTER(ctypes.c_float)
        f64p = ctypes.POINTER(ctypes.c_double)
        i32p = ctypes.POINTER(ctypes.c_int)
        cp = ctypes.POINTER(OConf)
        L.oracle_ring_f32.argtypes = [ctypes.c_float, ctypes.c_int, f32p, f32p, f32p]
        L.oracle_srrf_region_f64.argtypes = [f32p, i32p, cp, i32p, i32p, f64p, f64p, f64p]
        L.oracle_srrf_region_f32.argtypes = [f32p, i32p, cp, i32p, i32p, f32p, f32p, f32p]
        L.oracle_legacy_f64.argtypes = [f32p, i32p, cp, f64p]
        L.oracle_legacy_f32.argtypes = [f32p, i32p, cp, f32p]
        L.oracle_temporal_f64.argtypes = [cp, f64p, f64p, ctypes.c_int, f64p]
        L.oracle_adjoint_f64.argtypes = [f32p, i32p, cp, f64p, f64p, f64p, f64p, f64p]
        L.oracle_forward_shifted_f64.argtypes = [f32p, i32p, cp, f64p, f64p]
        L.oracle_shift_f64.argtypes = [f32p, i32p, f64p, f64p]
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def ring(radius: float = 0.5, axes: int = 6):
    n = 2 * axes
    x = np.zeros(n * n, np.float32)
    y = np.zeros(n * n, np.float32)
    z = np.zeros(n * n, np.float32)
    lib().oracle_ring_f32(radius, axes, _p(x, ctypes.c_float), _p(y, ctypes.c_float), _p(z, ctypes.c_float))
    return x, y, z


def srrf_region(img: np.ndarray, conf: OConf, lo=None, hi=None, dtype=np.float64, stacks: bool = False):
    """SRRF of one independent block. img is float32 [T][D][H][W]. Returns the
    map on the fine region [lo, hi) (x, y, z order), shape [nz][ny][nx]; with
    stacks=True also the radiality and intensity stacks [T][nz][ny][nx]."""
    img = np.ascontiguousarray(img, dtype=np.float32)
    T, D, H, W = img.shape
    dims = np.array([W, H, D, T], np.int32)
    mag = [conf.mag[i] for i in range(3)]
    lo = np.array(lo if lo is not None else (0, 0, 0), np.int32)
    hi = np.array(hi if hi is not None else (W * mag[0], H * mag[1], D * mag[2]), np.int32)
    nx, ny, nz = (hi - lo).tolist()
    out = np.zeros((nz, ny, nx), dtype)
    ct = ctypes.c_double if dtype == np.float64 else ctypes.c_float
    rs = np.zeros((T, nz, ny, nx), dtype) if stacks else None
    ist = np.zeros((T, nz, ny, nx), dtype) if stacks else None
    fn = lib().oracle_srrf_region_f64 if dtype == np.float64 else lib().oracle_srrf_region_f32
    fn(_p(img, ctypes.c_float), _p(dims, ctypes.c_int), ctypes.byref(conf), _p(lo, ctypes.c_int),
       _p(hi, ctypes.c_int), _p(out, ct), _p(rs, ct) if stacks else None, _p(ist, ct) if stacks else None)
    if stacks:
        return out, rs, ist
    return out


def legacy(img: np.ndarray, conf: OConf, dtype=np.float64, fill: float = 0.0):
    """The reference's SRRFGradientCalc block loop (GradientCalc.cpp:120-163) on
    an isotropic magnification; never-written voxels hold ``fill``."""
    img = np.ascontiguousarray(img, dtype=np.float32)
    T, D, H, W = img.shape
    m = conf.mag[0]
    dims = np.array([W, H, D, T], np.int32)
    out = np.full((D * m, H * m, W * m), fill, dtype)
    ct = ctypes.c_double if dtype == np.float64 else ctypes.c_float
    fn = lib().oracle_legacy_f64 if dtype == np.float64 else lib().oracle_legacy_f32
    fn(_p(img, ctypes.c_float), _p(dims, ctypes.c_int), ctypes.byref(conf), _p(out, ct))
    return out


def temporal(conf: OConf, rad: np.ndarray, inten: np.ndarray) -> float:
    rad = np.ascontiguousarray(rad, np.float64)
    inten = np.ascontiguousarray(inten, np.float64)
    out = ctypes.c_double()
    lib().oracle_temporal_f64(ctypes.byref(conf), _p(rad, ctypes.c_double), _p(inten, ctypes.c_double),
                              len(rad), ctypes.byref(out))
    return out.value


def _shifts_ptr(shifts, T):
    if shifts is None:
        return None, None
    s = np.ascontiguousarray(shifts, np.float64).reshape(T, 3)
    return s, _p(s, ctypes.c_double)


def forward_shifted(img: np.ndarray, conf: OConf, shifts=None) -> np.ndarray:
    """FP64 map of the drift-corrected series: each volume t resampled at
    x + shifts[t] (Catmull-Rom, edge clamp; x, y, z order) then the SRRF forward
    over the whole block."""
    img = np.ascontiguousarray(img, dtype=np.float32)
    T, D, H, W = img.shape
    dims = np.array([W, H, D, T], np.int32)
    m = [conf.mag[i] for i in range(3)]
    out = np.zeros((D * m[2], H * m[1], W * m[0]), np.float64)
    s, sp = _shifts_ptr(shifts, T)
    lib().oracle_forward_shifted_f64(_p(img, ctypes.c_float), _p(dims, ctypes.c_int), ctypes.byref(conf), sp,
                                     _p(out, ctypes.c_double))
    return out


def adjoint(img: np.ndarray, conf: OConf, gmap: np.ndarray, shifts=None):
    """FP64 forward map and the adjoint of L given dL/dmap = gmap: returns
    (map, dL/dinput [T][D][H][W], dL/dshifts [T][3] or None)."""
    img = np.ascontiguousarray(img, dtype=np.float32)
    T, D, H, W = img.shape
    dims = np.array([W, H, D, T], np.int32)
    m = [conf.mag[i] for i in range(3)]
    out = np.zeros((D * m[2], H * m[1], W * m[0]), np.float64)
    g = np.ascontiguousarray(gmap, np.float64).reshape(out.shape)
    din = np.zeros(img.shape, np.float64)
    s, sp = _shifts_ptr(shifts, T)
    dsh = np.zeros((T, 3), np.float64) if shifts is not None else None
    rc = lib().oracle_adjoint_f64(_p(img, ctypes.c_float), _p(dims, ctypes.c_int), ctypes.byref(conf), sp,
                                  _p(g, ctypes.c_double), _p(out, ctypes.c_double), _p(din, ctypes.c_double),
                                  _p(dsh, ctypes.c_double) if dsh is not None else None)
    if rc != 0:
        raise ValueError("no adjoint for this temporal reduction (TRA and TRAC with ITC 0 only)")
    return out, din, dsh


def shift(img: np.ndarray, shifts) -> np.ndarray:
    img = np.ascontiguousarray(img, dtype=np.float32)
    T, D, H, W = img.shape
    dims = np.array([W, H, D, T], np.int32)
    out = np.zeros(img.shape, np.float64)
    s, sp = _shifts_ptr(shifts, T)
    lib().oracle_shift_f64(_p(img, ctypes.c_float), _p(dims, ctypes.c_int), sp, _p(out, ctypes.c_double))
    return out


# ---------------------------------------------------------------------------
# The reference itself, compiled as host code (oracle/_ref), when available.
_ref = None


def ref_lib():
    """The reference GradientCalc built as host code, or None if not built."""
    global _ref
    if _ref is None:
        if not REF_LIB_PATH.exists():
            return None
        L = ctypes.CDLL(str(REF_LIB_PATH))
        f32p = ctypes.POINTER(ctypes.c_float)
        i32p = ctypes.POINTER(ctypes.c_int)
        L.SRRFGradientCalcGPU.argtypes = [f32p, i32p, f32p, ctypes.POINTER(RefSRRFConf)]
        L.SRRFGradientCalcGPU.restype = ctypes.c_int
        fn = getattr(L, "_Z16SRRFGradientCalcPfPiS_")
        fn.argtypes = [f32p, i32p, f32p]
        fn.restype = ctypes.c_int
        L.legacy_entry = fn
        _ref = L
    return _ref


def to_ref_conf(c: OConf) -> RefSRRFConf:
    r = RefSRRFConf()
    r.RingRadius = c.ring_radius
    r.Magnification = c.mag[0]
    r.AxesinRing = c.axes_in_ring
    r.MainRange, r.XRange, r.YRange, r.ZRange = c.main_range, c.x_range, c.y_range, c.z_range
    r.Method, r.ITC, r.TRACOrder = c.method, c.itc, c.trac_order
    r.RemoveCon, r.Renormalize, r.GradientSmooth, r.IntensityW = c.remove_con, c.renormalize, c.gradient_smooth, c.intensity_w
    r.blockSizeX, r.blockSizeY, r.blockSizeZ = c.block_size[0], c.block_size[1], c.block_size[2]
    return r


def ref_block(img: np.ndarray, conf: OConf) -> np.ndarray:
    """Reference SRRFGradientCalcGPU (kernel.cu:560) run on host cores: one
    block, isotropic magnification, full magnified output [D*m][H*m][W*m]."""
    L = ref_lib()
    assert L is not None, "oracle/_ref not built"
    img = np.ascontiguousarray(img, dtype=np.float32).copy()
    T, D, H, W = img.shape
    m = conf.mag[0]
    dims = np.array([W, H, D, T], np.int32)
    out = np.zeros((D * m, H * m, W * m), np.float32)
    rc = to_ref_conf(conf)
    L.SRRFGradientCalcGPU(_p(img, ctypes.c_float), _p(dims, ctypes.c_int), _p(out, ctypes.c_float), ctypes.byref(rc))
    return out


def seed_spots_rejection(srrf_map: np.ndarray, voxels: np.ndarray, mag: int, num_spots: int,
                         rng: np.random.Generator) -> np.ndarray:
    """The reference's SRRF-guided seeding (multispot5_place_methods.cc:291-341):
    candidates = the mag^3 subvoxels of each voxel in order (x offset slowest),
    element = floor(U * n), kept when U * max <= value, position
    (subvoxel + U - 0.5) / mag per axis in float. numpy's generator stands in
    for MT19937 (same algorithm, another random stream); draws are taken in
    batches, each kept in order. The map is used as the caller leaves it
    (NaN and negative values set to 0 first, multispot5_place_methods.cc:260-269)."""
    m = np.where(np.isnan(srrf_map) | (srrf_map < 0), 0.0, srrf_map).astype(np.float32)
    D, H, W = m.shape
    sub = np.array([(j1, j2, j3) for j1 in range(mag) for j2 in range(mag) for j3 in range(mag)], np.int64)
    pix = (np.asarray(voxels, np.int64)[:, None, :] * mag + sub[None, :, :]).reshape(-1, 3)
    inten = m[pix[:, 2], pix[:, 1], pix[:, 0]].astype(np.float64)
    mx = inten.max()
    out = []
    n = len(pix)
    while len(out) < num_spots:
        k = max(1024, 2 * (num_spots - len(out)))
        el = np.floor(rng.random(k) * n).astype(np.int64)
        y = rng.random(k) * mx
        keep = el[y <= inten[el]]
        for e in keep:
            if len(out) == num_spots:
                break
            jx, jy, jz = rng.random(3)
            x = np.float32(pix[e, 0] + jx - 0.5)
            yy = np.float32(pix[e, 1] + jy - 0.5)
            z = np.float32(pix[e, 2] + jz - 0.5)
            out.append((x / np.float32(mag), yy / np.float32(mag), z / np.float32(mag)))
    return np.array(out, np.float32)
