"""Python front end of librfba_srrf.so (ctypes over the C-ABI in
include/rfba_srrf.h).

Mirrors the reference's GradientCalc interface (RFBA Main/GradientCalc/
GradientCalc.h:4-5, kernel.cuh:3-26): ``SRRFGradientCalc``, ``SRRFGetMag`` and
``SRRFGradientCalcGPU`` take and return host float arrays laid out like the
reference's ([t][z][y][x] in, [z][y][x] magnified out), plus the extended
interface (explicit configuration, uint16 input, device tensors, block lists,
plain per-block path). There is no CPU implementation behind this module: if
the CUDA library is missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from pathlib import Path
from typing import Sequence

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "librfba_srrf.so"

RFBA_F32 = 0
RFBA_U16 = 1
RFBA_HOST_PTRS = 0
RFBA_DEVICE_PTRS = 1

STATUS = {0: "OK", -1: "INVALID", -2: "UNSUPPORTED", -3: "NOMEM", -4: "CUDA", -5: "TIMEOUT", -6: "IO"}


class RfbaError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"rfba status {status} ({STATUS.get(status, '?')}): {msg}")
        self.status = status


class SRRFConf(ctypes.Structure):
    """The reference's configuration record (kernel.cuh:3-24)."""

    _fields_ = [("RingRadius", ctypes.c_float), ("Magnification", ctypes.c_int), ("AxesinRing", ctypes.c_int),
                ("MainRange", ctypes.c_int), ("XRange", ctypes.c_int), ("YRange", ctypes.c_int),
                ("ZRange", ctypes.c_int), ("Method", ctypes.c_int), ("ITC", ctypes.c_int),
                ("TRACOrder", ctypes.c_int), ("RemoveCon", ctypes.c_int), ("Renormalize", ctypes.c_int),
                ("GradientSmooth", ctypes.c_int), ("IntensityW", ctypes.c_int), ("blockSizeX", ctypes.c_int),
                ("blockSizeY", ctypes.c_int), ("blockSizeZ", ctypes.c_int)]


class Config(ctypes.Structure):
    """rfba_srrf_config: SRRFConf with one magnification per axis."""

    _fields_ = [("ring_radius", ctypes.c_float), ("mag", ctypes.c_int * 3), ("axes_in_ring", ctypes.c_int),
                ("main_range", ctypes.c_int), ("x_range", ctypes.c_int), ("y_range", ctypes.c_int),
                ("z_range", ctypes.c_int), ("method", ctypes.c_int), ("itc", ctypes.c_int),
                ("trac_order", ctypes.c_int), ("remove_con", ctypes.c_int), ("renormalize", ctypes.c_int),
                ("gradient_smooth", ctypes.c_int), ("intensity_w", ctypes.c_int), ("block_size", ctypes.c_int * 3)]

    @classmethod
    def make(cls, **kw) -> "Config":
        """Defaults of GradientCalc.cpp:19-41, overridden by keyword; ``mag`` may
        be an int or a 3-sequence (x, y, z)."""
        c = cls()
        _check(lib().rfba_srrf_config_default(ctypes.byref(c)))
        for k, v in kw.items():
            if k == "mag":
                v = (v, v, v) if isinstance(v, int) else tuple(v)
                for i in range(3):
                    c.mag[i] = int(v[i])
            elif k == "block_size":
                v = (v, v, v) if isinstance(v, int) else tuple(v)
                for i in range(3):
                    c.block_size[i] = int(v[i])
            else:
                setattr(c, k, v)
        return c

    @classmethod
    def from_ini(cls, path: str) -> "Config":
        c = cls()
        _check(lib().rfba_srrf_config_load_ini(str(path).encode(), ctypes.byref(c)))
        return c

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["mag"] = tuple(self.mag)
        d["block_size"] = tuple(self.block_size)
        return d


class ThreeBModel(ctypes.Structure):
    """rfba_3b_model: the 3B spot model (states on / off / bleached)."""

    _fields_ = [("A", ctypes.c_double * 9), ("pi", ctypes.c_double * 3), ("variance", ctypes.c_double),
                ("z_factor", ctypes.c_double), ("mu_brightness", ctypes.c_double),
                ("sigma_brightness", ctypes.c_double), ("mu_blur", ctypes.c_double), ("sigma_blur", ctypes.c_double)]

    @classmethod
    def make(cls, A, pi, variance=1.0, z_factor=1.0, mu_brightness=3.5, sigma_brightness=1.0, mu_blur=0.252148,
             sigma_blur=0.1) -> "ThreeBModel":
        m = cls()
        m.A[:] = [float(v) for v in np.asarray(A, np.float64).reshape(9)]
        m.pi[:] = [float(v) for v in np.asarray(pi, np.float64).reshape(3)]
        m.variance, m.z_factor = variance, z_factor
        m.mu_brightness, m.sigma_brightness, m.mu_blur, m.sigma_blur = mu_brightness, sigma_brightness, mu_blur, sigma_blur
        return m


class ThreeBFitParams(ctypes.Structure):
    """rfba_3b_fit_params: settings of a 3B block fit (FitSpots), defaults the
    shipped multispot5.cfg's."""

    _fields_ = [("main_passes", ctypes.c_int), ("main_samples", ctypes.c_int),
                ("main_cg_max_iterations", ctypes.c_int), ("sweeps", ctypes.c_int),
                ("add_remove_tries", ctypes.c_int), ("opt_samples", ctypes.c_int), ("opt_attempts", ctypes.c_int),
                ("opt_hess_inner_samples", ctypes.c_int), ("h_outer_samples", ctypes.c_int),
                ("h_inner_samples", ctypes.c_int), ("thermo_samples", ctypes.c_int),
                ("limit", ctypes.c_double * 5), ("position_extra_radius", ctypes.c_double),
                ("guide_map", ctypes.c_void_p), ("guide_dims", ctypes.c_int * 3), ("guide_mag", ctypes.c_int)]

    @classmethod
    def make(cls, limit, guide=None, guide_mag: int = 1, **kw) -> "ThreeBFitParams":
        """guide: the SRRF map [z][y][x] proposed spots are drawn from
        (add_guide = 1), in the pixels' coordinates magnified by guide_mag."""
        p = cls()
        d = dict(main_passes=4, main_samples=10, main_cg_max_iterations=5, sweeps=1, add_remove_tries=10,
                 opt_samples=20, opt_attempts=10, opt_hess_inner_samples=1000, h_outer_samples=100,
                 h_inner_samples=1000, thermo_samples=1000, position_extra_radius=2.3)
        d.update(kw)
        for k, v in d.items():
            setattr(p, k, v)
        p.limit[:] = [float(v) for v in np.asarray(limit, np.float64).reshape(5)]
        if guide is not None:
            g = np.ascontiguousarray(guide, np.float32)
            p._guide = g  # kept alive with the settings
            p.guide_map = g.ctypes.data
            p.guide_dims[:] = [g.shape[2], g.shape[1], g.shape[0]]
            p.guide_mag = int(guide_mag)
        return p


class ThreeBModifyRecord(ctypes.Structure):
    """rfba_3b_modify_record: what one model modification did."""

    _fields_ = [("added", ctypes.c_int), ("kept", ctypes.c_int), ("zero_prior", ctypes.c_int),
                ("bad_hessian", ctypes.c_int), ("evaluations", ctypes.c_int), ("model1_energy", ctypes.c_double),
                ("model2_energy", ctypes.c_double), ("occam", ctypes.c_double),
                ("position_log_prior", ctypes.c_double), ("spot", ctypes.c_double * 5)]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["spot"] = list(self.spot)
        return d


FIT_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                          ctypes.c_void_p)


class Block(ctypes.Structure):
    """rfba_block: an independent input sub-volume and the magnified region of
    it that is computed and written."""

    _fields_ = [("origin", ctypes.c_int32 * 3), ("size", ctypes.c_int32 * 3), ("lo", ctypes.c_int32 * 3),
                ("hi", ctypes.c_int32 * 3), ("out_offset", ctypes.c_int64), ("out_stride", ctypes.c_int64 * 3)]


GRAD5_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                            ctypes.c_void_p)

_lib_handle = None


def lib():
    """The loaded CUDA library; raises if it was not built."""
    global _lib_handle
    if _lib_handle is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m rfba_gb300.build` "
                              "(the SRRF path has no CPU fallback)")
        L = ctypes.CDLL(str(LIB_PATH))
        vp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)
        fp = ctypes.POINTER(ctypes.c_float)
        cp = ctypes.POINTER(Config)
        bp = ctypes.POINTER(Block)
        L.rfba_last_error.restype = ctypes.c_char_p
        L.rfba_version.restype = ctypes.c_char_p
        L.rfba_ctx_create.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(vp)]
        L.rfba_ctx_destroy.argtypes = [vp]
        L.rfba_ctx_set_timing.argtypes = [vp, ctypes.c_int]
        L.rfba_ctx_last_timing.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_longlong)]
        L.rfba_ctx_set_launch.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        L.rfba_ctx_set_time_batch.argtypes = [vp, ctypes.c_int]
        L.rfba_ctx_last_time_batches.argtypes = [vp, ip, ip, ip]
        L.rfba_ctx_last_schedule.argtypes = [vp, ip, ip, ip, ip]
        L.rfba_combine_psf.argtypes = [ctypes.c_double, ctypes.c_double, vp, ctypes.c_longlong, ip]
        L.rfba_combine_load_result.argtypes = [ctypes.c_char_p, ctypes.c_int, ip, ip, vp, ctypes.c_longlong,
                                               ctypes.POINTER(ctypes.c_longlong)]
        L.rfba_combine_render.argtypes = [vp, vp, ctypes.c_longlong, ip, ctypes.c_int, vp, ip, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, vp, ctypes.POINTER(ctypes.c_longlong)]
        L.rfba_srrf_seed_spots.argtypes = [vp, vp, ip, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong,
                                           vp, ctypes.c_int, vp]
        L.rfba_srrf_config_default.argtypes = [cp]
        L.rfba_srrf_config_load_ini.argtypes = [ctypes.c_char_p, cp]
        L.rfba_srrf_config_from_legacy.argtypes = [ctypes.POINTER(SRRFConf), cp]
        L.rfba_srrf_forward.argtypes = [vp, cp, vp, ctypes.c_int, ip, vp, ctypes.c_int, vp]
        L.rfba_srrf_forward_blocks.argtypes = [vp, cp, vp, ctypes.c_int, ip, bp, ctypes.c_int, vp, ctypes.c_int64,
                                               ctypes.c_int, vp]
        L.rfba_srrf_forward_blocks_plain.argtypes = [vp, cp, vp, ctypes.c_int, ip, bp, ctypes.c_int, vp,
                                                     ctypes.c_int64]
        L.rfba_blocks_gradientcalc.argtypes = [cp, ip, bp, ctypes.c_int]
        L.rfba_blocks_dosplit.argtypes = [cp, ip, ip, ctypes.c_int, bp, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]
        L.rfba_srrf_plan_info.argtypes = [cp, ip, ip, ip, ip]
        L.rfba_srrf_forward_shifted.argtypes = [vp, cp, vp, vp, ip, vp, vp]
        L.rfba_srrf_backward.argtypes = [vp, cp, vp, vp, ip, vp, vp, vp, vp]
        L.rfba_srrf_forward_shifted_region.argtypes = [vp, cp, vp, vp, ip, ip, ip, vp, vp]
        L.rfba_srrf_backward_region.argtypes = [vp, cp, vp, vp, ip, ip, ip, vp, vp, vp, vp]
        L.rfba_ctx_last_backward_ms.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
        L.rfba_ctx_check.argtypes = [vp]
        dp = ctypes.POINTER(ctypes.c_double)
        L.rfba_3b_spot_gradient.argtypes = [vp, ctypes.POINTER(ThreeBModel), vp, vp, vp, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, dp, dp, dp, ctypes.c_int, vp]
        ipp = ctypes.POINTER(ctypes.c_int)
        ull = ctypes.c_ulonglong
        L.rfba_3b_spot_masks.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, vp, vp, ctypes.c_longlong,
                                         ctypes.POINTER(ctypes.c_longlong)]
        L.rfba_3b_gibbs_sample.argtypes = [vp, ctypes.POINTER(ThreeBModel), vp, vp, vp, vp, vp, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ull, ctypes.c_int,
                                           vp, vp, ctypes.c_int, vp]
        L.rfba_3b_gibbs_trace.argtypes = [vp, ctypes.POINTER(ThreeBModel), vp, vp, vp, vp, vp, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, ull, vp, vp, vp, ctypes.c_int, vp]
        L.rfba_3b_free_energy.argtypes = [vp, ctypes.POINTER(ThreeBModel), vp, vp, vp, vp, vp, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ull,
                                          ctypes.POINTER(ctypes.c_double), vp, ctypes.c_int, vp]
        L.rfba_3b_optimise_pass.argtypes = [vp, ctypes.POINTER(ThreeBModel), vp, vp, ctypes.c_int, ctypes.c_int, vp,
                                            ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, vp, ctypes.c_double, ull, ctypes.POINTER(ctypes.c_int)]
        L.rfba_3b_pass_seed.argtypes = [ull, ctypes.c_int, ctypes.c_int]
        L.rfba_3b_pass_seed.restype = ull
        L.rfba_3b_optimise_spot.argtypes = [vp, ctypes.POINTER(ThreeBModel), vp, vp, vp, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, dp, dp, ctypes.c_int, dp, ipp, ipp, ctypes.c_int, vp]
        L.rfba_cg_only_run.argtypes = [dp, dp, ctypes.c_int, GRAD5_FN, vp, dp, ipp, ipp]
        L.rfba_3b_spot_hessian.argtypes = [vp, ctypes.POINTER(ThreeBModel), vp, vp, vp, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, dp, ctypes.c_int, ull, dp, ctypes.c_int, vp]
        L.rfba_3b_modify_model.argtypes = [vp, ctypes.POINTER(ThreeBModel), vp, vp, ctypes.c_int, ctypes.c_int, vp,
                                           ipp, ctypes.c_int, ctypes.POINTER(ThreeBFitParams), ull,
                                           ctypes.POINTER(ThreeBModifyRecord)]
        L.rfba_3b_fit.argtypes = [vp, ctypes.POINTER(ThreeBModel), vp, vp, ctypes.c_int, ctypes.c_int, vp, ipp,
                                  ctypes.c_int, ctypes.POINTER(ThreeBFitParams), ctypes.c_int, ctypes.c_int, ull,
                                  FIT_FN, vp]
        L.rfba_3b_free_energy_hessian.argtypes = [vp, ctypes.POINTER(ThreeBModel), vp, vp, vp, ctypes.c_int,
                                                  ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                  ull, dp]
        L.rfba_3b_free_energy_models.argtypes = [vp, ctypes.POINTER(ThreeBModel), vp, vp, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, vp, vp, vp, vp, ctypes.c_int, ctypes.c_int, vp, dp]
        L.rfba_3b_support_masks.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, ctypes.c_double, vp, vp,
                                            ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]
        L.rfba_sym_eigen5.argtypes = [dp, dp, dp]
        L.rfba_det5.argtypes = [dp]
        L.rfba_det5.restype = ctypes.c_double
        L.rfba_probe_fp32_fma_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.SRRFGradientCalc.argtypes = [fp, ip, fp]
        L.SRRFGetMag.argtypes = []
        L.SRRFGradientCalcGPU.argtypes = [fp, ip, fp, ctypes.POINTER(SRRFConf)]
        _lib_handle = L
    return _lib_handle


def last_error() -> str:
    return lib().rfba_last_error().decode()


def _check(status: int):
    if status < 0:
        raise RfbaError(status, last_error())
    return status


def _dims(shape: Sequence[int]) -> np.ndarray:
    T, D, H, W = shape
    return np.array([W, H, D, T], np.int32)


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


# ---- reference-compatible entry points ------------------------------------

def SRRFGradientCalc(in_image: np.ndarray) -> np.ndarray:
    """GradientCalc.cpp:169 on a float32 [T][D][H][W] array; reads ./SRRF.ini.
    Returns the magnified map [D*m][H*m][W*m]."""
    a = np.ascontiguousarray(in_image, np.float32)
    dims = _dims(a.shape)
    m = SRRFGetMag()
    out = np.empty((a.shape[1] * m, a.shape[2] * m, a.shape[3] * m), np.float32)
    _check(lib().SRRFGradientCalc(_fptr(a), _iptr(dims), _fptr(out)))
    return out


def SRRFGetMag() -> int:
    return int(lib().SRRFGetMag())


def SRRFGradientCalcGPU(in_image: np.ndarray, conf: SRRFConf) -> np.ndarray:
    """kernel.cu:560: one block, explicit SRRFConf, full magnified output."""
    a = np.ascontiguousarray(in_image, np.float32)
    dims = _dims(a.shape)
    m = conf.Magnification
    out = np.empty((a.shape[1] * m, a.shape[2] * m, a.shape[3] * m), np.float32)
    _check(lib().SRRFGradientCalcGPU(_fptr(a), _iptr(dims), _fptr(out), ctypes.byref(conf)))
    return out


def plan_info(cfg: "Config") -> dict:
    """Ring factorisation the kernels use: distinct points, (x, y) pairs, x
    values, and the reference's raw sample count."""
    v = [ctypes.c_int() for _ in range(4)]
    _check(lib().rfba_srrf_plan_info(ctypes.byref(cfg), *[ctypes.byref(x) for x in v]))
    return {"points": v[0].value, "pairs": v[1].value, "xvalues": v[2].value, "raw": v[3].value}


def probe_fp32_fma_peak(device: int = 0) -> float:
    """Measured FP32 FMA throughput of the device, TFLOP/s."""
    v = ctypes.c_double()
    _check(lib().rfba_probe_fp32_fma_peak(device, ctypes.byref(v)))
    return v.value


def flops_per_voxel_volume(cfg: "Config") -> float:
    """Flops per output voxel-volume of the separable method as implemented
    (FMA = 2): per distinct ring point, the 4-tap z interpolation of three
    gradient components (21) and the radiality term in the rotated frame (21);
    per (x, y) pair, the 4-tap y pass and the frame rotation over coarse z
    ((21 + 6) / mag_z); per x value, the 4-tap x pass (21 / (mag_y mag_z)); the
    smoothed gradient (162 / (mag_x mag_y mag_z)); the intensity interpolation
    (9) and the temporal reduction (10)."""
    info = plan_info(cfg)
    mx, my, mz = cfg.mag[0], cfg.mag[1], cfg.mag[2]
    return (info["points"] * 42 + info["pairs"] * 27.0 / mz + info["xvalues"] * 21.0 / (my * mz)
            + 162.0 / (mx * my * mz) + 9 + 10)


# ---- block lists -------------------------------------------------------------

def blocks_gradientcalc(cfg: Config, shape: Sequence[int]):
    """GradientCalc.cpp:47-116 blocks (border 2) for an input [T][D][H][W]."""
    dims = _dims(shape)
    n = _check(lib().rfba_blocks_gradientcalc(ctypes.byref(cfg), _iptr(dims), None, 0))
    arr = (Block * max(n, 1))()
    _check(lib().rfba_blocks_gradientcalc(ctypes.byref(cfg), _iptr(dims), arr, n))
    return arr, n


def blocks_dosplit(cfg: Config, shape: Sequence[int], max_size, border: int):
    """doSplit.m blocks; each block's whole magnified output packed in order.
    Returns (blocks, count, out_elems)."""
    dims = _dims(shape)
    ms = np.array(max_size if not isinstance(max_size, int) else (max_size,) * 3, np.int32)
    oe = ctypes.c_int64()
    n = _check(lib().rfba_blocks_dosplit(ctypes.byref(cfg), _iptr(dims), _iptr(ms), border, None, 0, ctypes.byref(oe)))
    arr = (Block * max(n, 1))()
    _check(lib().rfba_blocks_dosplit(ctypes.byref(cfg), _iptr(dims), _iptr(ms), border, arr, n, ctypes.byref(oe)))
    return arr, n, int(oe.value)


def cg_only_run(grad, start, limit, max_iterations: int):
    """ConjugateGradientOnly<5> (conjugate_gradient_only.h) on the host with a
    Python gradient function grad(x: ndarray[5]) -> ndarray[5]: returns (final
    x, line searches, gradient evaluations)."""
    err = []

    def cb(x, g, user):
        try:
            v = np.asarray(grad(np.ctypeslib.as_array(x, (5,)).copy()), np.float64)
            for i in range(5):
                g[i] = float(v[i])
            return 0
        except Exception as e:  # stop the run, re-raised below
            err.append(e)
            return -1

    fn = GRAD5_FN(cb)
    dp = ctypes.POINTER(ctypes.c_double)
    st = np.ascontiguousarray(start, np.float64)
    lim = np.ascontiguousarray(limit, np.float64)
    out = np.zeros(5)
    it, ev = ctypes.c_int(), ctypes.c_int()
    rc = lib().rfba_cg_only_run(st.ctypes.data_as(dp), lim.ctypes.data_as(dp), int(max_iterations), fn, None,
                                out.ctypes.data_as(dp), ctypes.byref(it), ctypes.byref(ev))
    if err:
        raise err[0]
    _check(rc)
    return out, it.value, ev.value


def combine_psf(sigma: float = 3.5, crop_threshold: float = 1000.0) -> np.ndarray:
    """genpsf.m: the uint16 PSF of the CombineBlock reconstruction, [z][y][x]."""
    dims = np.zeros(3, np.int32)
    n = _check(lib().rfba_combine_psf(sigma, crop_threshold, None, 0, _iptr(dims)))
    out = np.empty(n, np.uint16)
    _check(lib().rfba_combine_psf(sigma, crop_threshold, ctypes.c_void_p(out.ctypes.data), n, _iptr(dims)))
    return out.reshape(int(dims[2]), int(dims[1]), int(dims[0]))


def combine_load_result(path, border: int, block_start, block_size) -> np.ndarray:
    """loadResult.m on one res_i_j_k.txt: spots (intensity, blur, x, y, z) inside the block."""
    st = np.array(block_start, np.int32)
    sz = np.array(block_size, np.int32)
    n = ctypes.c_longlong()
    _check(lib().rfba_combine_load_result(str(path).encode(), border, _iptr(st), _iptr(sz), None, 0,
                                          ctypes.byref(n)))
    out = np.empty((n.value, 5), np.float64)
    _check(lib().rfba_combine_load_result(str(path).encode(), border, _iptr(st), _iptr(sz),
                                          ctypes.c_void_p(out.ctypes.data), n.value, ctypes.byref(n)))
    return out


def dosplit(xall: int, max_size: int, border: int):
    """doSplit.m: (start (1-based), size) of the blocks along one axis."""
    if max_size >= xall:
        return [(1, xall)]
    pos = [[1, max_size]]
    while pos[-1][0] + max_size <= xall:
        pos.append([pos[-1][0] + pos[-1][1] - 2 * border, max_size])
    pos[-1][1] = xall - pos[-1][0] + 1
    return [tuple(p) for p in pos]


# ---- extended interface --------------------------------------------------------

@dataclass
class Timing:
    radiality_ms: float
    temporal_ms: float
    launches: int


class Context:
    """A device context: scratch buffers, ring plan cache, stream."""

    def __init__(self, device: int = 0, scratch_budget_bytes: int = 0):
        h = ctypes.c_void_p()
        _check(lib().rfba_ctx_create(device, scratch_budget_bytes, ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().rfba_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_timing(self, on: bool):
        _check(lib().rfba_ctx_set_timing(self.h, int(on)))

    def set_launch(self, grid: int = 0, t_chunk: int = 0):
        _check(lib().rfba_ctx_set_launch(self.h, grid, t_chunk))

    def set_time_batch(self, volumes: int = 0):
        """Time batches of forward / forward_blocks: 0 automatic (batches of 25
        volumes when the whole series' stacks do not fit the scratch budget),
        > 0 always batches of that many volumes, < 0 never."""
        _check(lib().rfba_ctx_set_time_batch(self.h, int(volumes)))

    def last_time_batches(self):
        """(volumes per batch, batches) of the last forward; (0, 0) when it
        reduced the whole series in one pass."""
        v, b = ctypes.c_int(0), ctypes.c_int(0)
        _check(lib().rfba_ctx_last_time_batches(self.h, ctypes.byref(v), ctypes.byref(b), None))
        return v.value, b.value

    def last_passes(self) -> int:
        """Spatial passes of the last forward (z slices or block groups)."""
        n = ctypes.c_int(0)
        _check(lib().rfba_ctx_last_time_batches(self.h, None, None, ctypes.byref(n)))
        return n.value

    def combine_render(self, spots, img_dims, zoom: int = 10, psf=None, noise_r: int = 30, noise_rz: int = 3,
                       noise_threshold: int = 70):
        """CombineBlock.m:24-173 on the GPU: uint16 volume [Z*zoom][Y*zoom][X*zoom] and the number of
        spots that fell outside the grid."""
        if psf is None:
            psf = combine_psf()
        psf = np.ascontiguousarray(psf, np.uint16)
        sp = np.ascontiguousarray(spots, np.float64).reshape(-1, 5)
        X, Y, Z = (int(d) for d in img_dims)
        out = np.empty((Z * zoom, Y * zoom, X * zoom), np.uint16)
        dims = np.array([X, Y, Z], np.int32)
        pd = np.array([psf.shape[2], psf.shape[1], psf.shape[0]], np.int32)
        dropped = ctypes.c_longlong()
        _check(lib().rfba_combine_render(self.h, ctypes.c_void_p(sp.ctypes.data) if len(sp) else None, len(sp),
                                         _iptr(dims), zoom, ctypes.c_void_p(psf.ctypes.data), _iptr(pd), noise_r,
                                         noise_rz, noise_threshold, ctypes.c_void_p(out.ctypes.data),
                                         ctypes.byref(dropped)))
        return out, dropped.value

    def combine_blocks(self, res_dir, img_dims, block_dims, border: int, zoom: int = 10, sigma: float = 3.5,
                       psf_threshold: float = 1000.0, noise_r: int = 30, noise_rz: int = 3,
                       noise_threshold: int = 70):
        """CombineBlock.m end to end: res_i_j_k.txt of every doSplit block (i, j, k 1-based, x outer),
        loadResult filter, then the GPU reconstruction."""
        xs, ys, zs = (dosplit(int(img_dims[a]), int(block_dims[a]), border) for a in range(3))
        parts = []
        for i, (sx, nx) in enumerate(xs, 1):
            for j, (sy, ny) in enumerate(ys, 1):
                for k, (sz, nz) in enumerate(zs, 1):
                    p = Path(res_dir) / f"res_{i}_{j}_{k}.txt"
                    if p.exists():
                        parts.append(combine_load_result(p, border, (sx, sy, sz), (nx, ny, nz)))
        spots = np.concatenate(parts) if parts else np.zeros((0, 5))
        return self.combine_render(spots, img_dims, zoom, combine_psf(sigma, psf_threshold), noise_r, noise_rz,
                                   noise_threshold)

    def seed_spots(self, srrf_map, voxels, mag: int, num_spots: int, seed: int = 0, stream=None):
        """SRRF-guided spot seeding (multispot5_place_methods.cc:291-341): num_spots
        positions [n][3] (x, y, z, input voxels) drawn with density proportional to
        the map over the mag^3 subvoxels of each input voxel in ``voxels`` ([n][3]
        x, y, z). ``srrf_map`` is [z][y][x] float32, numpy (host) or a CUDA tensor."""
        dev = not isinstance(srrf_map, np.ndarray)
        vox = np.ascontiguousarray(voxels, np.int32).reshape(-1, 3)
        if dev:
            import torch
            m = srrf_map.contiguous()
            vd = torch.from_numpy(vox).to(m.device)
            out = torch.empty((num_spots, 3), dtype=torch.float32, device=m.device)
            mp, vp_, op = ctypes.c_void_p(m.data_ptr()), ctypes.c_void_p(vd.data_ptr()), ctypes.c_void_p(out.data_ptr())
            shape = m.shape
        else:
            m = np.ascontiguousarray(srrf_map, np.float32)
            out = np.empty((num_spots, 3), np.float32)
            mp, vp_, op = (ctypes.c_void_p(m.ctypes.data), ctypes.c_void_p(vox.ctypes.data),
                           ctypes.c_void_p(out.ctypes.data))
            shape = m.shape
        dims = np.array([shape[2], shape[1], shape[0]], np.int32)
        st = _stream_arg(stream, dev)
        _check(lib().rfba_srrf_seed_spots(self.h, mp, _iptr(dims), mag, vp_, len(vox), num_spots, seed, op,
                                          RFBA_DEVICE_PTRS if dev else RFBA_HOST_PTRS, st))
        return out

    def schedule(self) -> dict:
        """Schedule of the last forward: tile rows, tile order, graph replay, autotuned now."""
        v = [ctypes.c_int() for _ in range(4)]
        _check(lib().rfba_ctx_last_schedule(self.h, *[ctypes.byref(x) for x in v]))
        return {"tile_rows": v[0].value, "tile_order": v[1].value, "graph": bool(v[2].value),
                "tuned": bool(v[3].value)}

    def timing(self) -> Timing:
        a, b, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        _check(lib().rfba_ctx_last_timing(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(n)))
        return Timing(a.value, b.value, n.value)

    @staticmethod
    def _in(x):
        """(pointer, dtype code, dims, is_device) of a numpy array or torch tensor."""
        if isinstance(x, np.ndarray):
            if x.dtype == np.uint16:
                dt = RFBA_U16
            elif x.dtype == np.float32:
                dt = RFBA_F32
            else:
                raise TypeError("input must be uint16 or float32")
            if not x.flags.c_contiguous:
                raise ValueError("input must be C-contiguous")
            return ctypes.c_void_p(x.ctypes.data), dt, _dims(x.shape), False
        import torch  # device tensors
        if x.dtype == torch.uint16 if hasattr(torch, "uint16") else False:
            dt = RFBA_U16
        elif x.dtype == torch.float32:
            dt = RFBA_F32
        elif str(x.dtype) == "torch.int16":  # uint16 bits carried in int16
            dt = RFBA_U16
        else:
            raise TypeError("input must be uint16 or float32")
        if not x.is_contiguous():
            raise ValueError("input must be contiguous")
        return ctypes.c_void_p(x.data_ptr()), dt, _dims(tuple(x.shape)), x.is_cuda

    def forward(self, cfg: Config, x, out=None, stream=None):
        """Whole volume as one block. x: numpy [T][D][H][W] (host) or a CUDA
        tensor (device); returns / fills the map [D*mz][H*my][W*mx]."""
        ptr, dt, dims, dev = self._in(x)
        shape = (int(dims[2]) * cfg.mag[2], int(dims[1]) * cfg.mag[1], int(dims[0]) * cfg.mag[0])
        if out is None:
            if dev:
                import torch
                out = torch.empty(shape, dtype=torch.float32, device=x.device)
            else:
                out = np.empty(shape, np.float32)
        optr = ctypes.c_void_p(out.data_ptr() if dev else out.ctypes.data)
        st = _stream_arg(stream, dev)
        _check(lib().rfba_srrf_forward(self.h, ctypes.byref(cfg), ptr, dt, _iptr(dims), optr,
                                       RFBA_DEVICE_PTRS if dev else RFBA_HOST_PTRS, st))
        return out

    def forward_blocks(self, cfg: Config, x, blocks, nblocks: int, out_elems: int, out=None, stream=None):
        ptr, dt, dims, dev = self._in(x)
        if out is None:
            if dev:
                import torch
                out = torch.zeros(out_elems, dtype=torch.float32, device=x.device)
            else:
                out = np.zeros(out_elems, np.float32)
        optr = ctypes.c_void_p(out.data_ptr() if dev else out.ctypes.data)
        st = _stream_arg(stream, dev)
        _check(lib().rfba_srrf_forward_blocks(self.h, ctypes.byref(cfg), ptr, dt, _iptr(dims), blocks, nblocks, optr,
                                              out_elems, RFBA_DEVICE_PTRS if dev else RFBA_HOST_PTRS, st))
        return out

    def forward_shifted(self, cfg: Config, x, shifts=None, out=None, stream=None):
        """Drift-corrected forward on device tensors: x float32 [T][D][H][W],
        shifts float32 [T][3] (x, y, z) or None. Keeps the stacks for backward."""
        import torch
        T, D, H, W = x.shape
        dims = _dims(x.shape)
        if out is None:
            out = torch.empty((D * cfg.mag[2], H * cfg.mag[1], W * cfg.mag[0]), dtype=torch.float32, device=x.device)
        sp = ctypes.c_void_p(shifts.data_ptr()) if shifts is not None else None
        st = _stream_arg(stream, True)
        _check(lib().rfba_srrf_forward_shifted(self.h, ctypes.byref(cfg), ctypes.c_void_p(x.data_ptr()), sp,
                                               _iptr(dims), ctypes.c_void_p(out.data_ptr()), st))
        return out

    def backward(self, cfg: Config, x, shifts, dL_dmap, din=None, dshift=None, stream=None):
        """Adjoint of forward_shifted: returns (dL/dx, dL/dshifts or None)."""
        import torch
        dims = _dims(x.shape)
        if din is None:
            din = torch.empty_like(x)
        if dshift is None and shifts is not None:
            dshift = torch.empty_like(shifts)
        sp = ctypes.c_void_p(shifts.data_ptr()) if shifts is not None else None
        dsp = ctypes.c_void_p(dshift.data_ptr()) if dshift is not None else None
        st = _stream_arg(stream, True)
        _check(lib().rfba_srrf_backward(self.h, ctypes.byref(cfg), ctypes.c_void_p(x.data_ptr()), sp, _iptr(dims),
                                        ctypes.c_void_p(dL_dmap.data_ptr()), ctypes.c_void_p(din.data_ptr()), dsp,
                                        st))
        return din, dshift

    def forward_shifted_region(self, cfg: Config, x, shifts, lo, hi, out=None, stream=None):
        """forward_shifted restricted to the fine region [lo, hi) (x, y, z):
        returns the region [z][y][x]."""
        import torch
        dims = _dims(x.shape)
        if out is None:
            out = torch.empty((hi[2] - lo[2], hi[1] - lo[1], hi[0] - lo[0]), dtype=torch.float32, device=x.device)
        sp = ctypes.c_void_p(shifts.data_ptr()) if shifts is not None else None
        st = _stream_arg(stream, True)
        _check(lib().rfba_srrf_forward_shifted_region(self.h, ctypes.byref(cfg), ctypes.c_void_p(x.data_ptr()), sp,
                                                      _iptr(dims), _iptr(np.asarray(lo, np.int32)),
                                                      _iptr(np.asarray(hi, np.int32)),
                                                      ctypes.c_void_p(out.data_ptr()), st))
        return out

    def backward_region(self, cfg: Config, x, shifts, lo, hi, dL_dregion, din=None, dshift=None, stream=None):
        """The region's contribution to the adjoint of forward_shifted:
        returns (dL/dx, dL/dshifts or None)."""
        import torch
        dims = _dims(x.shape)
        if din is None:
            din = torch.empty_like(x)
        if dshift is None and shifts is not None:
            dshift = torch.empty_like(shifts)
        sp = ctypes.c_void_p(shifts.data_ptr()) if shifts is not None else None
        dsp = ctypes.c_void_p(dshift.data_ptr()) if dshift is not None else None
        st = _stream_arg(stream, True)
        _check(lib().rfba_srrf_backward_region(self.h, ctypes.byref(cfg), ctypes.c_void_p(x.data_ptr()), sp,
                                               _iptr(dims), _iptr(np.asarray(lo, np.int32)),
                                               _iptr(np.asarray(hi, np.int32)),
                                               ctypes.c_void_p(dL_dregion.data_ptr()),
                                               ctypes.c_void_p(din.data_ptr()), dsp, st))
        return din, dshift

    def spot_gradient_3b(self, model: ThreeBModel, sample_bg, pix, pixels, spot, stream=None,
                         want_log_prob: bool = True):
        """SpotNegProbabilityDiffWithSampledBackground (multispot5.cc:616-664) on the
        GPU: returns (gradient [5], log probability per sample [S] or None).
        sample_bg [S][F][P], pix [F][P] (float64) and pixels [P][3] (int32) are
        numpy arrays (copied in) or CUDA tensors. Without the log probabilities
        the sums run in double-float arithmetic, as the optimisers run them."""
        dev = not isinstance(sample_bg, np.ndarray)
        if dev:
            S, F, P = (int(v) for v in sample_bg.shape)
            ptrs = [ctypes.c_void_p(t.data_ptr()) for t in (sample_bg, pix, pixels)]
        else:
            sample_bg = np.ascontiguousarray(sample_bg, np.float64)
            pix = np.ascontiguousarray(pix, np.float64)
            pixels = np.ascontiguousarray(pixels, np.int32)
            S, F, P = sample_bg.shape
            ptrs = [ctypes.c_void_p(a.ctypes.data) for a in (sample_bg, pix, pixels)]
        sp = np.ascontiguousarray(spot, np.float64)
        out = np.zeros(5)
        logp = np.zeros(S) if want_log_prob else None
        dp = ctypes.POINTER(ctypes.c_double)
        _check(lib().rfba_3b_spot_gradient(self.h, ctypes.byref(model), *ptrs, S, F, P, sp.ctypes.data_as(dp),
                                           out.ctypes.data_as(dp), logp.ctypes.data_as(dp) if want_log_prob else None,
                                           RFBA_DEVICE_PTRS if dev else RFBA_HOST_PTRS, _stream_arg(stream, dev)))
        return out, logp

    def optimise_spot_3b(self, model: ThreeBModel, sample_bg, pix, pixels, spot, limit, max_iterations: int,
                         stream=None):
        """3B's spot optimisation (multispot5.cc:1614-1636, ConjugateGradientOnly<5>)
        with the GPU spot gradient on data staged once: returns (final spot [5],
        line searches, gradient evaluations). Arguments as spot_gradient_3b, plus
        the per-parameter motion limits and the iteration limit."""
        dev = not isinstance(sample_bg, np.ndarray)
        if dev:
            S, F, P = (int(v) for v in sample_bg.shape)
            ptrs = [ctypes.c_void_p(t.data_ptr()) for t in (sample_bg, pix, pixels)]
        else:
            sample_bg = np.ascontiguousarray(sample_bg, np.float64)
            pix = np.ascontiguousarray(pix, np.float64)
            pixels = np.ascontiguousarray(pixels, np.int32)
            S, F, P = sample_bg.shape
            ptrs = [ctypes.c_void_p(a.ctypes.data) for a in (sample_bg, pix, pixels)]
        sp = np.ascontiguousarray(spot, np.float64)
        lim = np.ascontiguousarray(limit, np.float64)
        out = np.zeros(5)
        it, ev = ctypes.c_int(), ctypes.c_int()
        dp = ctypes.POINTER(ctypes.c_double)
        _check(lib().rfba_3b_optimise_spot(self.h, ctypes.byref(model), *ptrs, S, F, P, sp.ctypes.data_as(dp),
                                           lim.ctypes.data_as(dp), int(max_iterations), out.ctypes.data_as(dp),
                                           ctypes.byref(it), ctypes.byref(ev),
                                           RFBA_DEVICE_PTRS if dev else RFBA_HOST_PTRS, _stream_arg(stream, dev)))
        return out, it.value, ev.value

    def gibbs_sample_3b(self, model: ThreeBModel, pix, pixels, spots, masks=None, sweeps: int = 1,
                        n_draws: int = 1, seed: int = 0, exclude_spot: int = -1, want_states: bool = True,
                        want_intensities: bool = True):
        """GibbsSampler2 (sampled_multispot.h:360-690) on the GPU from all spots off:
        returns (states [n_draws][K][F] uint8 or None, sample intensities
        [n_draws][F][P] or None). pix [F][P] float64, pixels [P][3] int32 sorted by
        (z, y, x), spots [K][5]; masks = (offsets, indices), default spot_masks_3b."""
        pix = np.ascontiguousarray(pix, np.float64)
        pixels = np.ascontiguousarray(pixels, np.int32)
        spots = np.ascontiguousarray(spots, np.float64).reshape(-1, 5)
        moff, midx = masks if masks is not None else spot_masks_3b(pixels, spots)
        moff = np.ascontiguousarray(moff, np.int32)
        midx = np.ascontiguousarray(midx, np.int32) if len(midx) else np.zeros(1, np.int32)
        F, P = pix.shape
        K = len(spots)
        st = np.empty((n_draws, K, F), np.uint8) if want_states else None
        ints = np.empty((n_draws, F, P)) if want_intensities else None
        vp = ctypes.c_void_p
        _check(lib().rfba_3b_gibbs_sample(self.h, ctypes.byref(model), vp(pix.ctypes.data), vp(pixels.ctypes.data),
                                          vp(spots.ctypes.data), vp(moff.ctypes.data), vp(midx.ctypes.data), K, F, P,
                                          sweeps, n_draws, seed, exclude_spot,
                                          vp(st.ctypes.data) if st is not None else None,
                                          vp(ints.ctypes.data) if ints is not None else None, RFBA_HOST_PTRS, None))
        return st, ints

    def gibbs_trace_3b(self, model: ThreeBModel, pix, pixels, spots, masks=None, seed: int = 0):
        """One sweep from all spots off: (states [K][F], log p(on / off) [K][F][2],
        forward filter [K][F][3])."""
        pix = np.ascontiguousarray(pix, np.float64)
        pixels = np.ascontiguousarray(pixels, np.int32)
        spots = np.ascontiguousarray(spots, np.float64).reshape(-1, 5)
        moff, midx = masks if masks is not None else spot_masks_3b(pixels, spots)
        moff = np.ascontiguousarray(moff, np.int32)
        midx = np.ascontiguousarray(midx, np.int32) if len(midx) else np.zeros(1, np.int32)
        F, P = pix.shape
        K = len(spots)
        st = np.empty((K, F), np.uint8)
        lp = np.empty((K, F, 2))
        filt = np.empty((K, F, 3))
        vp = ctypes.c_void_p
        _check(lib().rfba_3b_gibbs_trace(self.h, ctypes.byref(model), vp(pix.ctypes.data), vp(pixels.ctypes.data),
                                         vp(spots.ctypes.data), vp(moff.ctypes.data), vp(midx.ctypes.data), K, F, P,
                                         seed, vp(st.ctypes.data), vp(lp.ctypes.data), vp(filt.ctypes.data),
                                         RFBA_HOST_PTRS, None))
        return st, lp, filt

    def free_energy_3b(self, model: ThreeBModel, pix, pixels, spots, masks=None, samples: int = 1000,
                       sweeps: int = 1, seed: int = 0):
        """NegativeFreeEnergy::compute_with_mask (multispot5.cc:335-405): returns
        (its value, each draw's sum of squared residuals [samples])."""
        pix = np.ascontiguousarray(pix, np.float64)
        pixels = np.ascontiguousarray(pixels, np.int32)
        spots = np.ascontiguousarray(spots, np.float64).reshape(-1, 5)
        moff, midx = masks if masks is not None else spot_masks_3b(pixels, spots)
        moff = np.ascontiguousarray(moff, np.int32)
        midx = np.ascontiguousarray(midx, np.int32) if len(midx) else np.zeros(1, np.int32)
        F, P = pix.shape
        K = len(spots)
        v = ctypes.c_double()
        res = np.empty(samples)
        vp = ctypes.c_void_p
        _check(lib().rfba_3b_free_energy(self.h, ctypes.byref(model), vp(pix.ctypes.data), vp(pixels.ctypes.data),
                                         vp(spots.ctypes.data), vp(moff.ctypes.data), vp(midx.ctypes.data), K, F, P,
                                         samples, sweeps, seed, ctypes.byref(v), vp(res.ctypes.data),
                                         RFBA_HOST_PTRS, None))
        return v.value, res

    def optimise_pass_3b(self, model: ThreeBModel, pix, pixels, spots, pass_index: int = 0, main_samples: int = 10,
                         sweeps: int = 1, cg_max_iterations: int = 5, limit=None, position_extra_radius: float = -1.0,
                         seed: int = 0):
        """One pass of FitSpots' main loop (multispot5.cc:1511-1690): returns (spots
        [K'][5] after the pass, gradient evaluations)."""
        pix = np.ascontiguousarray(pix, np.float64)
        pixels = np.ascontiguousarray(pixels, np.int32)
        sp = np.ascontiguousarray(spots, np.float64).reshape(-1, 5).copy()
        lim = np.ascontiguousarray(limit if limit is not None else [0.5] * 5, np.float64)
        F, P = pix.shape
        n = ctypes.c_int(len(sp))
        ev = ctypes.c_int()
        vp = ctypes.c_void_p
        _check(lib().rfba_3b_optimise_pass(self.h, ctypes.byref(model), vp(pix.ctypes.data), vp(pixels.ctypes.data),
                                           F, P, vp(sp.ctypes.data), ctypes.byref(n), pass_index, main_samples, sweeps,
                                           cg_max_iterations, vp(lim.ctypes.data), float(position_extra_radius),
                                           seed, ctypes.byref(ev)))
        return sp[:n.value].copy(), ev.value

    def spot_hessian_3b(self, model: ThreeBModel, sample_bg, pix, pixels, spot, bs_iterations: int = 1000,
                        seed: int = 0, stream=None):
        """sampled_background_spot_hessian_ffbs (multispot5.cc:824-985) on the GPU:
        the 5x5 Hessian of the spot's log probability. Arguments as
        spot_gradient_3b."""
        dev = not isinstance(sample_bg, np.ndarray)
        if dev:
            S, F, P = (int(v) for v in sample_bg.shape)
            ptrs = [ctypes.c_void_p(t.data_ptr()) for t in (sample_bg, pix, pixels)]
        else:
            sample_bg = np.ascontiguousarray(sample_bg, np.float64)
            pix = np.ascontiguousarray(pix, np.float64)
            pixels = np.ascontiguousarray(pixels, np.int32)
            S, F, P = sample_bg.shape
            ptrs = [ctypes.c_void_p(a.ctypes.data) for a in (sample_bg, pix, pixels)]
        sp = np.ascontiguousarray(spot, np.float64)
        out = np.zeros((5, 5))
        dp = ctypes.POINTER(ctypes.c_double)
        _check(lib().rfba_3b_spot_hessian(self.h, ctypes.byref(model), *ptrs, S, F, P, sp.ctypes.data_as(dp),
                                          int(bs_iterations), seed, out.ctypes.data_as(dp),
                                          RFBA_DEVICE_PTRS if dev else RFBA_HOST_PTRS, _stream_arg(stream, dev)))
        return out

    def free_energies_3b(self, model: ThreeBModel, pix, pixels, models, samples: int = 1000, sweeps: int = 1,
                         seeds=(0, 1)):
        """rfba_3b_free_energy_models: compute_with_mask's value for one or two
        models (lists of spots [K][5]) side by side; masks from spot_masks_3b."""
        pix = np.ascontiguousarray(pix, np.float64)
        pixels = np.ascontiguousarray(pixels, np.int32)
        F, P = pix.shape
        n = len(models)
        keep = []
        sp_p, off_p, idx_p = (ctypes.c_void_p * n)(), (ctypes.c_void_p * n)(), (ctypes.c_void_p * n)()
        Ks = (ctypes.c_int * n)()
        for i, sp in enumerate(models):
            sp = np.ascontiguousarray(sp, np.float64).reshape(-1, 5)
            off, idx = spot_masks_3b(pixels, sp)
            idx = np.ascontiguousarray(idx if len(idx) else np.zeros(1, np.int32), np.int32)
            keep += [sp, off, idx]
            sp_p[i], off_p[i], idx_p[i], Ks[i] = sp.ctypes.data, off.ctypes.data, idx.ctypes.data, len(sp)
        sd = (ctypes.c_ulonglong * n)(*[int(v) for v in seeds[:n]])
        vals = np.zeros(n)
        _check(lib().rfba_3b_free_energy_models(self.h, ctypes.byref(model), ctypes.c_void_p(pix.ctypes.data),
                                                ctypes.c_void_p(pixels.ctypes.data), F, P, n, sp_p, Ks, off_p, idx_p,
                                                samples, sweeps, sd,
                                                vals.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return vals

    def free_energy_hessian_3b(self, model: ThreeBModel, pix, pixels, spots, spot: int, samples: int = 100,
                               sweeps: int = 1, seed: int = 0):
        """FreeEnergyHessian::hessian (multispot5.cc:693-775): the 5x5 Hessian of
        the negative free energy with respect to spots[spot]."""
        pix = np.ascontiguousarray(pix, np.float64)
        pixels = np.ascontiguousarray(pixels, np.int32)
        sp = np.ascontiguousarray(spots, np.float64).reshape(-1, 5)
        F, P = pix.shape
        out = np.zeros((5, 5))
        vp = ctypes.c_void_p
        _check(lib().rfba_3b_free_energy_hessian(self.h, ctypes.byref(model), vp(pix.ctypes.data),
                                                 vp(pixels.ctypes.data), vp(sp.ctypes.data), len(sp), F, P, spot,
                                                 samples, sweeps, seed,
                                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def modify_model_3b(self, model: ThreeBModel, pix, pixels, spots, params: ThreeBFitParams, seed: int = 0):
        """One try of FitSpots::try_modifying_model (multispot5.cc:1840-2160):
        returns (spots kept [K'][5], record dict)."""
        pix = np.ascontiguousarray(pix, np.float64)
        pixels = np.ascontiguousarray(pixels, np.int32)
        sp0 = np.ascontiguousarray(spots, np.float64).reshape(-1, 5)
        sp = np.zeros((len(sp0) + 1, 5))
        sp[:len(sp0)] = sp0
        F, P = pix.shape
        n = ctypes.c_int(len(sp0))
        rec = ThreeBModifyRecord()
        vp = ctypes.c_void_p
        _check(lib().rfba_3b_modify_model(self.h, ctypes.byref(model), vp(pix.ctypes.data), vp(pixels.ctypes.data), F,
                                          P, vp(sp.ctypes.data), ctypes.byref(n), len(sp), ctypes.byref(params),
                                          seed, ctypes.byref(rec)))
        return sp[:n.value].copy(), rec.as_dict()

    def fit_3b(self, model: ThreeBModel, pix, pixels, spots, params: ThreeBFitParams, iterations: int = 1,
               first_iteration: int = 0, seed: int = 0, capacity: int = 0, progress=None):
        """FitSpots::run (multispot5.cc:2234-2278) on the GPU: returns the spots
        after `iterations` iterations. progress(iteration, step, spots) may
        return True to stop."""
        pix = np.ascontiguousarray(pix, np.float64)
        pixels = np.ascontiguousarray(pixels, np.int32)
        sp0 = np.ascontiguousarray(spots, np.float64).reshape(-1, 5)
        cap = max(capacity, len(sp0) + max(1, params.add_remove_tries) * max(1, iterations) + 1)
        sp = np.zeros((cap, 5))
        sp[:len(sp0)] = sp0
        F, P = pix.shape
        n = ctypes.c_int(len(sp0))

        def cb(it, step, ptr, k, user):
            arr = np.ctypeslib.as_array(ptr, shape=(k * 5,)).reshape(k, 5).copy() if k else np.zeros((0, 5))
            return 1 if (progress is not None and progress(it, step, arr)) else 0

        fn = FIT_FN(cb)
        vp = ctypes.c_void_p
        _check(lib().rfba_3b_fit(self.h, ctypes.byref(model), vp(pix.ctypes.data), vp(pixels.ctypes.data), F, P,
                                 vp(sp.ctypes.data), ctypes.byref(n), cap, ctypes.byref(params), first_iteration,
                                 iterations, seed, fn, None))
        return sp[:n.value].copy()

    def check(self):
        """Wait for this context's queued work and raise RfbaError for a failure its
        kernels recorded (a bounded device wait that gave up: RFBA_ERR_TIMEOUT).
        Device-tensor calls are asynchronous and report only through this."""
        _check(lib().rfba_ctx_check(self.h))

    def last_backward_ms(self) -> float:
        v = ctypes.c_double()
        _check(lib().rfba_ctx_last_backward_ms(self.h, ctypes.byref(v)))
        return v.value

    def forward_blocks_plain(self, cfg: Config, x: np.ndarray, blocks, nblocks: int, out_elems: int, out=None):
        ptr, dt, dims, dev = self._in(x)
        if dev:
            raise ValueError("the plain per-block path takes host arrays")
        if out is None:
            out = np.zeros(out_elems, np.float32)
        _check(lib().rfba_srrf_forward_blocks_plain(self.h, ctypes.byref(cfg), ptr, dt, _iptr(dims), blocks, nblocks,
                                                    ctypes.c_void_p(out.ctypes.data), out_elems))
        return out


def spot_masks_3b(pixels, spots):
    """get_spot_pixels (multispot5.cc:1001-1020) for every spot: (offsets [K+1],
    indices); pixels [P][3] sorted by (z, y, x). Host only."""
    px = np.ascontiguousarray(pixels, np.int32)
    sp = np.ascontiguousarray(spots, np.float64).reshape(-1, 5)
    K, P = len(sp), len(px)
    off = np.zeros(K + 1, np.int32)
    nnz = ctypes.c_longlong()
    vp = ctypes.c_void_p
    _check(lib().rfba_3b_spot_masks(vp(px.ctypes.data), P, vp(sp.ctypes.data), K, vp(off.ctypes.data), None, 0,
                                    ctypes.byref(nnz)))
    idx = np.zeros(max(nnz.value, 1), np.int32)
    _check(lib().rfba_3b_spot_masks(vp(px.ctypes.data), P, vp(sp.ctypes.data), K, vp(off.ctypes.data),
                                    vp(idx.ctypes.data), nnz.value, ctypes.byref(nnz)))
    return off, idx[:nnz.value]


def support_masks_3b(pixels, spots, z_factor: float = 1.0):
    """Each spot's support (Gaussian factor >= 2^-60) in pixel order, the masks of
    the library's unmasked sampler: (offsets [K+1], indices). Host only."""
    px = np.ascontiguousarray(pixels, np.int32)
    sp = np.ascontiguousarray(spots, np.float64).reshape(-1, 5)
    K, P = len(sp), len(px)
    off = np.zeros(K + 1, np.int32)
    nnz = ctypes.c_longlong()
    vp = ctypes.c_void_p
    _check(lib().rfba_3b_support_masks(vp(px.ctypes.data), P, vp(sp.ctypes.data), K, float(z_factor),
                                       vp(off.ctypes.data), None, 0, ctypes.byref(nnz)))
    idx = np.zeros(max(nnz.value, 1), np.int32)
    _check(lib().rfba_3b_support_masks(vp(px.ctypes.data), P, vp(sp.ctypes.data), K, float(z_factor),
                                       vp(off.ctypes.data), vp(idx.ctypes.data), nnz.value, ctypes.byref(nnz)))
    return off, idx[:nnz.value]


def sym_eigen5(a):
    """Eigenvalues (ascending) and eigenvectors (rows) of a symmetric 5x5 matrix,
    the library's host routine for 3B's model modification."""
    a = np.ascontiguousarray(a, np.float64).reshape(5, 5)
    ev, V = np.zeros(5), np.zeros((5, 5))
    dp = ctypes.POINTER(ctypes.c_double)
    _check(lib().rfba_sym_eigen5(a.ctypes.data_as(dp), ev.ctypes.data_as(dp), V.ctypes.data_as(dp)))
    return ev, V


def det5(a) -> float:
    a = np.ascontiguousarray(a, np.float64).reshape(5, 5)
    return float(lib().rfba_det5(a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))


def _stream_arg(stream, device_tensors: bool):
    """cudaStream_t for a call: the given handle, else torch's current stream
    when the call works on CUDA tensors (so torch work on them stays ordered),
    else the legacy default stream. Handle 0 is the legacy default stream."""
    if stream is not None:
        return ctypes.c_void_p(stream) if stream else None
    if device_tensors:
        import torch
        h = torch.cuda.current_stream().cuda_stream
        return ctypes.c_void_p(h) if h else None
    return None


def version() -> str:
    return lib().rfba_version().decode()
