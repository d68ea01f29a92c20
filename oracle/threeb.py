"""ctypes front end of the 3B spot-gradient oracle (oracle/threeb_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/ and by the CPU-baseline leg of
bench.py, never by the product package. `spot_neg_prob_diff` restates
SpotNegProbabilityDiffWithSampledBackground::operator() (RFBA Main/
multispot5.cc:616-664) in FP64; `ref_spot_neg_prob_diff` runs the reference's
own headers compiled on the host (oracle/_ref/libref3b_host.so, built by
oracle/build_ref.sh where the reference tree exists).
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "threeb_oracle.cpp"
LIB_PATH = HERE / "_build" / "libthreeb_oracle.so"
REF_LIB_PATH = HERE / "_ref" / "libref3b_host.so"

# the shipped 3B model (RFBA Main/multispot5.cfg:15-16): spot on, off, bleached
A_SHIPPED = np.array([[0.16, 0.84, 0.0], [0.495, 0.495, 0.01], [0.0, 0.0, 1.0]])
PI_SHIPPED = np.array([0.5, 0.5, 0.0])

_lib = None
_ref = None


def build(force: bool = False) -> Path:
    if LIB_PATH.exists() and not force and LIB_PATH.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB_PATH
    LIB_PATH.parent.mkdir(parents=True, exist_ok=True)
    tmp = LIB_PATH.with_suffix(".so.tmp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                    str(SRC), "-o", str(tmp)], check=True)
    tmp.replace(LIB_PATH)
    return LIB_PATH



def _bind(L, name):
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    fn = getattr(L, name)
    d, i = ctypes.c_double, ctypes.c_int
    args = [dp, dp, ip, i, i, i, dp, d, d, dp, dp, d, d, d, d, i, dp]
    if name.startswith("oracle"):
        args.append(dp)
    fn.argtypes = args
    fn.restype = ctypes.c_int
    return fn


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        L.f = _bind(L, "oracle_3b_spot_neg_prob_diff")
        _lib = L
    return _lib


def ref_lib():
    global _ref
    if _ref is None:
        if not REF_LIB_PATH.exists():
            return None
        L = ctypes.CDLL(str(REF_LIB_PATH))
        L.f = _bind(L, "ref3b_spot_neg_prob_diff")
        _ref = L
    return _ref


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def _args(sample_bg, pix, pixels, spot, A, pi):
    sample_bg = np.ascontiguousarray(sample_bg, np.float64)
    pix = np.ascontiguousarray(pix, np.float64)
    pixels = np.ascontiguousarray(pixels, np.int32)
    S, F, P = sample_bg.shape
    assert pix.shape == (F, P) and pixels.shape == (P, 3)
    spot = np.ascontiguousarray(spot, np.float64)
    A = np.ascontiguousarray(A, np.float64).reshape(9)
    pi = np.ascontiguousarray(pi, np.float64)
    return sample_bg, pix, pixels, spot, A, pi, S, F, P


def spot_neg_prob_diff(sample_bg, pix, pixels, spot, z_factor=1.0, variance=1.0, A=A_SHIPPED, pi=PI_SHIPPED,
                       mu_brightness=3.5, sigma_brightness=1.0, mu_blur=0.252148, sigma_blur=0.1, nthreads=8,
                       with_logp=False):
    """The oracle: gradient [5] (and each sample's log probability)."""
    sample_bg, pix, pixels, spot, A, pi, S, F, P = _args(sample_bg, pix, pixels, spot, A, pi)
    out = np.zeros(5)
    logp = np.zeros(S)
    rc = lib().f(_p(sample_bg, ctypes.c_double), _p(pix, ctypes.c_double), _p(pixels, ctypes.c_int), S, F, P,
                 _p(spot, ctypes.c_double), z_factor, variance, _p(A, ctypes.c_double), _p(pi, ctypes.c_double),
                 mu_brightness, sigma_brightness, mu_blur, sigma_blur, nthreads, _p(out, ctypes.c_double),
                 _p(logp, ctypes.c_double))
    assert rc == 0
    return (out, logp) if with_logp else out


def ref_spot_neg_prob_diff(sample_bg, pix, pixels, spot, z_factor=1.0, variance=1.0, A=A_SHIPPED, pi=PI_SHIPPED,
                           mu_brightness=3.5, sigma_brightness=1.0, mu_blur=0.252148, sigma_blur=0.1, nthreads=8):
    """The reference's headers on the host (None when not built)."""
    L = ref_lib()
    if L is None:
        return None
    sample_bg, pix, pixels, spot, A, pi, S, F, P = _args(sample_bg, pix, pixels, spot, A, pi)
    out = np.zeros(5)
    rc = L.f(_p(sample_bg, ctypes.c_double), _p(pix, ctypes.c_double), _p(pixels, ctypes.c_int), S, F, P,
             _p(spot, ctypes.c_double), z_factor, variance, _p(A, ctypes.c_double), _p(pi, ctypes.c_double),
             mu_brightness, sigma_brightness, mu_blur, sigma_blur, nthreads, _p(out, ctypes.c_double))
    assert rc == 0
    return out


def synthetic_block(seed: int, S: int, F: int, shape=(9, 9, 7), n_spots: int = 6, spot=None, variance=1.0):
    """Seeded stand-in for a 3B block: the mask's voxels (x fastest), a data
    series made of a few blinking Gaussian spots over a flat background plus
    Gaussian noise, and S background samples (the same spots, each switched on
    or off at random per frame, without the spot being fitted). Intensities are
    in the normalised units 3B works in (unit noise variance)."""
    rng = np.random.default_rng(seed)
    X, Y, Z = shape
    zz, yy, xx = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    pixels = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], 1).astype(np.int32)
    P = len(pixels)
    centres = rng.uniform([1, 1, 1], [X - 2, Y - 2, Z - 2], size=(n_spots, 3))
    bright = rng.uniform(20, 60, n_spots)
    blur = rng.uniform(0.9, 1.6, n_spots)

    def shape_of(k):
        d = pixels - centres[k]
        return bright[k] / (blur[k] * np.sqrt(2 * np.pi)) * np.exp(-(d * d).sum(1) / (2 * blur[k] ** 2))

    shapes = np.stack([shape_of(k) for k in range(n_spots)])
    on = rng.random((F, n_spots)) < 0.5
    pix = 2.0 + on.astype(np.float64) @ shapes + rng.normal(0, np.sqrt(variance), (F, P))
    samples = np.empty((S, F, P))
    for s in range(S):
        son = rng.random((F, n_spots)) < 0.5
        son[:, 0] = False  # the spot being fitted is removed from the samples
        samples[s] = 2.0 + son.astype(np.float64) @ shapes
    if spot is None:
        spot = np.array([bright[0] * 0.9, blur[0] * 1.1, *(centres[0] + 0.3)])
    return samples, pix, pixels, np.asarray(spot, np.float64)
