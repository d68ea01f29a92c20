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


# the CPU port of the Gibbs sampler and of a main-loop pass, in the same library
GIBBS_SRC = HERE / "gibbs_port.cpp"
CG_HDR = HERE.parent / "rfba_gb300" / "csrc" / "cg_only.h"


def build(force: bool = False) -> Path:
    newest = max(p.stat().st_mtime for p in (SRC, GIBBS_SRC, CG_HDR))
    if LIB_PATH.exists() and not force and LIB_PATH.stat().st_mtime >= newest:
        return LIB_PATH
    LIB_PATH.parent.mkdir(parents=True, exist_ok=True)
    tmp = LIB_PATH.with_suffix(".so.tmp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-Wno-psabi",
                    str(SRC), str(GIBBS_SRC), "-o", str(tmp)], check=True)
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


def ref_cg_optimise(sample_bg, pix, pixels, spot, limit, max_iterations, z_factor=1.0, variance=1.0, A=A_SHIPPED,
                    pi=PI_SHIPPED, mu_brightness=3.5, sigma_brightness=1.0, mu_blur=0.252148, sigma_blur=0.1,
                    nthreads=8):
    """The reference's ConjugateGradientOnly<5> with the reference's spot
    gradient (multispot5.cc:1624-1636), compiled on the host: (final spot,
    line searches), or None when not built."""
    L = ref_lib()
    if L is None:
        return None
    if not hasattr(L, "cg"):
        dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        d, i = ctypes.c_double, ctypes.c_int
        L.cg = L.ref3b_cg_optimise
        L.cg.argtypes = [dp, dp, ip, i, i, i, dp, d, d, dp, dp, d, d, d, d, i, dp, i, dp, ip]
        L.cg.restype = ctypes.c_int
    sample_bg, pix, pixels, spot, A, pi, S, F, P = _args(sample_bg, pix, pixels, spot, A, pi)
    limit = np.ascontiguousarray(limit, np.float64)
    out = np.zeros(5)
    it = ctypes.c_int()
    rc = L.cg(_p(sample_bg, ctypes.c_double), _p(pix, ctypes.c_double), _p(pixels, ctypes.c_int), S, F, P,
              _p(spot, ctypes.c_double), z_factor, variance, _p(A, ctypes.c_double), _p(pi, ctypes.c_double),
              mu_brightness, sigma_brightness, mu_blur, sigma_blur, nthreads, _p(limit, ctypes.c_double),
              int(max_iterations), _p(out, ctypes.c_double), ctypes.byref(it))
    assert rc == 0
    return out, it.value


def synthetic_block(seed: int, S: int, F: int, shape=(9, 9, 7), n_spots: int = 6, spot=None, variance=1.0):
    """The seeded 3B block of rfba_gb300.synth.threeb_block (mask voxels, data,
    background samples, a starting spot)."""
    from rfba_gb300 import synth
    return synth.threeb_block(seed, S, F, shape, n_spots, spot, variance)
