"""Comparison helpers for the parity tests.

Relative L-infinity error of a map against the FP64 oracle:
    max |gpu - oracle| / max |oracle|   over voxels finite in both,
with the NaN masks required to be identical. Tolerances (from the
benchmark statement): 1e-5 for the temporal mean (and TRM / TRPPM maps),
1e-4 for TRAC maps.
"""
import numpy as np

TOL_MEAN = 1e-5
TOL_TRAC = 1e-4


def tol_for(method: int) -> float:
    return TOL_TRAC if method == 3 else TOL_MEAN


def rel_linf(got: np.ndarray, ref: np.ndarray) -> float:
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    fin = np.isfinite(ref) & np.isfinite(got)
    if not fin.any():
        return 0.0
    scale = np.max(np.abs(ref[fin]))
    if scale == 0:
        return float(np.max(np.abs(got[fin])))
    return float(np.max(np.abs(got[fin] - ref[fin])) / scale)


def assert_parity(got, ref, tol, what=""):
    got = np.asarray(got)
    ref = np.asarray(ref)
    assert got.shape == ref.shape, f"{what}: shape {got.shape} != {ref.shape}"
    nan_g, nan_r = np.isnan(got), np.isnan(ref)
    assert np.array_equal(nan_g, nan_r), (
        f"{what}: NaN masks differ ({int(nan_g.sum())} vs {int(nan_r.sum())}, "
        f"{int((nan_g != nan_r).sum())} mismatches)")
    inf_g, inf_r = np.isinf(got), np.isinf(ref)
    assert np.array_equal(inf_g, inf_r), f"{what}: Inf masks differ"
    e = rel_linf(got, ref)
    assert e <= tol, f"{what}: relative L-inf error {e:.3e} > {tol:.0e}"
    return e
