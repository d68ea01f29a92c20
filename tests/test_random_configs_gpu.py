"""Seeded random configurations through the CUDA path against the FP64 oracle:
per-axis magnification 1-5, every temporal method and order, integrated lag
times on and off, gradient ranges 0-2 and smoothing on/off, ring radius and
axis count, renormalisation, positivity, intensity weighting, float or uint16
input, odd volume shapes and lengths."""
import numpy as np
import pytest

from tests.parity import assert_parity, tol_for

pytestmark = pytest.mark.gpu


def _random_case(i):
    rng = np.random.default_rng(1000 + i)
    mag = tuple(int(v) for v in rng.integers(1, 6, size=3))
    method = int(rng.integers(0, 4))
    kw = dict(mag=mag, method=method, itc=int(rng.integers(0, 2)), trac_order=int(rng.integers(2, 5)),
              gradient_smooth=int(rng.integers(0, 2)), main_range=int(rng.integers(1, 3)),
              x_range=int(rng.integers(0, 3)), y_range=int(rng.integers(0, 3)), z_range=int(rng.integers(0, 3)),
              axes_in_ring=int(rng.integers(2, 8)), ring_radius=float(rng.choice([0.3, 0.5, 0.7, 1.0])),
              renormalize=int(rng.integers(0, 2)), remove_con=int(rng.integers(0, 2)),
              intensity_w=int(rng.integers(0, 2)))
    # the separable tables need the ring inside one cell of every axis' taps
    kw["ring_radius"] = min(kw["ring_radius"], 0.45 * (1 + min(mag)))
    T = int(rng.integers(1, 14))
    D, H, W = (int(v) for v in rng.integers(5, 13, size=3))
    dtype = np.float32 if rng.random() < 0.5 else np.uint16
    return kw, (T, D, H, W), dtype


@pytest.mark.parametrize("i", range(24))
def test_random_configuration_matches_oracle(ctx, oracle_mod, i):
    from rfba_gb300 import synth
    from rfba_gb300.srrf import Config
    kw, (T, D, H, W), dtype = _random_case(i)
    scene = synth.make_scene(2000 + i, T, (W, H, D), 8)
    x = synth.render(scene, (W, H, D), 2000 + i, dtype)
    got = ctx.forward(Config.make(**kw), np.ascontiguousarray(x))
    ref = oracle_mod.srrf_region(x.astype(np.float32), oracle_mod.make_conf(**kw))
    e = assert_parity(got, ref, tol_for(kw["method"]), f"case {i} {kw} {(T, D, H, W)} {np.dtype(dtype).name}")
    print(f"[random] {i}: rel L-inf {e:.2e} {kw} {(T, D, H, W)}")
