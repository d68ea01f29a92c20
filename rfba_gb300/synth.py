"""Seeded synthetic light-sheet time series for the SRRF workloads.

The reference publishes no benchmark data (its result TIFFs are missing), so the
workloads run on generated volumes with the statistics of the benchmark
description:
  * point emitters, either uniform over the volume or placed every ~0.5 voxel
    of arc length along random smooth cubic (Bezier) curves (filament-like);
  * 2-state Markov blinking per emitter per volume, P(on->off) = 0.3,
    P(off->on) = 0.1, the first state drawn from the stationary distribution
    (on with probability 0.25);
  * 500 photons per on-emitter through an anisotropic Gaussian PSF integrated
    over each voxel (sigma_xy = 1.2, sigma_z = 2.5 voxels; voxel i spans
    [i, i+1)), plus a background of 100 photons;
  * Poisson shot noise plus Gaussian read noise (sigma 2 counts), rounded and
    clipped to uint16 (or kept as float32);
  * optional per-volume drift: a random walk of the given step sigma per axis,
    applied to the noise-free volume by Catmull-Rom resampling.
Arrays are [t][z][y][x].
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import os

import numpy as np

SIGMA_XY = 1.2
SIGMA_Z = 2.5
PHOTONS = 500.0
BACKGROUND = 100.0
READ_SIGMA = 2.0
P_ON_OFF = 0.3
P_OFF_ON = 0.1


@dataclass
class Scene:
    positions: np.ndarray  # [N, 3] (x, y, z) in voxel units, voxel centres at i + 0.5
    states: np.ndarray     # [T, N] bool, emitter on
    drift: np.ndarray      # [T, 3] (x, y, z) shift applied to volume t


def _erf(x: np.ndarray) -> np.ndarray:
    # numpy has no vectorised erf; math.erf per element over small windows
    return np.vectorize(math.erf, otypes=[np.float64])(x)


def _axis_weights(mu: float, sigma: float, n: int):
    """Fraction of a 1-D Gaussian (centre mu) falling in voxels [i, i+1),
    over a +-4 sigma window clipped to [0, n)."""
    lo = max(int(math.floor(mu - 4 * sigma)), 0)
    hi = min(int(math.ceil(mu + 4 * sigma)) + 1, n)
    if hi <= lo:
        return lo, np.zeros(0)
    edges = np.arange(lo, hi + 1, dtype=np.float64)
    c = _erf((edges - mu) / (sigma * math.sqrt(2.0)))
    return lo, 0.5 * (c[1:] - c[:-1])


def uniform_emitters(rng: np.random.Generator, n: int, shape_xyz, margin: float = 2.0) -> np.ndarray:
    W, H, D = shape_xyz
    lo = np.array([margin, margin, margin])
    hi = np.array([W - margin, H - margin, D - margin], dtype=np.float64)
    return lo + rng.random((n, 3)) * (hi - lo)


def filament_emitters(rng: np.random.Generator, n: int, n_curves: int, shape_xyz, spacing: float = 0.5,
                      margin: float = 3.0) -> np.ndarray:
    """n emitters spread over n_curves random cubic Bezier curves, one every
    `spacing` voxels of arc length from each curve's start."""
    W, H, D = shape_xyz
    dims = np.array([W, H, D], np.float64)
    per = [n // n_curves + (1 if i < n % n_curves else 0) for i in range(n_curves)]
    out = []
    for k in per:
        length_needed = k * spacing
        span = max(length_needed * 0.9, 4.0)
        centre = margin + rng.random(3) * np.maximum(dims - 2 * margin, 1e-3)
        ctrl = centre + (rng.random((4, 3)) - 0.5) * span
        ctrl = np.clip(ctrl, margin, dims - margin)
        s = np.linspace(0.0, 1.0, 4001)[:, None]
        pts = ((1 - s) ** 3) * ctrl[0] + 3 * ((1 - s) ** 2) * s * ctrl[1] + 3 * (1 - s) * s * s * ctrl[2] + (s ** 3) * ctrl[3]
        seg = np.linalg.norm(np.diff(pts, axis=0), axis=1)
        arc = np.concatenate([[0.0], np.cumsum(seg)])
        targets = np.arange(k) * spacing
        targets = np.minimum(targets, arc[-1])  # a short curve stacks its tail
        idx = np.searchsorted(arc, targets).clip(0, len(pts) - 1)
        out.append(pts[idx])
    return np.concatenate(out, axis=0) if out else np.zeros((0, 3))


def blinking(rng: np.random.Generator, n_vol: int, n_em: int) -> np.ndarray:
    states = np.zeros((n_vol, n_em), bool)
    p_stat = P_OFF_ON / (P_OFF_ON + P_ON_OFF)  # 0.25
    s = rng.random(n_em) < p_stat
    for t in range(n_vol):
        states[t] = s
        u = rng.random(n_em)
        s = np.where(s, u >= P_ON_OFF, u < P_OFF_ON)
    return states


def random_walk(rng: np.random.Generator, n_vol: int, sigma: float) -> np.ndarray:
    if sigma <= 0:
        return np.zeros((n_vol, 3))
    steps = rng.normal(0.0, sigma, size=(n_vol, 3))
    steps[0] = 0.0
    return np.cumsum(steps, axis=0)


def render_expected(positions: np.ndarray, on: np.ndarray, shape_zyx) -> np.ndarray:
    """Noise-free photon expectation of one volume (float64, [z][y][x])."""
    D, H, W = shape_zyx
    vol = np.full((D, H, W), BACKGROUND, np.float64)
    for (x, y, z) in positions[on]:
        x0, wx = _axis_weights(x, SIGMA_XY, W)
        y0, wy = _axis_weights(y, SIGMA_XY, H)
        z0, wz = _axis_weights(z, SIGMA_Z, D)
        if wx.size == 0 or wy.size == 0 or wz.size == 0:
            continue
        vol[z0:z0 + wz.size, y0:y0 + wy.size, x0:x0 + wx.size] += PHOTONS * (
            wz[:, None, None] * wy[None, :, None] * wx[None, None, :])
    return vol


def catmull_rom(x):
    """Catmull-Rom kernel, a = 0.5 (the reference's cubic, kernel.cu:128-138)."""
    ax = np.abs(x)
    a = 0.5
    return np.where(ax < 1, ax * ax * (ax * (2 - a) + (a - 3)) + 1,
                    np.where(ax < 2, -a * ax ** 3 + 5 * a * ax ** 2 - 8 * a * ax + 4 * a, 0.0))


def shift_volume(vol: np.ndarray, d) -> np.ndarray:
    """out[z,y,x] = sum_{k,j,i} c(z+dz-k) c(y+dy-j) c(x+dx-i) vol[clamp(k), clamp(j), clamp(i)]:
    the volume sampled at x + d with Catmull-Rom taps and edge clamping."""
    out = vol
    for axis, dd in zip((2, 1, 0), d):  # x, y, z
        n = out.shape[axis]
        pos = np.arange(n) + dd
        base = np.floor(pos).astype(np.int64)
        acc = np.zeros_like(out)
        for k in range(-1, 3):
            idx = np.clip(base + k, 0, n - 1)
            w = catmull_rom(pos - (base + k))
            shp = [1, 1, 1]
            shp[axis] = n
            acc += np.take(out, idx, axis=axis) * w.reshape(shp)
        out = acc
    return out


def make_scene(seed: int, n_vol: int, shape_xyz, n_emitters: int, filament_curves: int = 0,
               drift_sigma: float = 0.0) -> Scene:
    rng = np.random.default_rng(seed)
    if filament_curves > 0:
        pos = filament_emitters(rng, n_emitters, filament_curves, shape_xyz)
    else:
        pos = uniform_emitters(rng, n_emitters, shape_xyz)
    states = blinking(rng, n_vol, len(pos))
    drift = random_walk(rng, n_vol, drift_sigma)
    return Scene(pos, states, drift)


def render(scene: Scene, shape_xyz, seed: int, dtype=np.uint16) -> np.ndarray:
    """Noisy series [T][D][H][W] (uint16 or float32)."""
    W, H, D = shape_xyz
    T = scene.states.shape[0]
    rng = np.random.default_rng(seed + 7919)
    out = np.empty((T, D, H, W), dtype)
    for t in range(T):
        lam = render_expected(scene.positions, scene.states[t], (D, H, W))
        if np.any(scene.drift[t] != 0):
            lam = np.maximum(shift_volume(lam, scene.drift[t]), 0.0)
        noisy = rng.poisson(lam).astype(np.float64) + rng.normal(0.0, READ_SIGMA, size=lam.shape)
        if dtype == np.uint16:
            out[t] = np.clip(np.rint(noisy), 0, 65535).astype(np.uint16)
        else:
            out[t] = noisy.astype(np.float32)
    return out


# The five benchmark workloads (sizes, emitter model, seed = 1234 + index).
WORKLOADS = {
    "small": dict(index=0, n_vol=30, shape=(32, 32, 32), n_emitters=40, curves=0, drift=0.0, dtype=np.uint16),
    "mid": dict(index=1, n_vol=100, shape=(128, 128, 64), n_emitters=600, curves=20, drift=0.0, dtype=np.uint16),
    "batching": dict(index=2, n_vol=50, shape=(160, 160, 120), n_emitters=3000, curves=100, drift=0.0,
                     dtype=np.uint16),
    "diff": dict(index=3, n_vol=60, shape=(64, 64, 64), n_emitters=300, curves=0, drift=0.15, dtype=np.float32),
    "large": dict(index=4, n_vol=200, shape=(256, 256, 128), n_emitters=8000, curves=200, drift=0.1,
                  dtype=np.uint16),
}


def render_volume(scene: Scene, shape_xyz, seed: int, t: int, dtype=np.uint16) -> np.ndarray:
    """Volume t of a series with its own noise stream (seed, t), so volumes can
    be rendered in parallel."""
    W, H, D = shape_xyz
    rng = np.random.default_rng([seed + 7919, t])
    lam = render_expected(scene.positions, scene.states[t], (D, H, W))
    if np.any(scene.drift[t] != 0):
        lam = np.maximum(shift_volume(lam, scene.drift[t]), 0.0)
    noisy = rng.poisson(lam).astype(np.float64) + rng.normal(0.0, READ_SIGMA, size=lam.shape)
    if dtype == np.uint16:
        return np.clip(np.rint(noisy), 0, 65535).astype(np.uint16)
    return noisy.astype(np.float32)


def _render_one(args):
    return render_volume(*args)


def render_parallel(scene: Scene, shape_xyz, seed: int, dtype=np.uint16, workers: int | None = None) -> np.ndarray:
    """render_volume for every volume on a spawn-started process pool."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    W, H, D = shape_xyz
    T = scene.states.shape[0]
    out = np.empty((T, D, H, W), dtype)
    workers = workers or max(1, min(16, (os.cpu_count() or 1)))
    with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        for t, vol in enumerate(ex.map(_render_one, [(scene, shape_xyz, seed, t, dtype) for t in range(T)])):
            out[t] = vol
    return out


def workload(name: str, n_vol: int | None = None, shape=None):
    """(series, scene) for a named workload; n_vol/shape override for reduced
    parity cases."""
    w = dict(WORKLOADS[name])
    if n_vol is not None:
        w["n_vol"] = n_vol
    if shape is not None:
        w["shape"] = tuple(shape)
    seed = 1234 + w["index"]
    scene = make_scene(seed, w["n_vol"], w["shape"], w["n_emitters"], w["curves"], w["drift"])
    return render(scene, w["shape"], seed, w["dtype"]), scene


def threeb_block(seed: int, S: int, F: int, shape=(9, 9, 7), n_spots: int = 6, spot=None, variance=1.0):
    """Seeded stand-in for one 3B block (the localisation step after SRRF): the
    mask's voxels (x fastest), a data series made of a few blinking Gaussian
    spots over a flat background plus Gaussian noise, S background samples (the
    same spots, each switched on or off at random per frame, without the spot
    being fitted) and a starting spot near the first one. Intensities are in
    the normalised units 3B works in (unit noise variance)."""
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


def threeb_spots_block(seed: int, F: int, shape=(12, 12, 9), n_spots: int = 4, variance=1.0, blink=(0.3, 0.1),
                       background: float = 2.0):
    """Seeded stand-in for one 3B block with several spots, for the Gibbs
    sampler: the mask's voxels [P][3] in the reference's (z, y, x) order, a data
    series [F][P] of Gaussian spots blinking as 2-state Markov chains (on -> off
    and off -> on probabilities `blink`) over a flat background plus Gaussian
    noise, and the spots [K][5] (brightness, blur, x, y, z) near the true ones.
    background 0 is data as 3B's preprocessing leaves it (background removed,
    unit noise: load_and_normalize_images, storm_imagery.cc:358-410); 3B's
    model has no background term, so a constant offset pulls the fitted blur
    wide."""
    rng = np.random.default_rng(seed)
    X, Y, Z = shape
    zz, yy, xx = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    pixels = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], 1).astype(np.int32)
    centres = rng.uniform([2, 2, 2], [X - 3, Y - 3, Z - 3], size=(n_spots, 3))
    bright = rng.uniform(30, 80, n_spots)
    blur = rng.uniform(0.9, 1.4, n_spots)
    d = pixels[None, :, :] - centres[:, None, :]
    shapes = bright[:, None] / (blur[:, None] * np.sqrt(2 * np.pi)) * np.exp(-(d * d).sum(2) / (2 * blur[:, None] ** 2))
    on = np.zeros((F, n_spots), bool)
    state = rng.random(n_spots) < blink[1] / (blink[0] + blink[1])
    for f in range(F):
        on[f] = state
        flip = rng.random(n_spots)
        state = np.where(state, flip >= blink[0], flip < blink[1])
    pix = background + on.astype(np.float64) @ shapes + rng.normal(0, np.sqrt(variance), (F, len(pixels)))
    spots = np.column_stack([bright * rng.uniform(0.9, 1.1, n_spots), blur * rng.uniform(0.95, 1.05, n_spots),
                             centres + rng.normal(0, 0.2, (n_spots, 3))])
    return pix, pixels, spots
