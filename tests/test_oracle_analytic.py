"""The FP64 oracle on analytic fields, with answers known in closed form (CPU).

- A Gaussian blob: the radiality map peaks at the subvoxel of the blob's
  centre.
- A constant series: every gradient is 0, so every radiality sample is the
  reference's 0/0 and the whole map is NaN.
- A linear ramp: the smoothed gradient is the same vector at every cell away
  from the volume's edge, and Catmull-Rom interpolation reproduces constant and
  linear fields exactly. So the interior radiality is one value everywhere, and
  the interpolated intensity at each subvoxel centre is the ramp at that
  centre, coarse coordinate (X + 1/2) / mag - 1/2. The value is close to 0
  but not exactly 0: the ring's samples are not exactly antipodal.
"""
import numpy as np
import pytest

SH = dict(gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)
D, H, W = 12, 13, 14


def _grid():
    return np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")


@pytest.mark.parametrize("mag", [2, 3])
@pytest.mark.parametrize("method", [0, 1])
def test_blob_peaks_at_its_centre(oracle_mod, mag, method):
    zz, yy, xx = _grid()
    c = (6.0, 6.0, 7.0)  # z, y, x
    blob = 100 * np.exp(-((xx - c[2]) ** 2 + (yy - c[1]) ** 2) / (2 * 1.5 ** 2) - (zz - c[0]) ** 2 / 8.0) + 10
    img = np.stack([blob, 1.1 * blob, 0.9 * blob]).astype(np.float32)
    m = oracle_mod.srrf_region(img, oracle_mod.make_conf(mag=mag, method=method, itc=0, **SH))
    am = np.unravel_index(np.argmax(np.where(np.isfinite(m), m, -np.inf)), m.shape)
    for a in range(3):
        assert abs(am[a] - (c[a] * mag + (mag - 1) / 2)) <= 0.5, (am, c)


def test_constant_series_is_all_nan(oracle_mod):
    img = np.full((3, D, H, W), 7.0, np.float32)
    for kw in (SH, dict(gradient_smooth=0)):
        m = oracle_mod.srrf_region(img, oracle_mod.make_conf(mag=2, method=1, itc=0, **kw))
        assert np.isnan(m).all()


@pytest.mark.parametrize("slope", [(3.0, 2.0, 1.0), (1.0, 0.0, 0.0), (0.0, 0.0, 5.0)])
@pytest.mark.parametrize("mag", [2, 3])
def test_linear_ramp(oracle_mod, slope, mag):
    zz, yy, xx = _grid()
    a, b, c = slope
    ramp = np.broadcast_to((a * xx + b * yy + c * zz + 50)[None], (3, D, H, W)).astype(np.float32).copy()
    lo = (4 * mag,) * 3
    hi = (mag * W - 4 * mag, mag * H - 4 * mag, mag * D - 4 * mag)
    for kw in (SH, dict(gradient_smooth=0)):
        conf = oracle_mod.make_conf(mag=mag, method=1, itc=0, **kw)
        _, rad, inten = oracle_mod.srrf_region(ramp, conf, lo, hi, stacks=True)
        assert np.isfinite(rad).all()
        assert rad.max() - rad.min() <= 1e-12
        assert np.abs(rad).max() <= 1e-5
        Z, Y, X = np.meshgrid(*(np.arange(lo[k], hi[k]) for k in (2, 1, 0)), indexing="ij")
        f = lambda q: (q + 0.5) / mag - 0.5  # noqa: E731
        want = a * f(X) + b * f(Y) + c * f(Z) + 50
        for t in range(3):
            np.testing.assert_allclose(inten[t], want, rtol=0, atol=1e-9)
