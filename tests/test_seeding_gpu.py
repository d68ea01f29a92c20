"""SRRF-guided spot seeding on the GPU (inverse CDF, counter-based RNG)
against the reference's rejection sampler (restated in the oracle): the
subvoxel picked follows the same distribution (chi-square on counts, and a
two-sample test against the oracle's draws), zero-weight subvoxels are never
picked, the position inside a subvoxel is uniform, an all-zero map is uniform,
seeds reproduce, and a voxel outside the map is an error."""
import numpy as np
import pytest
from scipy import stats

pytestmark = pytest.mark.gpu


def _setup(mag=2):
    rng = np.random.default_rng(5)
    D, H, W = 6, 7, 8
    m = rng.gamma(2.0, 1.0, size=(D * mag, H * mag, W * mag)).astype(np.float32)
    m[m < 0.8] = 0.0
    m.flat[rng.choice(m.size, 20, replace=False)] = np.nan
    m.flat[rng.choice(m.size, 20, replace=False)] = -3.0
    vox = np.array([(x, y, z) for z in range(1, 4) for y in range(2, 5) for x in range(3, 7)], np.int32)
    return m, vox


def _counts(xyz, vox, mag):
    sub = np.floor(xyz * mag + 0.5).astype(np.int64)
    vs = np.array([(j1, j2, j3) for j1 in range(mag) for j2 in range(mag) for j3 in range(mag)])
    pix = (vox[:, None, :].astype(np.int64) * mag + vs[None]).reshape(-1, 3)
    index = {tuple(p): i for i, p in enumerate(pix)}
    c = np.zeros(len(pix), np.int64)
    for s in map(tuple, sub):
        c[index[s]] += 1
    return c, pix


def test_distribution_matches_reference_sampler(ctx, oracle_mod):
    m, vox = _setup()
    mag, n = 2, 300000
    xyz = ctx.seed_spots(m, vox, mag, n, seed=11)
    assert xyz.shape == (n, 3) and np.all(np.isfinite(xyz))
    c, pix = _counts(xyz, vox, mag)
    w = m[pix[:, 2], pix[:, 1], pix[:, 0]].astype(np.float64)
    w = np.where(np.isnan(w) | (w < 0), 0.0, w)
    assert np.all(c[w == 0] == 0)
    nz = w > 0
    exp = n * w[nz] / w[nz].sum()
    chi = stats.chisquare(c[nz], exp)
    print(f"[seeding] chi-square vs weights: p = {chi.pvalue:.3g}")
    assert chi.pvalue > 1e-4
    ref = oracle_mod.seed_spots_rejection(m, vox, mag, 100000, np.random.default_rng(3))
    cr, _ = _counts(ref, vox, mag)
    tab = np.vstack([c[nz], cr[nz]])
    p2 = stats.chi2_contingency(tab)[1]
    print(f"[seeding] two-sample vs reference rejection sampler: p = {p2:.3g}")
    assert p2 > 1e-4
    frac = xyz * mag + 0.5 - np.floor(xyz * mag + 0.5)
    for a in range(3):
        assert stats.kstest(frac[:, a], "uniform").pvalue > 1e-4


def test_zero_map_uniform_and_seeds(ctx):
    import torch
    m, vox = _setup()
    z = np.zeros_like(m)
    xyz = ctx.seed_spots(z, vox, 2, 96000, seed=1)
    c, _ = _counts(xyz, vox, 2)
    assert stats.chisquare(c).pvalue > 1e-4
    a = ctx.seed_spots(m, vox, 2, 1000, seed=7)
    b = ctx.seed_spots(torch.from_numpy(m).cuda(), vox, 2, 1000, seed=7).cpu().numpy()
    assert np.array_equal(a, b)
    assert not np.array_equal(a, ctx.seed_spots(m, vox, 2, 1000, seed=8))


def test_voxel_outside_map_is_an_error(ctx):
    from rfba_gb300.srrf import RfbaError
    m, vox = _setup()
    bad = np.vstack([vox, [[100, 0, 0]]]).astype(np.int32)
    with pytest.raises(RfbaError):
        ctx.seed_spots(m, bad, 2, 10, seed=0)
