"""3B's sampled-background Hessian and the model modification's host algebra,
without a GPU.

The oracle's exact expectation of sampled_background_spot_hessian_ffbs
(oracle/gibbs_oracle.py hessian_expectation) is pinned to the reference's own
code compiled on the host (oracle/refshim/ref3b_gibbs_harness.cpp
ref_spot_hessian): bit-close when the chain is forced on in every frame (no
sampling involved), and within the Monte-Carlo error of 20,000 backward
samples per draw otherwise. The library's 5x5 eigen-decomposition and
determinant are checked against numpy, and the fit entry points' argument
checks need no device.
"""
import ctypes

import numpy as np
import pytest

MODEL = dict(variance=1.0, z_factor=1.0, mu_b=3.5, sigma_b=1.0, mu_blur=0.12869, sigma_blur=0.1)
A_MAIN = np.array([[0.16, 0.84, 0.0], [0.495, 0.495, 0.01], [0.0, 0.0, 1.0]])
PI_MAIN = np.array([0.5, 0.5, 0.0])
IU = np.triu_indices(5)  # the reference leaves its entry [4][3] unwritten


def hessian_block(seed, F, n=9, bright=6.0, S=3):
    """One dim blinking spot on a flat background of 2 in an n^3 block, and S
    background samples near the background: (bg [S][F][P], pix [F][P], pixels,
    spot [5])."""
    rng = np.random.default_rng(seed)
    zz, yy, xx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    pixels = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], 1).astype(np.int32)
    c = np.array([n / 2 - 0.3, n / 2 - 0.7, n / 2 - 0.4])
    d = pixels - c
    shape = bright / np.sqrt(2 * np.pi) * np.exp(-(d * d).sum(1) / 2)
    on = rng.random(F) < 0.5
    pix = 2.0 + on[:, None] * shape[None] + rng.normal(0, 1, (F, len(pixels)))
    bg = 2.0 + rng.normal(0, 0.05, (S,) + pix.shape)
    spot = np.array([bright, 1.0, *(c + 0.2)])
    return bg, pix, pixels, spot


def _ref():
    from oracle import gibbs_oracle as G
    if not G.ref_available():
        pytest.skip("reference 3B harness not built (oracle/build_ref.sh)")
    return G


def test_exact_expectation_matches_reference_when_always_on():
    G = _ref()
    bg, pix, pixels, spot = hessian_block(3, 16)
    A, pi = np.eye(3), np.array([1.0, 0.0, 0.0])
    ex = G.hessian_expectation(bg, pix, pixels, spot, A, pi, **MODEL)
    rf = G.ref_spot_hessian(bg, pix, pixels, spot, A, pi, bs_iterations=3, seed=1, **MODEL)
    assert np.max(np.abs(ex[IU] - rf[IU])) <= 1e-11 * np.abs(rf[IU]).max()
    np.testing.assert_allclose(ex, ex.T, rtol=0, atol=0)


@pytest.mark.parametrize("seed", [3, 7])
def test_exact_expectation_matches_reference_sampling(seed):
    G = _ref()
    bg, pix, pixels, spot = hessian_block(seed, 16)
    ex = G.hessian_expectation(bg, pix, pixels, spot, A_MAIN, PI_MAIN, **MODEL)
    rf = G.ref_spot_hessian(bg, pix, pixels, spot, A_MAIN, PI_MAIN, bs_iterations=20000, seed=5, **MODEL)
    assert np.max(np.abs(ex[IU] - rf[IU])) <= 1e-3 * np.abs(ex[IU]).max()


def test_sym_eigen5_and_det5_match_numpy():
    from rfba_gb300 import srrf
    rng = np.random.default_rng(1)
    for trial in range(100):
        B = rng.normal(size=(5, 5)) * 10 ** rng.uniform(-3, 3)
        a = B + B.T
        if trial % 5 == 0:
            a[:, 2] = a[2, :] = 0  # a zero eigenvalue
        ev, V = srrf.sym_eigen5(a)
        w = np.linalg.eigvalsh(a)
        scale = np.abs(w).max()
        np.testing.assert_allclose(ev, w, rtol=0, atol=1e-12 * scale)
        for n in range(5):
            np.testing.assert_allclose(a @ V[n], ev[n] * V[n], rtol=0, atol=1e-11 * scale)
            assert V[n][np.argmax(np.abs(V[n]))] > 0
        np.testing.assert_allclose(V @ V.T, np.eye(5), rtol=0, atol=1e-12)
        d = np.linalg.det(a)
        assert abs(srrf.det5(a) - d) <= 1e-10 * max(abs(d), 1e-6 * scale ** 5)
    assert srrf.det5(np.zeros((5, 5))) == 0.0


def test_fit_entry_points_check_arguments():
    from rfba_gb300 import srrf
    L = srrf.lib()
    m = srrf.ThreeBModel.make(A_MAIN, PI_MAIN)
    prm = srrf.ThreeBFitParams.make([1, 0.5, 0.5, 0.5, 0.5])
    pix = np.zeros((4, 8))
    pixels = np.zeros((8, 3), np.int32)
    sp = np.zeros((2, 5))
    n = ctypes.c_int(1)
    vp = ctypes.c_void_p
    args = (ctypes.byref(m), vp(pix.ctypes.data), vp(pixels.ctypes.data), 4, 8, vp(sp.ctypes.data), ctypes.byref(n))
    assert L.rfba_3b_modify_model(None, *args, 2, ctypes.byref(prm), 0, None) == -1
    assert L.rfba_3b_fit(None, *args, 2, ctypes.byref(prm), 0, 1, 0, srrf.FIT_FN(0), None) == -1
    hess = np.zeros(25)
    dp = ctypes.POINTER(ctypes.c_double)
    assert L.rfba_3b_spot_hessian(None, ctypes.byref(m), vp(pix.ctypes.data), vp(pix.ctypes.data),
                                  vp(pixels.ctypes.data), 1, 4, 8, sp.ctypes.data_as(dp), 10, 0,
                                  hess.ctypes.data_as(dp), srrf.RFBA_HOST_PTRS, None) == -1


def test_free_energy_hessian_oracle_matches_reference():
    """FreeEnergyHessian::hessian given the reference sampler's own draws
    (GibbsSampler2 with every pixel in every mask is the unmasked GibbsSampler):
    the oracle's restatement against the reference's loop compiled here."""
    G = _ref()
    from rfba_gb300 import synth
    pix, pixels, spots = synth.threeb_spots_block(8, 20, (9, 9, 9), 3)
    si = G.spot_intensity(pixels, spots, 1.0)
    P, K = len(pixels), len(spots)
    moff = np.arange(K + 1, dtype=np.int32) * P
    midx = np.tile(np.arange(P, dtype=np.int32), K)
    st, ints = G.ref_run(pix, si, moff, midx, A_MAIN, PI_MAIN, 1.0, 1, 6, 5, want_int=True)
    for spot in range(K):
        want = G.ref_free_energy_hessian_draws(pix, pixels, spots, spot, st, ints, **MODEL)
        got = G.free_energy_hessian_draws(pix, pixels, spots, spot, st, ints, **MODEL)
        assert np.max(np.abs(got[IU] - want[IU])) <= 1e-12 * np.abs(want[IU]).max()


def test_support_masks_are_the_spots_supports():
    """rfba_3b_support_masks: each spot's pixels with Gaussian factor >= 2^-60 (z
    scaled by the z factor), in pixel order."""
    from rfba_gb300 import srrf, synth
    for zf in (1.0, 1.7):
        pix, pixels, spots = synth.threeb_spots_block(12, 4, (29, 21, 17), 5)
        off, idx = srrf.support_masks_3b(pixels, spots, zf)
        d = (pixels[None, :, :] - spots[:, None, 2:]).astype(np.float64)
        d[:, :, 2] /= zf
        e = -(d ** 2).sum(2) / (2 * spots[:, 1:2] ** 2)
        for k in range(len(spots)):
            want = np.nonzero(e[k] >= -41.58883083359672)[0]
            np.testing.assert_array_equal(idx[off[k]:off[k + 1]], want)
        assert 0 < off[1] < len(pixels)  # a support cut by the threshold, not the block
