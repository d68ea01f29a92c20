"""3B Gibbs sampler and free energy: the oracle against the reference's own code.

oracle/gibbs_oracle.py restates the deterministic parts of GibbsSampler2
(RFBA Main/sampled_multispot.h:658-690) and of NegativeFreeEnergy::
compute_with_mask (multispot5.cc:335-405). Here it is pinned to the reference
compiled on the host (oracle/_ref/libref3b_gibbs_host.so, where the reference
tree exists): spot intensities, the masked emission log probabilities, the
forward filter and posterior of a sweep with given drawn states, and the free
energy's arithmetic on the reference sampler's own residuals. The library's
host-side mask builder (rfba_3b_spot_masks, no GPU needed) is checked against
the oracle's. The reference sampler's draws are also checked against the
posterior they should follow (the reference's own distribution, which the GPU
sampler must match).
"""
import ctypes

import numpy as np
import pytest

from oracle import gibbs_oracle as G
from oracle import threeb as T3

needs_ref = pytest.mark.skipif(not G.ref_available(), reason="reference tree not present (harness not built)")


def _block(seed=5, F=40, n=3, shape=(11, 10, 8)):
    from rfba_gb300 import synth
    pix, pixels, spots = synth.threeb_spots_block(seed, F, shape, n)
    moff, midx = G.spot_masks(pixels, spots)
    return pix, pixels, spots, moff, midx


def test_library_masks_equal_oracle(built_lib):
    from rfba_gb300 import srrf
    pix, pixels, spots, moff, midx = _block()
    L = srrf.lib()
    K, P = len(spots), len(pixels)
    off = np.zeros(K + 1, np.int32)
    nnz = ctypes.c_longlong()
    px = np.ascontiguousarray(pixels, np.int32)
    sp = np.ascontiguousarray(spots, np.float64)
    assert L.rfba_3b_spot_masks(px.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), P,
                                sp.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), K,
                                off.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), None, 0, ctypes.byref(nnz)) == 0
    idx = np.zeros(nnz.value, np.int32)
    assert L.rfba_3b_spot_masks(px.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), P,
                                sp.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), K,
                                off.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), nnz.value, ctypes.byref(nnz)) == 0
    np.testing.assert_array_equal(off, moff)
    np.testing.assert_array_equal(idx, midx)
    assert 0 < moff[1] < P  # the ball is cut by the block edge
    # unsorted pixels are refused
    bad = np.ascontiguousarray(px[::-1])
    assert L.rfba_3b_spot_masks(bad.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), P,
                                sp.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), K,
                                off.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), None, 0, ctypes.byref(nnz)) == -1


def test_masks_of_wide_spots_scan_the_pixels(built_lib):
    """A ball with more offsets than the block has pixels is found by testing
    the pixels (in their (z, y, x) order, which is the ball's order): the same
    masks as enumerating the ball, on an irregular pixel set; a blur that is not
    finite or enormous still returns at once."""
    from oracle import gibbs_oracle as G
    from rfba_gb300 import srrf
    rng = np.random.default_rng(3)
    n = 17
    zz, yy, xx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    pixels = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], 1).astype(np.int32)
    pixels = pixels[rng.random(len(pixels)) < 0.8]
    spots = np.array([[30, 0.3, 8.2, 7.6, 8.9], [30, 1.1, 3.4, 12.5, 5.5], [30, 2.5, 8, 8, 8],
                      [30, 4.0, 2.2, 3.3, 14.6], [30, 0.8, -3.2, 20.4, 8.0]])
    off, idx = srrf.spot_masks_3b(pixels, spots)
    off2, idx2 = G.spot_masks(pixels, spots)
    np.testing.assert_array_equal(off, off2)
    np.testing.assert_array_equal(idx, idx2)
    off, _ = srrf.spot_masks_3b(pixels, np.array([[30, 1e6, 8, 8, 8], [30, np.nan, 8, 8, 8]]))
    assert off.tolist() == [0, len(pixels), len(pixels)]


@needs_ref
def test_spot_intensity_matches_reference():
    pix, pixels, spots, moff, midx = _block()
    for zf in (1.0, 1.7):
        a = G.spot_intensity(pixels, spots, zf)
        b = G.ref_spot_intensity(pixels, spots, zf)
        assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)) < 1e-14


@needs_ref
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_trace_matches_reference(seed):
    pix, pixels, spots, moff, midx = _block(seed, F=30, n=4)
    si = G.spot_intensity(pixels, spots, 1.0)
    rng = np.random.default_rng(seed)
    states = rng.integers(0, 3, size=(len(spots), pix.shape[0])).astype(np.uint8)
    for A, pi in ((T3.A_SHIPPED, T3.PI_SHIPPED), (np.full((3, 3), 1 / 3), np.full(3, 1 / 3))):
        a = G.trace(pix, si, moff, midx, A, pi, 1.0, states)
        b = G.ref_trace(pix, si, moff, midx, A, pi, 1.0, states)
        assert np.max(np.abs(a[0] - b[0]) / np.abs(b[0])) < 1e-13
        assert np.max(np.abs(a[1] - b[1])) < 1e-12
        assert np.max(np.abs(a[2] - b[2])) < 1e-12


@needs_ref
def test_free_energy_arithmetic_matches_reference_bit_for_bit():
    pix, pixels, spots, moff, midx = _block(7, F=20, n=2, shape=(9, 9, 7))
    for samples in (12, 40):
        v, res = G.ref_free_energy(pix, pixels, spots, moff, midx, T3.A_SHIPPED, T3.PI_SHIPPED, 1.0, 1.0,
                                   np.log(40), 0.5, 0.0, 0.1, samples, 1, 11)
        w = G.free_energy(res, 1.0, len(pixels), pix.shape[0], spots, np.log(40), 0.5, 0.0, 0.1)
        assert w == v


@needs_ref
def test_reference_sampler_follows_the_posterior():
    """One spot with no others: every draw is an independent sample of the
    posterior, so the per-frame state frequencies over many draws must match
    the forward-backward marginals."""
    pix, pixels, spots, moff, midx = _block(9, F=25, n=1, shape=(9, 9, 7))
    si = G.spot_intensity(pixels, spots, 1.0)
    n = 4000
    st, _ = G.ref_run(pix, si, moff, midx, T3.A_SHIPPED, T3.PI_SHIPPED, 1.0, 1, n, 3)
    _, _, post = G.trace(pix, si, moff, midx, T3.A_SHIPPED, T3.PI_SHIPPED, 1.0, st[0])
    for j in range(3):
        freq = (st[:, 0, :] == j).mean(0)
        sd = np.sqrt(post[0, :, j] * (1 - post[0, :, j]) / n) + 1e-3
        assert np.all(np.abs(freq - post[0, :, j]) < 5 * sd), (j, freq, post[0, :, j])


@needs_ref
@pytest.mark.parametrize("seed,sweeps", [(3, 1), (17, 2)])
def test_port_draws_are_the_references_draws(seed, sweeps):
    """The C++ port (the bench's CPU baseline) with the reference's MT19937
    stream: the same states and intensities as the reference's GibbsSampler2,
    bit for bit."""
    pix, pixels, spots, moff, midx = _block(seed, F=30, n=4)
    si = G.spot_intensity(pixels, spots, 1.0)
    a = G.port_run(pix, si, moff, midx, T3.A_SHIPPED, T3.PI_SHIPPED, 1.0, sweeps, 5, seed, want_int=True)
    b = G.ref_run(pix, si, moff, midx, T3.A_SHIPPED, T3.PI_SHIPPED, 1.0, sweeps, 5, seed, want_int=True)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_port_pass_runs_and_keeps_spots():
    from rfba_gb300 import synth
    pix, pixels, spots = synth.threeb_spots_block(41, 30, (12, 12, 9), 3)
    lim = np.array([10.0, 0.5, 0.5, 0.5, 0.5])
    out, (tg, tc) = G.port_pass(pix, pixels, spots, 0, 4, 1, 3, lim, 2.3, T3.A_SHIPPED, T3.PI_SHIPPED, 1.0, 1.0,
                                np.log(40.0), 0.5, 0.0, 0.1, 5, nthreads=4)
    assert out.shape == (3, 5) and tg > 0 and tc > 0
    assert np.all(np.isfinite(out)) and np.all(out[:, 0] > 0)
