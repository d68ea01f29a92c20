"""3B's sampled-background Hessian on the GPU (rfba_3b_spot_hessian) against
the oracle's exact expectation of sampled_background_spot_hessian_ffbs, which
tests/test_hessian_cpu.py pins to the reference's own code.

With the chain forced on in every frame nothing is sampled and the GPU value
must equal the expectation to rounding; with 3B's shipped transition matrix
it must agree within the Monte-Carlo error of its backward samples.
"""
import numpy as np
import pytest

from test_hessian_cpu import A_MAIN, IU, MODEL, PI_MAIN, hessian_block

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from rfba_gb300 import srrf
    c = srrf.Context(0)
    yield c
    c.close()


def _model(A, pi):
    from rfba_gb300 import srrf
    return srrf.ThreeBModel.make(A, pi, variance=MODEL["variance"], z_factor=MODEL["z_factor"],
                                 mu_brightness=MODEL["mu_b"], sigma_brightness=MODEL["sigma_b"],
                                 mu_blur=MODEL["mu_blur"], sigma_blur=MODEL["sigma_blur"])


def test_always_on_equals_expectation(ctx):
    from oracle import gibbs_oracle as G
    bg, pix, pixels, spot = hessian_block(3, 16)
    A, pi = np.eye(3), np.array([1.0, 0.0, 0.0])
    got = ctx.spot_hessian_3b(_model(A, pi), bg, pix, pixels, spot, bs_iterations=7, seed=1)
    want = G.hessian_expectation(bg, pix, pixels, spot, A, pi, **MODEL)
    err = np.max(np.abs(got - want)) / np.abs(want).max()
    print(f"[3B Hessian] always on: rel L-inf {err:.1e}")
    assert err <= 1e-10
    np.testing.assert_array_equal(got, got.T)


@pytest.mark.parametrize("seed,F,n", [(3, 16, 9), (7, 40, 7), (11, 300, 5)])
def test_sampled_matches_expectation(ctx, seed, F, n):
    from oracle import gibbs_oracle as G
    bg, pix, pixels, spot = hessian_block(seed, F, n=n)
    got = ctx.spot_hessian_3b(_model(A_MAIN, PI_MAIN), bg, pix, pixels, spot, bs_iterations=20000, seed=seed)
    want = G.hessian_expectation(bg, pix, pixels, spot, A_MAIN, PI_MAIN, **MODEL)
    err = np.max(np.abs(got[IU] - want[IU])) / np.abs(want[IU]).max()
    print(f"[3B Hessian] F={F} P={n ** 3}: rel L-inf vs expectation {err:.1e}")
    assert err <= 1e-3


def test_device_pointers_and_seeds(ctx):
    import torch
    bg, pix, pixels, spot = hessian_block(5, 24)
    m = _model(A_MAIN, PI_MAIN)
    a = ctx.spot_hessian_3b(m, bg, pix, pixels, spot, bs_iterations=500, seed=9)
    b = ctx.spot_hessian_3b(m, torch.from_numpy(bg).cuda(), torch.from_numpy(pix).cuda(),
                            torch.from_numpy(pixels).cuda(), spot, bs_iterations=500, seed=9)
    np.testing.assert_array_equal(a, b)
    c = ctx.spot_hessian_3b(m, bg, pix, pixels, spot, bs_iterations=500, seed=10)
    assert not np.array_equal(a, c)


def test_argument_checks(ctx):
    from rfba_gb300 import srrf
    bg, pix, pixels, spot = hessian_block(5, 8)
    m = _model(A_MAIN, PI_MAIN)
    with pytest.raises(srrf.RfbaError):
        ctx.spot_hessian_3b(m, bg, pix, pixels, spot, bs_iterations=0)
    big = np.zeros((1, 2049, 8))
    with pytest.raises(srrf.RfbaError):
        ctx.spot_hessian_3b(m, big, np.zeros((2049, 8)), pixels[:8], spot, bs_iterations=1)


def test_free_energy_hessian_replays_its_draws(ctx):
    """rfba_3b_free_energy_hessian against the oracle given the same draws: the
    unmasked sampler is rfba_3b_gibbs_sample with each spot's support as its
    mask (rfba_3b_support_masks) and the same seed, so the GPU's draws are
    replayed exactly."""
    from oracle import gibbs_oracle as G
    from rfba_gb300 import srrf, synth
    pix, pixels, spots = synth.threeb_spots_block(8, 20, (9, 9, 9), 3)
    m = _model(A_MAIN, PI_MAIN)
    P, K = len(pixels), len(spots)
    masks = srrf.support_masks_3b(pixels, spots, 1.0)
    st, ints = ctx.gibbs_sample_3b(m, pix, pixels, spots, masks, sweeps=1, n_draws=12, seed=21)
    for spot in range(K):
        got = ctx.free_energy_hessian_3b(m, pix, pixels, spots, spot, samples=12, seed=21)
        want = G.free_energy_hessian_draws(pix, pixels, spots, spot, st, ints, **MODEL)
        err = np.max(np.abs(got - want)) / np.abs(want).max()
        print(f"[3B free-energy Hessian] spot {spot}: rel L-inf {err:.1e}, on in {(st[:, spot] == 0).sum()} frames")
        assert err <= 1e-10
