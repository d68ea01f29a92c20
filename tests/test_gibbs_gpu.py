"""3B Gibbs sampler and free energy on the GPU (rfba_3b_gibbs_sample /
rfba_3b_gibbs_trace / rfba_3b_free_energy), against the oracle and the
reference's own sampler.

- Deterministic parts: one sweep's masked emission log probabilities and
  forward filter (the quantities every draw is made from), given the states
  the GPU drew, equal the oracle's (oracle/gibbs_oracle.py, pinned to the
  reference's code in tests/test_gibbs_cpu.py); the free energy's host
  arithmetic on the GPU's residuals equals the oracle's bit for bit.
- Sampled parts, by distribution (the GPU uses Philox, the reference MT19937):
  one spot alone is drawn from its forward-backward posterior; a three-spot
  chain's state frequencies match a long run of the reference's GibbsSampler2
  (tests/golden/gibbs_golden.npz); free-energy estimates agree with the
  reference's over seeds.
- Same seed, same draws; the exclude_spot output; argument checks.
"""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "gibbs_golden.npz"


def _model(variance=1.0):
    from oracle import threeb as T3
    from rfba_gb300 import srrf
    return srrf.ThreeBModel.make(T3.A_SHIPPED, T3.PI_SHIPPED, variance=variance, z_factor=1.0,
                                 mu_brightness=float(np.log(40.0)), sigma_brightness=0.5, mu_blur=0.0,
                                 sigma_blur=0.1)


def _block(seed, F, n, shape=(11, 10, 8)):
    from rfba_gb300 import synth
    return synth.threeb_spots_block(seed, F, shape, n)


@pytest.mark.parametrize("seed,F,n", [(1, 40, 4), (2, 100, 6), (3, 7, 2)])
def test_trace_matches_oracle(ctx, seed, F, n):
    from oracle import gibbs_oracle as G
    from oracle import threeb as T3
    from rfba_gb300 import srrf
    pix, pixels, spots = _block(seed, F, n)
    masks = srrf.spot_masks_3b(pixels, spots)
    st, lp, filt = ctx.gibbs_trace_3b(_model(), pix, pixels, spots, masks, seed=seed)
    si = G.spot_intensity(pixels, spots, 1.0)
    lp_o, filt_o, _ = G.trace(pix, si, masks[0], masks[1], T3.A_SHIPPED, T3.PI_SHIPPED, 1.0, st)
    e_lp = float(np.max(np.abs(lp - lp_o) / np.abs(lp_o)))
    e_f = float(np.max(np.abs(filt - filt_o)))
    print(f"[gibbs trace] K={n} F={F}: log p rel {e_lp:.1e}, filter abs {e_f:.1e}")
    assert e_lp < 1e-12
    assert e_f < 1e-10
    assert set(np.unique(st)) <= {0, 1, 2}
    assert (st == 0).any() and (st != 0).any()


def test_one_spot_draws_follow_the_posterior(ctx):
    """A spot with no others: every draw is an independent sample of its
    posterior (forward-backward marginals of the oracle)."""
    from oracle import gibbs_oracle as G
    from oracle import threeb as T3
    from rfba_gb300 import srrf
    pix, pixels, spots = _block(9, 25, 1, (9, 9, 7))
    masks = srrf.spot_masks_3b(pixels, spots)
    n = 6000
    st, _ = ctx.gibbs_sample_3b(_model(), pix, pixels, spots, masks, n_draws=n, seed=77, want_intensities=False)
    si = G.spot_intensity(pixels, spots, 1.0)
    _, _, post = G.trace(pix, si, masks[0], masks[1], T3.A_SHIPPED, T3.PI_SHIPPED, 1.0, st[0])
    for j in range(3):
        freq = (st[:, 0, :] == j).mean(0)
        sd = np.sqrt(post[0, :, j] * (1 - post[0, :, j]) / n) + 1e-3
        assert np.all(np.abs(freq - post[0, :, j]) < 5 * sd), (j, freq, post[0, :, j])


def test_chain_statistics_match_reference_sampler(ctx):
    """Three spots that share pixels: the chain's per-spot, per-frame state
    frequencies against 40,000 draws of the reference's own GibbsSampler2."""
    g = np.load(GOLDEN)
    pix, pixels, spots = g["chain_pix"], g["chain_pixels"], g["chain_spots"]
    ref = g["chain_freq"]
    n = 20000
    st, _ = ctx.gibbs_sample_3b(_model(), pix, pixels, spots, n_draws=n, seed=5, want_intensities=False)
    freq = np.stack([(st == j).mean(0) for j in range(3)], -1)
    d = np.abs(freq - ref)
    print(f"[gibbs chain] max |freq - reference| {d.max():.3f}, per-spot mean {np.abs(freq.mean(1) - ref.mean(1)).max():.4f}")
    assert d.max() < 0.06
    assert np.abs(freq.mean(1) - ref.mean(1)).max() < 0.015


def test_free_energy_arithmetic_and_reference_estimates(ctx):
    from oracle import gibbs_oracle as G
    from rfba_gb300 import srrf
    g = np.load(GOLDEN)
    pix, pixels, spots = g["fe_pix"], g["fe_pixels"], g["fe_spots"]
    mu_b, sg_b, mu_bl, sg_bl = (float(v) for v in g["fe_prior"])
    samples = int(g["fe_samples"])
    from oracle import threeb as T3
    m = srrf.ThreeBModel.make(T3.A_SHIPPED, T3.PI_SHIPPED, variance=1.0, z_factor=1.0, mu_brightness=mu_b,
                              sigma_brightness=sg_b, mu_blur=mu_bl, sigma_blur=sg_bl)
    vals = []
    for seed in range(1, 17):
        v, res = ctx.free_energy_3b(m, pix, pixels, spots, samples=samples, seed=seed)
        # the host arithmetic of compute_with_mask, bit for bit
        assert v == G.free_energy(res, 1.0, len(pixels), pix.shape[0], spots, mu_b, sg_b, mu_bl, sg_bl)
        vals.append(v)
    ref = g["fe_values"]
    se = np.sqrt(np.var(ref, ddof=1) / len(ref) + np.var(vals, ddof=1) / len(vals))
    print(f"[gibbs free energy] GPU {np.mean(vals):.3f} +- {np.std(vals, ddof=1):.3f}, "
          f"reference {np.mean(ref):.3f} +- {np.std(ref, ddof=1):.3f}")
    assert abs(np.mean(vals) - np.mean(ref)) < 5 * se + 1e-9 * abs(np.mean(ref))


def test_same_seed_same_draws_and_exclude_spot(ctx):
    from oracle import gibbs_oracle as G
    pix, pixels, spots = _block(11, 30, 3, (9, 9, 7))
    m = _model()
    a_st, a_int = ctx.gibbs_sample_3b(m, pix, pixels, spots, n_draws=4, sweeps=2, seed=99)
    b_st, b_int = ctx.gibbs_sample_3b(m, pix, pixels, spots, n_draws=4, sweeps=2, seed=99)
    np.testing.assert_array_equal(a_st, b_st)
    np.testing.assert_array_equal(a_int, b_int)
    c_st, _ = ctx.gibbs_sample_3b(m, pix, pixels, spots, n_draws=4, sweeps=2, seed=100, want_intensities=False)
    assert not np.array_equal(a_st, c_st)
    # exclude_spot: the spot's intensity off every pixel of the frames where it is on
    e_st, e_int = ctx.gibbs_sample_3b(m, pix, pixels, spots, n_draws=4, sweeps=2, seed=99, exclude_spot=1)
    np.testing.assert_array_equal(e_st, a_st)
    si = G.spot_intensity(pixels, spots, 1.0)
    want = a_int - (a_st[:, 1, :, None] == 0) * si[1][None, None, :]
    assert np.max(np.abs(e_int - want)) <= 1e-12 * max(1.0, np.abs(want).max())
    # the intensities are the drawn states' spots over their masks
    from rfba_gb300 import srrf
    moff, midx = srrf.spot_masks_3b(pixels, spots)
    d = 3
    exp = np.zeros_like(a_int[d])
    for k in range(3):
        mk = midx[moff[k]:moff[k + 1]]
        rows = np.nonzero(a_st[d, k] == 0)[0]
        exp[np.ix_(rows, mk)] += si[k][mk]
    assert np.max(np.abs(a_int[d] - exp)) < 1e-9


def test_argument_checks(ctx):
    from rfba_gb300 import srrf
    pix, pixels, spots = _block(12, 10, 2, (8, 8, 6))
    m = _model()
    moff, midx = srrf.spot_masks_3b(pixels, spots)
    bad = midx.copy()
    bad[0] = len(pixels)
    with pytest.raises(srrf.RfbaError, match="outside"):
        ctx.gibbs_sample_3b(m, pix, pixels, spots, (moff, bad))
    dup = midx.copy()
    dup[1] = dup[0]
    with pytest.raises(srrf.RfbaError, match="twice"):
        ctx.gibbs_sample_3b(m, pix, pixels, spots, (moff, dup))
    with pytest.raises(srrf.RfbaError):
        ctx.gibbs_sample_3b(m, pix, pixels, spots, exclude_spot=2)
    # and the context still samples afterwards
    st, _ = ctx.gibbs_sample_3b(m, pix, pixels, spots, n_draws=2, want_intensities=False)
    assert st.shape == (2, 2, 10)


def test_pass_replays_its_pieces(ctx):
    """With one spot, a pass is: the spot's Gibbs draws (seed rfba_3b_pass_seed,
    the spot taken off them) then the conjugate-gradient optimisation on them;
    the pass must equal those two calls made separately, bit for bit."""
    from rfba_gb300 import srrf
    pix, pixels, spots = _block(31, 40, 1, (10, 10, 8))
    m = _model()
    lim = np.array([0.5 * 20, 0.5, 0.5, 0.5, 0.5])
    for pass_index in (0, 3):
        got, ev = ctx.optimise_pass_3b(m, pix, pixels, spots, pass_index=pass_index, main_samples=6,
                                       cg_max_iterations=5, limit=lim, seed=12)
        seed = srrf.lib().rfba_3b_pass_seed(12, pass_index, 0)
        _, bg = ctx.gibbs_sample_3b(m, pix, pixels, spots, n_draws=6, seed=seed, exclude_spot=0, want_states=False)
        want, _, ev2 = ctx.optimise_spot_3b(m, bg, pix, pixels, spots[0], lim, 5)
        np.testing.assert_array_equal(got[0], want)
        assert ev == ev2


def test_pass_moves_spots_towards_the_data_and_ejects(ctx):
    from rfba_gb300 import synth
    rng = np.random.default_rng(4)
    pix, pixels, spots = synth.threeb_spots_block(41, 60, (14, 14, 10), 4)
    start = spots.copy()
    start[:, 2:] += rng.normal(0, 0.6, (4, 3))
    m = _model()
    lim = np.array([0.5 * 20, 0.5, 0.5, 0.5, 0.5])
    cur = start.copy()
    for p in range(3):
        cur, ev = ctx.optimise_pass_3b(m, pix, pixels, cur, pass_index=p, main_samples=10, limit=lim, seed=3)
        assert len(cur) == 4 and ev > 0
    # a pass returns the spots in its sweep order (sorted by position), so the
    # error is taken over the best matching of found spots to true ones
    import itertools

    def err(found):
        d = np.linalg.norm(found[:, None, 2:] - spots[None, :, 2:], axis=2)
        return min(np.mean([d[i, j] for i, j in enumerate(perm)]) for perm in itertools.permutations(range(4)))

    err0, err1 = err(start), err(cur)
    print(f"[3B pass] mean position error {err0:.3f} -> {err1:.3f} after 3 passes")
    assert err1 < err0
    # a spot far outside the block has no pixels in its mask and is erased
    far = np.vstack([cur, [[40.0, 1.0, -60.0, 3.0, 3.0]]])
    kept, _ = ctx.optimise_pass_3b(m, pix, pixels, far, pass_index=0, main_samples=4, cg_max_iterations=1, limit=lim,
                                   seed=3)
    assert len(kept) == 4


def test_free_energies_side_by_side_equal_single_runs(ctx):
    """Two models' chains in one launch (a model comparison) give each model the
    value of its own single run with the same seed, bit for bit: a frame's work
    stays on one CTA in the same order whatever the grid."""
    from rfba_gb300 import synth
    pix, pixels, spots = synth.threeb_spots_block(41, 30, (12, 12, 9), 3, background=0.0)
    m = _model()
    a, b = spots, spots[:2]
    pair = ctx.free_energies_3b(m, pix, pixels, [a, b], samples=60, seeds=(5, 9))
    one_a, _ = ctx.free_energy_3b(m, pix, pixels, a, samples=60, seed=5)
    one_b, _ = ctx.free_energy_3b(m, pix, pixels, b, samples=60, seed=9)
    assert pair.tolist() == [one_a, one_b]
    assert ctx.free_energies_3b(m, pix, pixels, [b], samples=60, seeds=(9,)).tolist() == [one_b]
