"""3B spot gradient on the GPU (rfba_3b_spot_gradient) against the FP64 oracle
(pinned to the reference's headers in tests/test_threeb_cpu.py). Both compute
in FP64; the GPU sums each frame's voxels in a tree instead of in sequence and
runs the forward algorithm on probabilities with a power-of-two exponent per
state instead of in log space, so the gradient agrees to 1e-9 of its largest
component and every sample's log probability to 1e-12 (relative)."""
import numpy as np
import pytest

from oracle import threeb as T

pytestmark = pytest.mark.gpu

CASES = [  # (seed, S, F, mask shape, z factor, variance)
    (0, 4, 12, (7, 6, 5), 1.3, 1.2),
    (1, 10, 30, (9, 9, 7), 1.0, 1.0),
    (2, 3, 1, (5, 5, 5), 2.0, 0.7),
    (3, 1, 25, (11, 8, 6), 1.0, 1.5),
    (4, 10, 50, (29, 29, 29), 1.5, 1.0),
]


def _model(zf, var):
    from rfba_gb300.srrf import ThreeBModel
    return ThreeBModel.make(T.A_SHIPPED, T.PI_SHIPPED, variance=var, z_factor=zf)


def _compare(got, lp, want, lpw):
    scale = np.max(np.abs(want))
    assert np.max(np.abs(got - want)) <= 1e-9 * scale, (got, want)
    assert np.max(np.abs(lp - lpw) / np.abs(lpw)) <= 1e-12, (lp, lpw)


@pytest.mark.parametrize("case", CASES, ids=[f"seed{c[0]}" for c in CASES])
def test_spot_gradient_matches_oracle(ctx, case):
    seed, S, F, shape, zf, var = case
    bg, pix, px, spot = T.synthetic_block(seed, S, F, shape, variance=var)
    want, lpw = T.spot_neg_prob_diff(bg, pix, px, spot, z_factor=zf, variance=var, with_logp=True)
    got, lp = ctx.spot_gradient_3b(_model(zf, var), bg, pix, px, spot)
    _compare(got, lp, want, lpw)


@pytest.mark.parametrize("case", CASES, ids=[f"seed{c[0]}" for c in CASES])
def test_double_float_gradient_matches_oracle(ctx, case):
    """The optimisers' gradient-only path: the per-frame sums in double-float
    arithmetic on residuals staged once, within the same 1e-9 of the largest
    component as the FP64 path."""
    seed, S, F, shape, zf, var = case
    bg, pix, px, spot = T.synthetic_block(seed, S, F, shape, variance=var)
    want = T.spot_neg_prob_diff(bg, pix, px, spot, z_factor=zf, variance=var)
    got, none = ctx.spot_gradient_3b(_model(zf, var), bg, pix, px, spot, want_log_prob=False)
    fp64, _ = ctx.spot_gradient_3b(_model(zf, var), bg, pix, px, spot)
    assert none is None
    scale = np.max(np.abs(want))
    err = np.max(np.abs(got - want)) / scale
    print(f"[3B gradient] double-float path: rel L-inf {err:.1e} (FP64 path "
          f"{np.max(np.abs(fp64 - want)) / scale:.1e})")
    assert err <= 1e-9


def test_device_pointers_and_repeated_calls(ctx):
    import torch
    bg, pix, px, spot = T.synthetic_block(7, 6, 20, (9, 8, 7))
    m = _model(1.2, 1.0)
    d = [torch.from_numpy(a).cuda() for a in (bg, pix, px)]
    for k in range(3):  # the optimiser's pattern: data stay, the spot moves
        sp = spot + 0.1 * k
        want, lpw = T.spot_neg_prob_diff(bg, pix, px, sp, z_factor=1.2, with_logp=True)
        got, lp = ctx.spot_gradient_3b(m, *d, sp)
        _compare(got, lp, want, lpw)


def test_non_positive_brightness_or_blur_gives_nan(ctx):
    bg, pix, px, spot = T.synthetic_block(8, 2, 4, (5, 5, 5))
    for i in (0, 1):
        s = spot.copy()
        s[i] = -1.0
        got, _ = ctx.spot_gradient_3b(_model(1.0, 1.0), bg, pix, px, s)
        assert np.isnan(got).all()


def test_long_bleach_then_bright_frames(ctx):
    """1400 dark frames (the absorbing bleached state ends up holding all the
    mass, more than e^709 above the others) followed by frames with a very
    bright spot, which the bleached state cannot emit: probabilities without
    their own exponents underflow to 0 here, the log-space reference does not."""
    bg, pix, px, spot = T.synthetic_block(7, 3, 1400)
    rng = np.random.default_rng(1)
    pix = bg.mean(0) + rng.normal(0, 1, pix.shape)
    d = px - spot[2:]
    pix[-5:] += spot[0] * 3 / (spot[1] * np.sqrt(2 * np.pi)) * np.exp(-(d * d).sum(1) / (2 * spot[1] ** 2))
    want, lpw = T.spot_neg_prob_diff(bg, pix, px, spot, with_logp=True)
    got, lp = ctx.spot_gradient_3b(_model(1.0, 1.0), bg, pix, px, spot)
    assert np.isfinite(want).all() and np.isfinite(lpw).all()
    _compare(got, lp, want, lpw)


def test_dense_transition_matrix(ctx):
    """A model where every state can reach every other, with a non-zero start
    probability for each."""
    from rfba_gb300.srrf import ThreeBModel
    A = np.array([[0.7, 0.2, 0.1], [0.3, 0.6, 0.1], [0.05, 0.05, 0.9]])
    pi = np.array([0.2, 0.5, 0.3])
    bg, pix, px, spot = T.synthetic_block(11, 5, 40, (8, 8, 6))
    want, lpw = T.spot_neg_prob_diff(bg, pix, px, spot, A=A, pi=pi, with_logp=True)
    got, lp = ctx.spot_gradient_3b(ThreeBModel.make(A, pi), bg, pix, px, spot)
    _compare(got, lp, want, lpw)


def test_rejects_probabilities_outside_unit_interval(ctx):
    from rfba_gb300.srrf import RfbaError, ThreeBModel
    bg, pix, px, spot = T.synthetic_block(8, 2, 4, (5, 5, 5))
    A = T.A_SHIPPED.copy()
    A[0, 0] = -0.1
    with pytest.raises(RfbaError, match="probabilities"):
        ctx.spot_gradient_3b(ThreeBModel.make(A, T.PI_SHIPPED), bg, pix, px, spot)


def _limit(mu=3.5, sigma=1.0, max_motion=0.5):
    return max_motion * np.array([np.sqrt((np.exp(sigma ** 2) - 1) * np.exp(2 * mu + sigma ** 2)), 1, 1, 1, 1])


@pytest.mark.parametrize("seed,S,F,shape,iters", [(0, 4, 12, (7, 6, 5), 5), (1, 6, 30, (9, 9, 7), 20)])
def test_optimise_spot_matches_host_optimiser(ctx, seed, S, F, shape, iters):
    """rfba_3b_optimise_spot (the optimiser on the GPU gradient, data staged
    once, its sums in double-float) against the same optimiser on the host
    driven by the oracle's gradient (itself pinned bit for bit to the
    reference's optimiser in tests/test_threeb_cpu.py). The gradients agree to
    ~1e-14 of their largest component; along the brightness, whose curvature is
    small next to that component, twenty line searches carry the difference to
    about 1e-6 of the brightness, so the spots agree to 1e-5 relative and the
    line-search count is the same."""
    from rfba_gb300 import srrf
    bg, pix, px, spot = T.synthetic_block(seed, S, F, shape)
    want, it_w, ev_w = srrf.cg_only_run(lambda x: T.spot_neg_prob_diff(bg, pix, px, x), spot, _limit(), iters)
    got, it, ev = ctx.optimise_spot_3b(_model(1.0, 1.0), bg, pix, px, spot, _limit(), iters)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-8)
    assert it == it_w
    import torch
    d = [torch.from_numpy(a).cuda() for a in (bg, pix, px)]
    got2, it2, ev2 = ctx.optimise_spot_3b(_model(1.0, 1.0), *d, spot, _limit(), iters)
    np.testing.assert_array_equal(got2, got)  # the same device arithmetic either way
    assert (it2, ev2) == (it, ev)


def test_golden_gradient_and_optimiser(ctx):
    """The GPU against the reference's own results committed in
    tests/golden/threeb_golden.npz (make_golden_3b.py): gradient to 1e-9 of
    its largest component, optimised spot to 1e-6."""
    from pathlib import Path
    z = np.load(Path(__file__).resolve().parent / "golden" / "threeb_golden.npz")
    for i in range(int(z["ncases"])):
        c = {k.split("_", 1)[1]: z[k] for k in z.files if k.startswith(f"c{i}_")}
        g, _ = ctx.spot_gradient_3b(_model(1.0, 1.0), c["bg"], c["pix"], c["px"], c["spot"])
        assert np.max(np.abs(g - c["grad"])) <= 1e-9 * np.max(np.abs(c["grad"])), (g, c["grad"])
        x, it, ev = ctx.optimise_spot_3b(_model(1.0, 1.0), c["bg"], c["pix"], c["px"], c["spot"], _limit(),
                                         int(c["iters"]))
        np.testing.assert_allclose(x, c["opt"], rtol=1e-6, atol=1e-8)
