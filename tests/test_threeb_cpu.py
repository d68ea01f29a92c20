"""3B spot-gradient oracle (oracle/threeb_oracle.cpp), CPU only: pinned bit for
bit to the reference's own headers compiled on the host (where the reference
tree exists), and checked against central differences of the log probability
it reports."""
import numpy as np
import pytest

from oracle import threeb as T

CASES = [  # (seed, S, F, mask shape, nthreads, z factor, variance)
    (0, 4, 12, (7, 6, 5), 8, 1.3, 1.2),
    (1, 10, 30, (9, 9, 7), 3, 1.0, 1.0),
    (2, 3, 1, (5, 5, 5), 8, 2.0, 0.7),
    (3, 1, 25, (11, 8, 6), 8, 1.0, 1.5),
    (4, 7, 9, (6, 7, 8), 2, 0.8, 1.0),
]


@pytest.mark.parametrize("case", CASES, ids=[f"seed{c[0]}" for c in CASES])
def test_oracle_reproduces_reference_bits(case):
    if T.ref_lib() is None:
        pytest.skip("oracle/_ref/libref3b_host.so not built (reference sources absent)")
    seed, S, F, shape, nt, zf, var = case
    bg, pix, px, spot = T.synthetic_block(seed, S, F, shape, variance=var)
    a = T.spot_neg_prob_diff(bg, pix, px, spot, z_factor=zf, variance=var, nthreads=nt)
    b = T.ref_spot_neg_prob_diff(bg, pix, px, spot, z_factor=zf, variance=var, nthreads=nt)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), (a, b)


def test_non_positive_brightness_or_blur_gives_nan():
    bg, pix, px, spot = T.synthetic_block(5, 2, 4, (5, 5, 5))
    for i in (0, 1):
        s = spot.copy()
        s[i] = 0.0
        assert np.isnan(T.spot_neg_prob_diff(bg, pix, px, s)).all()
        r = T.ref_spot_neg_prob_diff(bg, pix, px, s)
        if r is not None:
            assert np.isnan(r).all()


def test_gradient_matches_central_differences():
    """With z factor 1 the returned vector is the gradient of
    -(mean over samples of log P + log priors); the reference's z derivative
    omits the 1/z_factor^2 of the shape's z scaling, which only z factor 1
    makes exact."""
    bg, pix, px, spot = T.synthetic_block(6, 5, 15, (8, 8, 6))
    kw = dict(z_factor=1.0, variance=1.0, mu_brightness=3.5, sigma_brightness=1.0, mu_blur=0.252148, sigma_blur=0.1)

    def f(sp):
        _, lp = T.spot_neg_prob_diff(bg, pix, px, sp, with_logp=True, **kw)

        def lln(x, mu, s):
            return -(np.log(x) - mu) ** 2 / (2 * s * s) - np.log(x) - np.log(s * np.sqrt(2 * np.pi))
        return -(lp.mean() + lln(sp[0], kw["mu_brightness"], kw["sigma_brightness"]) +
                 lln(sp[1], kw["mu_blur"], kw["sigma_blur"]))

    g = T.spot_neg_prob_diff(bg, pix, px, spot, **kw)
    for n in range(5):
        h = 1e-5 * max(1.0, abs(spot[n]))
        e = np.zeros(5)
        e[n] = h
        fd = (f(spot + e) - f(spot - e)) / (2 * h)
        assert abs(fd - g[n]) <= 1e-5 * max(1.0, abs(g[n])), (n, fd, g[n])


def _bleach_then_bright():
    """1400 dark frames, then 5 frames with a bright spot (see the GPU test)."""
    bg, pix, px, spot = T.synthetic_block(7, 3, 1400)
    rng = np.random.default_rng(1)
    pix = bg.mean(0) + rng.normal(0, 1, pix.shape)
    d = px - spot[2:]
    pix[-5:] += spot[0] * 3 / (spot[1] * np.sqrt(2 * np.pi)) * np.exp(-(d * d).sum(1) / (2 * spot[1] ** 2))
    return bg, pix, px, spot


def test_oracle_reproduces_reference_bits_long_bleach():
    if T.ref_lib() is None:
        pytest.skip("oracle/_ref/libref3b_host.so not built (reference sources absent)")
    bg, pix, px, spot = _bleach_then_bright()
    a = T.spot_neg_prob_diff(bg, pix, px, spot)
    b = T.ref_spot_neg_prob_diff(bg, pix, px, spot)
    assert np.isfinite(a).all()
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), (a, b)


def _emissions(bg, pix, px, spot):
    """Per (sample, frame): log p_on - log p_off, log p_off and d(log p_on)/d phi
    (spot_with_background.hh:98-133, unit z factor and variance)."""
    x = px.astype(np.float64)
    d0, d1, d2 = x[:, 0] - spot[2], x[:, 1] - spot[3], x[:, 2] - spot[4]
    s = -(d0 * d0 + d1 * d1 + d2 * d2) / (2 * spot[1] ** 2)
    k = np.exp(s) / (spot[1] * np.sqrt(2 * np.pi))
    v = k * spot[0]
    q = spot[0] / spot[1] ** 2
    der = np.stack([k, k * (-spot[0] * (1 + 2 * s) / spot[1]), k * d0 * q, k * d1 * q, k * d2 * q], 1)
    c0 = len(px) * np.log(2 * np.pi) / 2
    r = pix[None] - bg
    off = -(r * r).sum(-1) / 2 - c0
    gap = ((r * v).sum(-1) * 2 - (v * v).sum()) / 2
    de = np.einsum("sfp,pn->sfn", r - v, der)
    return gap, off, de


def _forward_exponent_form(gap, off, de, A, pi, per_state=True):
    """The GPU kernel's recursion (rfba_gb300/csrc/threeb.cu forward_kernel) in
    numpy: probabilities alpha_j and D_jk = alpha_j d(delta_j)/d phi_k as
    mantissas with an integer exponent per state (per_state=False: one scale
    for all states, which underflows when the mass sits in a state that cannot
    reach the one the frames favour). Returns (mean gradient of log P, log P)."""
    S, F = gap.shape
    g = np.zeros((S, 5))
    lp = np.zeros(S)
    zero = -(1 << 29)
    for s in range(S):
        m = np.where(gap[s] <= 0, off[s], off[s] + gap[s])
        p = np.stack([np.exp(np.minimum(gap[s], 0)), np.exp(np.minimum(-gap[s], 0))], 1)
        p = np.column_stack([p[:, 0], p[:, 1], p[:, 1]])  # bleached emits like off
        X = np.zeros((3, 6))
        X[:, 5] = pi * p[0]
        X[0, :5] = X[0, 5] * de[s, 0]
        E = np.zeros(3, np.int64)

        def normalise(X, E):
            for j in range(3 if per_state else 1):
                rows = [j] if per_state else [0, 1, 2]
                ref = X[j, 5] if per_state else X[:, 5].sum()
                if ref == 0:
                    E[rows] = zero
                    continue
                sh = np.frexp(ref)[1]
                X[rows] = np.ldexp(X[rows], -sh)
                E[rows] += sh
            return X, E

        X, E = normalise(X, E)
        for t in range(1, F):
            Y = np.zeros((3, 6))
            En = np.zeros(3, np.int64)
            for j in range(3):
                live = [i for i in range(3) if A[i, j] != 0]
                Em = max([E[i] for i in live] + [zero])
                c = np.array([A[i, j] * np.ldexp(1.0, int(E[i] - Em)) if -1022 <= E[i] - Em <= 0 else 0.0
                              for i in range(3)])
                Y[j] = p[t, j] * (c @ X)
                En[j] = Em
            Y[0, :5] += Y[0, 5] * de[s, t]
            X, E = normalise(Y, En)
        Em = E.max()
        w = np.array([np.ldexp(1.0, int(e - Em)) if e - Em >= -1022 else 0.0 for e in E])
        tot = w @ X
        with np.errstate(all="ignore"):
            g[s] = tot[:5] / tot[5]
            lp[s] = m.sum() + np.log(tot[5]) + Em * np.log(2)
    return g, lp


def _prior(spot):
    def dlln(x, mu, sg):
        return -(1 + (np.log(x) - mu) / (sg * sg)) / x
    return np.array([dlln(spot[0], 3.5, 1.0), dlln(spot[1], 0.252148, 0.1), 0, 0, 0])


@pytest.mark.parametrize("case", ["seed0", "seed3", "dense", "long_bleach"])
def test_exponent_form_matches_log_space(case):
    """The probability form with per-state exponents (what the GPU runs) gives
    the log-space reference's gradient to 1e-10 and log probability to 1e-13;
    with one scale for all states the long-bleach case underflows to NaN."""
    A, pi = T.A_SHIPPED, T.PI_SHIPPED
    if case == "long_bleach":
        bg, pix, px, spot = _bleach_then_bright()
    elif case == "dense":
        A = np.array([[0.7, 0.2, 0.1], [0.3, 0.6, 0.1], [0.05, 0.05, 0.9]])
        pi = np.array([0.2, 0.5, 0.3])
        bg, pix, px, spot = T.synthetic_block(11, 4, 40, (8, 8, 6))
    else:
        bg, pix, px, spot = T.synthetic_block(int(case[-1]), 4, 60)
    want, lpw = T.spot_neg_prob_diff(bg, pix, px, spot, A=A, pi=pi, with_logp=True)
    gap, off, de = _emissions(bg, pix, px, spot)
    g, lp = _forward_exponent_form(gap, off, de, A, pi)
    got = -(g.mean(0) + _prior(spot))
    assert np.max(np.abs(got - want)) <= 1e-10 * np.max(np.abs(want)), (got, want)
    assert np.max(np.abs(lp - lpw) / np.abs(lpw)) <= 1e-13
    if case == "long_bleach":
        g1, lp1 = _forward_exponent_form(gap, off, de, A, pi, per_state=False)
        assert not np.isfinite(lp1).all()


def _limit(mu=3.5, sigma=1.0, max_motion=0.5):
    """The reference's motion limits (multispot5.cc:1484, storm.h:386-389):
    cg.max_motion x (log-normal std of the brightness prior, 1, 1, 1, 1)."""
    return max_motion * np.array([np.sqrt((np.exp(sigma ** 2) - 1) * np.exp(2 * mu + sigma ** 2)), 1, 1, 1, 1])


OPT_CASES = [  # (seed, S, F, mask shape, start scale, max iterations)
    (0, 4, 12, (7, 6, 5), (1.0, 1.0, 1, 1, 1), 5),
    (1, 6, 30, (9, 9, 7), (1.0, 1.0, 1, 1, 1), 20),
    (2, 3, 20, (8, 8, 6), (0.05, 1.0, 1, 1, 1), 5),   # dim start: the first steps reach brightness <= 0 (NaN)
    (3, 2, 25, (9, 8, 6), (1.0, 3.0, 1, 1, 1), 8),    # wide start
]


@pytest.mark.parametrize("case", OPT_CASES, ids=[f"seed{c[0]}" for c in OPT_CASES])
def test_optimiser_reproduces_reference_bits(case):
    """rfba_cg_only_run (the library's ConjugateGradientOnly<5>) driven by the
    oracle's gradient retraces the reference's own optimiser driven by the
    reference's gradient, bit for bit, line search for line search."""
    if T.ref_lib() is None:
        pytest.skip("oracle/_ref/libref3b_host.so not built (reference sources absent)")
    from rfba_gb300 import srrf
    seed, S, F, shape, scale, iters = case
    bg, pix, px, spot = T.synthetic_block(seed, S, F, shape)
    spot = spot * np.array(scale)
    limit = _limit()
    want, it_want = T.ref_cg_optimise(bg, pix, px, spot, limit, iters)
    got, it, ev = srrf.cg_only_run(lambda x: T.spot_neg_prob_diff(bg, pix, px, x), spot, limit, iters)
    assert it == it_want
    assert ev >= it + 1
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (got, want)


def test_optimiser_moves_towards_the_spot():
    """On a block whose data hold the spot being fitted, the optimiser shrinks
    the gradient and moves the position towards the spot's centre."""
    from rfba_gb300 import srrf
    bg, pix, px, spot = T.synthetic_block(4, 6, 40, (9, 9, 7))
    g0 = T.spot_neg_prob_diff(bg, pix, px, spot)
    got, it, ev = srrf.cg_only_run(lambda x: T.spot_neg_prob_diff(bg, pix, px, x), spot, _limit(), 30)
    g1 = T.spot_neg_prob_diff(bg, pix, px, got)
    assert np.all(np.isfinite(got)) and got[0] > 0 and got[1] > 0
    assert np.max(np.abs(g1)) < 0.1 * np.max(np.abs(g0))


def test_optimiser_callback_error_stops_the_run():
    from rfba_gb300 import srrf
    calls = []

    def grad(x):
        calls.append(1)
        if len(calls) == 3:
            raise RuntimeError("gradient failed")
        return x - 1.0

    with pytest.raises(RuntimeError, match="gradient failed"):
        srrf.cg_only_run(grad, np.full(5, 3.0), np.ones(5), 10)
    assert len(calls) == 3


def test_optimiser_halves_steps_into_nan_region():
    """A gradient that is NaN for x0 <= 0 (as the spot gradient is for
    brightness or blur <= 0) with its minimum beyond that wall: the line search
    halves the step until the gradient is finite and the run stays finite, on
    the valid side."""
    from rfba_gb300 import srrf
    c = np.array([-5.0, 1.0, 2.0, -1.0, 0.5])
    seen_nan = []

    def grad(x):
        if x[0] <= 0:
            seen_nan.append(1)
            return np.full(5, np.nan)
        return x - c

    x0 = np.array([0.5, 0.0, 0.0, 0.0, 0.0])
    got, it, ev = srrf.cg_only_run(grad, x0, np.full(5, 2.0), 10)
    assert seen_nan, "the first step should cross into the NaN region"
    assert np.all(np.isfinite(got)) and got[0] > 0
    assert np.sum((got - c) ** 2) < np.sum((x0 - c) ** 2)  # it still descends


def test_optimiser_stops_on_a_zero_gradient():
    """A start where the gradient is exactly zero: the allowed step is
    infinite (the reference's search then steps to NaN, or halves an infinite
    step forever when the gradient there is NaN); this one stays at the start
    and finishes, the gradient being under tolerance."""
    from rfba_gb300 import srrf
    got, it, ev = srrf.cg_only_run(lambda x: np.zeros(5), np.ones(5), np.ones(5), 7)
    np.testing.assert_array_equal(got, np.ones(5))
    assert it == 1 and ev == 1
    # a gradient that is NaN away from the start and zero at it
    got, it, ev = srrf.cg_only_run(lambda x: np.zeros(5) if np.all(x == 1) else np.full(5, np.nan), np.ones(5),
                                   np.ones(5), 7)
    np.testing.assert_array_equal(got, np.ones(5))


def _golden_cases():
    from pathlib import Path
    z = np.load(Path(__file__).resolve().parent / "golden" / "threeb_golden.npz")
    return [{k.split("_", 1)[1]: z[k] for k in z.files if k.startswith(f"c{i}_")} for i in range(int(z["ncases"]))]


def test_golden_reproduced_by_oracle_and_optimiser():
    """tests/golden/threeb_golden.npz holds the reference's own gradient and
    optimised spot (its headers compiled on the host, make_golden_3b.py): the
    oracle gives the same gradient bits and the library's optimiser, on the
    oracle's gradient, the same spot bits and line-search count, without the
    reference tree."""
    from rfba_gb300 import srrf
    limit = _limit()
    for c in _golden_cases():
        bg, pix, px, spot = c["bg"], c["pix"], c["px"], c["spot"]
        g = T.spot_neg_prob_diff(bg, pix, px, spot)
        assert np.array_equal(g.view(np.uint64), c["grad"].view(np.uint64)), (g, c["grad"])
        x, it, ev = srrf.cg_only_run(lambda v: T.spot_neg_prob_diff(bg, pix, px, v), spot, limit,
                                     int(c["iters"]))
        assert it == int(c["opt_it"])
        assert np.array_equal(x.view(np.uint64), c["opt"].view(np.uint64)), (x, c["opt"])
