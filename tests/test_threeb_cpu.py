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
