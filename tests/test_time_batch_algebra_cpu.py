"""The algebra behind the time-batched temporal reduction and its adjoint
(temporal_stream.cu), restated in float64 numpy and checked against the
direct two-pass formulas (kernel.cu:423-500, TRAC with ITC 0):

- the window sums of deviation products, carried batch by batch as sums of
  products of y_t = r_t - K (K the first batch's mean) and expanded in
  c = mean - K after the last batch, equal the sums of (r_t - mean) products;
- the cumulant of order 2, 3 and 4 formed from them equals the direct one;
- the mean over s of dC/da_s in closed form (a polynomial in those sums)
  equals the mean of the direct per-volume derivatives.
No GPU: this pins the arithmetic the kernels implement, not the kernels.
"""
import itertools

import numpy as np
import pytest


def _carry(r, k, tb):
    """The carried sums of temporal_stream.cu's trac_carry, batch by batch:
    (K, sum y, {subset: window sum of y products})."""
    T = len(r)
    N = T - k
    K = r[:min(tb, T)].mean()
    y = r - K
    sums = {}
    for size in range(1, k + 1):
        for sub in itertools.combinations(range(k), size):
            sums[sub] = 0.0
    ysum = 0.0
    for t0 in range(0, T, tb):
        for t in range(t0, min(T, t0 + tb)):
            ysum += y[t]
            w = t - (k - 1)
            if 0 <= w < N:
                win = y[w:w + k]
                for sub in sums:
                    sums[sub] += np.prod(win[list(sub)])
    return K, ysum, sums


def _deviation_sums(ysum, sums, k, T):
    """Window sums of deviation products from the carried y sums: every product
    of (y - c) terms expanded over the subsets it contains."""
    N = T - k
    c = ysum / T
    dev = {}
    for sub in sums:
        total = 0.0
        for size in range(len(sub) + 1):
            for part in itertools.combinations(sub, size):
                # the terms of the expansion keep `part` as y and take -c elsewhere
                ypart = sums[part] if part else float(N)
                total += ypart * (-c) ** (len(sub) - len(part))
        dev[sub] = total
    return dev


def _direct(r, k):
    T = len(r)
    N = T - k
    d = r - r.mean()
    dev = {}
    for size in range(1, k + 1):
        for sub in itertools.combinations(range(k), size):
            dev[sub] = sum(np.prod(d[w:w + k][list(sub)]) for w in range(max(N, 0)))
    return dev


def _cumulant(dev, k):
    if k == 2:
        return dev[(0, 1)]
    if k == 3:
        return dev[(0, 1, 2)]
    return dev[(0, 1, 2, 3)] - dev[(0, 1)] * dev[(2, 3)] - dev[(0, 2)] * dev[(1, 3)] - dev[(0, 3)] * dev[(1, 2)]


def _mean_dcda_closed(dev, k, T):
    """The closed form of temporal_stream_adjoint_kernel's mean_d."""
    if k == 2:
        s = dev[(0,)] + dev[(1,)]
    elif k == 3:
        s = dev[(1, 2)] + dev[(0, 2)] + dev[(0, 1)]
    else:
        S = [dev[(j,)] for j in range(4)]
        ab, ac, ad, bc, bd, cd = (dev[(0, 1)], dev[(0, 2)], dev[(0, 3)], dev[(1, 2)], dev[(1, 3)], dev[(2, 3)])
        s = (dev[(1, 2, 3)] + dev[(0, 2, 3)] + dev[(0, 1, 3)] + dev[(0, 1, 2)]) - \
            (S[1] * cd + S[2] * bd + S[3] * bc) - (S[0] * cd + S[3] * ac + S[2] * ad) - \
            (S[3] * ab + S[0] * bd + S[1] * ad) - (S[2] * ab + S[1] * ac + S[0] * bc)
    return s / T


def _mean_dcda_direct(r, k):
    """mean_s dC/da_s of temporal_adjoint_kernel, summed directly."""
    T = len(r)
    N = T - k
    a = r - r.mean()
    dev = _direct(r, k)

    def at(t):
        return a[t] if 0 <= t < T else 0.0

    total = 0.0
    for s in range(T):
        for l in range(k):
            t0 = s - l
            if not 0 <= t0 < N:
                continue
            if k == 2:
                total += at(t0 + 1 - l)
            elif k == 3:
                total += np.prod([at(t0 + q) for q in range(3) if q != l])
            else:
                A, B, C, D = at(t0), at(t0 + 1), at(t0 + 2), at(t0 + 3)
                AB, AC, AD, BC, BD, CD = (dev[(0, 1)], dev[(0, 2)], dev[(0, 3)], dev[(1, 2)], dev[(1, 3)],
                                          dev[(2, 3)])
                total += [B * C * D - B * CD - C * BD - D * BC, A * C * D - A * CD - D * AC - C * AD,
                          A * B * D - D * AB - A * BD - B * AD, A * B * C - C * AB - B * AC - A * BC][l]
    return total / T


@pytest.mark.parametrize("k", [2, 3, 4])
@pytest.mark.parametrize("T,tb", [(31, 1), (31, 7), (40, 25), (26, 25), (6, 2), (5, 3)])
def test_carried_sums_expand_to_the_direct_cumulant(k, T, tb):
    rng = np.random.default_rng(1000 * k + T + tb)
    r = rng.normal(3.0, 2.0, size=T) + 0.3 * np.sin(np.arange(T))
    K, ysum, sums = _carry(r, k, tb)
    dev = _deviation_sums(ysum, sums, k, T)
    want = _direct(r, k)
    scale = max(1.0, max(abs(v) for v in want.values()))
    for sub in want:
        assert abs(dev[sub] - want[sub]) <= 1e-11 * scale, (sub, dev[sub], want[sub])
    c_got, c_want = _cumulant(dev, k), _cumulant(want, k)
    assert abs(c_got - c_want) <= 1e-10 * max(1.0, abs(c_want)) * scale
    m_got, m_want = _mean_dcda_closed(dev, k, T), _mean_dcda_direct(r, k)
    assert abs(m_got - m_want) <= 1e-10 * max(1.0, abs(m_want)) * scale


@pytest.mark.parametrize("k", [2, 3, 4])
def test_series_no_longer_than_the_order(k):
    """An empty window: every sum, the cumulant and mean_d are zero."""
    r = np.array([1.0, 2.0, 0.5, 4.0])[:k]
    K, ysum, sums = _carry(r, k, 1)
    dev = _deviation_sums(ysum, sums, k, len(r))
    assert all(abs(v) < 1e-12 for v in dev.values())
    assert _cumulant(_direct(r, k), k) == 0.0
    assert _mean_dcda_direct(r, k) == 0.0
