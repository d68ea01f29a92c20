"""Oracle for 3B's Gibbs sampler and free energy (numpy restatement).

TEST INFRASTRUCTURE ONLY: imported by tests/ and by bench.py's CPU legs, never
by the product package. It restates, in FP64 and in the reference's operation
order where that decides the bits:

- `spot_intensity`: compute_spot_intensity with spot_shape (RFBA Main/
  sampled_multispot.h:182-191, storm.h:229-235);
- `spot_masks`: get_spot_pixels with getBall (multispot5.cc:1001-1020,
  1259-1272);
- `trace`: the deterministic part of one GibbsSampler2 sweep
  (sampled_multispot.h:658-690) given the states it drew: per spot, the masked
  emission log probabilities (spot_with_background.hh:98-137), the forward
  filter (forward_algorithm.h:385-431, normalised) and the forward-backward
  posterior (forward_algorithm.h:447-484);
- `free_energy`: the arithmetic of NegativeFreeEnergy::compute_with_mask
  (multispot5.cc:335-405) given each draw's sum of squared residuals;
- `spot_hessian_table`: spot_shape_hess_position (storm.h:87-146), value,
  gradient and Hessian of a spot at every pixel;
- `free_energy_hessian_draws`: FreeEnergyHessian::hessian (multispot5.cc:
  693-775) given the sampler's draws;
- `hessian_expectation`: what sampled_background_spot_hessian_ffbs
  (multispot5.cc:824-985) converges to as its backward samples grow: the
  per-frame parts over all pixels, the posterior of the spot's chain per
  sample (SpotWithBackground, forward_algorithm_delta, backward_sampling) and
  the expectation of hess + deriv deriv^T under it, exactly, from the
  posterior's single and pair marginals (backward sampling walks a reverse-time
  Markov chain, so P(s_t = 0, s_u = 0) is a product of its transitions).

`port_*` run the C++ port in oracle/gibbs_port.cpp (the reference's MT19937
stream, sampler and main-loop pass restated; built everywhere, the CPU
baseline of bench.py). `ref_*` run the reference's own code compiled on the host
(oracle/_ref/libref3b_gibbs_host.so, built by oracle/build_ref.sh where the
reference tree exists), which pins this module in tests/test_gibbs_cpu.py.
"""
from __future__ import annotations

import ctypes
import math
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_LIB_PATH = HERE / "_ref" / "libref3b_gibbs_host.so"
_ref = None


def _ln(x: float) -> float:
    """forward_algorithm.h:34-40: ln(0) is -1e100."""
    return -1e100 if x == 0 else math.log(x)


def spot_intensity(pixels: np.ndarray, spots: np.ndarray, z_factor: float) -> np.ndarray:
    """[K][P]: exp(s) * brightness / (blur sqrt(2 pi)), s = -|x - mu|^2 / (2 blur^2)
    with the z difference divided by the z factor."""
    px = np.asarray(pixels, np.float64).reshape(-1, 3)
    sp = np.asarray(spots, np.float64).reshape(-1, 5)
    out = np.empty((len(sp), len(px)))
    r_2_pi = math.sqrt(2 * math.pi)
    for k, phi in enumerate(sp):
        d0 = px[:, 0] - phi[2]
        d1 = px[:, 1] - phi[3]
        d2 = (px[:, 2] - phi[4]) / z_factor
        s = -(d0 * d0 + d1 * d1 + d2 * d2) / (2 * phi[1] * phi[1])
        out[k] = np.exp(s) * phi[0] / (phi[1] * r_2_pi)
    return out


def _ball(radius: float):
    r32 = np.float32(radius)
    r = int(math.ceil(np.float32(r32 + np.float32(1))))
    lim = np.float32(r32 * r32)
    pts = []
    for z in range(-r, r + 1):
        for y in range(-r, r + 1):
            for x in range(-r, r + 1):
                if np.float32(x * x + y * y + z * z) <= lim:
                    pts.append((x, y, z))
    return pts


def _round_away(v: float) -> int:
    return int(v + 0.5) if v > 0.0 else int(v - 0.5)


def spot_masks(pixels: np.ndarray, spots: np.ndarray):
    """(offsets [K+1], indices): get_spot_pixels for every spot; pixels sorted
    by (z, y, x)."""
    px = np.asarray(pixels, np.int64).reshape(-1, 3)
    index = {(int(a), int(b), int(c)): i for i, (a, b, c) in enumerate(px)}
    offs, idx = [0], []
    for phi in np.asarray(spots, np.float64).reshape(-1, 5):
        o = (_round_away(phi[2]), _round_away(phi[3]), _round_away(phi[4]))
        for (x, y, z) in _ball(float(phi[1] * 6 + 1)):
            i = index.get((x + o[0], y + o[1], z + o[2]))
            if i is not None:
                idx.append(i)
        offs.append(len(idx))
    return np.asarray(offs, np.int32), np.asarray(idx, np.int32)


def _emission(pix, cur, v, mask, var):
    """log p(on), log p(off) per frame over the mask."""
    d = pix[:, mask]
    c = cur[:, mask]
    vv = v[mask]
    n = len(mask)
    off = -np.sum((d - c) ** 2, axis=1)
    on = -np.sum((d - (c + vv)) ** 2, axis=1)
    cst = n * math.log(2 * math.pi * var) / 2
    return on / (2 * var) - cst, off / (2 * var) - cst


def _forward_log(lp_on, lp_off, A, pi):
    """delta [F][3] (forward_algorithm_delta2)."""
    F = len(lp_on)
    lA = np.array([[_ln(A[i][j]) for j in range(3)] for i in range(3)])
    B = np.stack([lp_on, lp_off, lp_off], 1)
    delta = np.empty((F, 3))
    delta[0] = [_ln(pi[i]) + B[0, i] for i in range(3)]
    for t in range(1, F):
        for j in range(3):
            z = max(delta[t - 1][i] + lA[i][j] for i in range(3))
            s = sum(math.exp(delta[t - 1][i] + lA[i][j] - z) for i in range(3))
            delta[t][j] = B[t, j] + z + _ln(s)
    return delta, B, lA


def _backward_log(B, lA):
    F = len(B)
    eps = np.zeros((F, 3))
    for t in range(F - 2, -1, -1):
        for i in range(3):
            z = max(lA[i][j] + B[t + 1, j] + eps[t + 1][j] for j in range(3))
            s = sum(math.exp(lA[i][j] + B[t + 1, j] + eps[t + 1][j] - z) for j in range(3))
            eps[t][i] = _ln(s) + z
    return eps


def _normalise(a):
    a = a - a.max(axis=1, keepdims=True)
    e = np.exp(a)
    return e / e.sum(axis=1, keepdims=True)


def trace(pix, si, moff, midx, A, pi, variance, states):
    """One sweep from all spots off with drawn states [K][F]: lp [K][F][2],
    filtered [K][F][3], posterior [K][F][3]."""
    pix = np.asarray(pix, np.float64)
    F, P = pix.shape
    K = len(si)
    A = np.asarray(A, np.float64).reshape(3, 3)
    cur = np.zeros((F, P))
    lp = np.empty((K, F, 2))
    filt = np.empty((K, F, 3))
    post = np.empty((K, F, 3))
    for k in range(K):
        mask = np.asarray(midx[moff[k]:moff[k + 1]], np.int64)
        on, off = _emission(pix, cur, si[k], mask, variance)
        lp[k, :, 0], lp[k, :, 1] = on, off
        delta, B, lA = _forward_log(on, off, A, pi)
        eps = _backward_log(B, lA)
        filt[k] = _normalise(delta)
        post[k] = _normalise(delta + eps)
        rows = np.nonzero(np.asarray(states[k]) == 0)[0]
        if len(rows) and len(mask):
            cur[np.ix_(rows, mask)] += si[k][mask]
    return lp, filt, post


def variance_from_sample(sample, samples, base_sigma, scale_pow):
    scale = math.pow(1.25, sample * 1. / samples * scale_pow)
    sigma = base_sigma * scale
    return sigma * sigma


def log_log_normal(x, mu, sigma):
    a = _ln(x) - mu
    return -(a * a) / (2 * (sigma * sigma)) - _ln(x) - _ln(sigma * math.sqrt(2 * math.pi))


def free_energy(residuals, variance, P, F, spots, mu_b, sigma_b, mu_blur, sigma_blur):
    """compute_with_mask's value from each draw's sum of squared residuals."""
    samples = len(residuals)
    base_sigma = math.sqrt(variance)
    scale_pow = 100.0
    n = (P * F) & 0xFFFFFFFF  # unsigned int product, as the reference
    total = 0.0
    for sample in range(samples):
        v1 = variance_from_sample(sample - 2, samples, base_sigma, scale_pow)
        v2 = variance_from_sample(sample - 1, samples, base_sigma, scale_pow)
        v3 = variance_from_sample(sample + 1, samples, base_sigma, scale_pow)
        v4 = variance_from_sample(sample + 2, samples, base_sigma, scale_pow)
        err_sum = -float(residuals[sample])
        e = [err_sum / (2 * v) - n * math.log(2 * math.pi * v) / 2 for v in (v1, v2, v3, v4)]
        total += (-e[0] + 8 * e[1] - 8 * e[2] + e[3]) / 12
    log_final = (math.log(variance_from_sample(samples, samples, base_sigma, scale_pow) * 2 * math.pi) / 2) * P * F
    priors = 0.0
    for phi in np.asarray(spots, np.float64).reshape(-1, 5):
        priors += log_log_normal(float(phi[0]), mu_b, sigma_b)
        priors += log_log_normal(float(phi[1]), mu_blur, sigma_blur)
    return -(total + priors - log_final)


def spot_hessian_table(pixels, spot, z_factor):
    """(value [P], gradient [P][5], Hessian [P][5][5]) of spot_shape_hess_position
    at every pixel (storm.h:87-146), symmetric (the reference leaves [4][3]
    unwritten)."""
    px = np.asarray(pixels, np.float64).reshape(-1, 3)
    p0, p1 = float(spot[0]), float(spot[1])
    dx, dy, dz = px[:, 0] - spot[2], px[:, 1] - spot[3], px[:, 2] - spot[4]
    s = -(dx * dx + dy * dy + (dz / z_factor) ** 2) / (2 * p1 * p1)
    r = math.sqrt(2 * math.pi)
    es = np.exp(s)
    val = es * p0 / (p1 * r)
    c = es / (p1 * r)
    g = np.stack([c, c * (-p0 * (1 + 2 * s) / p1), c * dx * (p0 / p1 ** 2), c * dy * (p0 / p1 ** 2),
                  c * dz * (p0 / p1 ** 2)], 1)
    H = np.zeros((len(px), 5, 5))
    H[:, 0, 1] = -es * (1 + 2 * s) / (p1 * p1 * r)
    for a, d in ((2, dx), (3, dy), (4, dz)):
        H[:, 0, a] = es * d / (p1 ** 3 * r)
        H[:, 1, a] = -p0 * es * (3 + 2 * s) * d / (p1 ** 4 * r)
        H[:, a, a] = p0 * es * (d * d - p1 * p1) / (r * p1 ** 5)
    H[:, 1, 1] = 2 * p0 * es * (1 + 5 * s + 2 * s * s) / (p1 ** 3 * r)
    H[:, 2, 3] = p0 * es * dx * dy / (r * p1 ** 5)
    H[:, 2, 4] = p0 * es * dx * dz / (r * p1 ** 5)
    H[:, 3, 4] = p0 * es * dy * dz / (r * p1 ** 5)
    iu = np.triu_indices(5, 1)
    H[:, iu[1], iu[0]] = H[:, iu[0], iu[1]]
    return val, g, H


def free_energy_hessian_draws(pix, pixels, spots, spot, states, ints, variance, z_factor, mu_b, sigma_b, mu_blur,
                              sigma_blur):
    """FreeEnergyHessian::hessian given the draws: states [S][K][F], draw
    intensities [S][F][P] (holding every spot)."""
    pix = np.asarray(pix, np.float64)
    S = len(states)
    sp = np.asarray(spots, np.float64).reshape(-1, 5)[spot]
    _, g, H = spot_hessian_table(pixels, sp, z_factor)
    gg = np.einsum("pa,pb->ab", g, g)
    sum1, sum2, sumd = np.zeros((5, 5)), np.zeros((5, 5)), np.zeros(5)
    for i in range(S):
        on = np.asarray(states[i][spot]) == 0
        e = (pix - ints[i])[on]  # [frames on][P]
        h = np.einsum("fp,pab->ab", e, H) - on.sum() * gg
        d = (e @ g).sum(0)
        h[0, 0] += (1 + (_ln(sp[0]) - mu_b - 1) / (sigma_b * sigma_b)) / (sp[0] * sp[0])
        h[1, 1] += (1 + (_ln(sp[1]) - mu_blur - 1) / (sigma_blur * sigma_blur)) / (sp[1] * sp[1])
        d[0] += -(1 + (_ln(sp[0]) - mu_b) / (sigma_b * sigma_b)) / sp[0]
        d[1] += -(1 + (_ln(sp[1]) - mu_blur) / (sigma_blur * sigma_blur)) / sp[1]
        sum1 += h
        sum2 += np.outer(d, d)
        sumd += d
    sum1 /= S * variance
    sum2 /= S * variance
    sumd /= S * variance
    return sum1 + sum2 - np.outer(sumd, sumd)


def _posterior_chain(lp_on, lp_off, A, pi):
    """Single marginals m [F][3] and the reverse-time transitions R [F][3][3]
    (R[t][j][i] = P(s_t = i | s_{t+1} = j)) of the chain's posterior."""
    F = len(lp_on)
    A = np.asarray(A, np.float64).reshape(3, 3)
    lB = np.stack([lp_on, lp_off, lp_off], 1)
    alpha = np.empty((F, 3))
    a = np.asarray(pi, np.float64) * np.exp(lB[0] - lB[0].max())
    alpha[0] = a / a.sum()
    for t in range(1, F):
        a = (alpha[t - 1] @ A) * np.exp(lB[t] - lB[t].max())
        alpha[t] = a / a.sum()
    R = np.zeros((F, 3, 3))
    for t in range(F - 1):
        w = alpha[t][:, None] * A  # [i][j]
        tot = w.sum(0)
        R[t] = np.where(tot[:, None] > 0, (w / np.where(tot > 0, tot, 1)).T, 0)
    m = np.empty((F, 3))
    m[F - 1] = alpha[F - 1]
    for t in range(F - 2, -1, -1):
        m[t] = m[t + 1] @ R[t]
    return m, R


def hessian_expectation(bg, pix, pixels, spot, A, pi, variance, z_factor, mu_b, sigma_b, mu_blur, sigma_blur):
    """The limit of sampled_background_spot_hessian_ffbs as bs_iterations grows."""
    bg = np.asarray(bg, np.float64)
    pix = np.asarray(pix, np.float64)
    S, F, P = bg.shape
    val, g, H = spot_hessian_table(pixels, spot, z_factor)
    gg = np.einsum("pa,pb->ab", g, g)
    cst = P * math.log(2 * math.pi * variance) / 2
    sum_h = np.zeros((5, 5))
    sum_d = np.zeros(5)
    for i in range(S):
        e = pix - (bg[i] + val)  # [F][P]
        hp = np.einsum("fp,pab->fab", e, H) - gg
        dp = e @ g
        lon = -np.sum(e * e, 1) / (2 * variance) - cst
        loff = -np.sum((pix - bg[i]) ** 2, 1) / (2 * variance) - cst
        m, R = _posterior_chain(lon, loff, A, pi)
        on = m[:, 0]
        sum_h += np.einsum("f,fab->ab", on, hp)
        sum_d += on @ dp
        # E[D D^T] = sum_t P(t on) d_t d_t^T + sum_{t < u} P(t on, u on) (d_t d_u^T + d_u d_t^T)
        for u in range(F):
            sum_h += on[u] * np.outer(dp[u], dp[u])
            cond = np.array([1.0, 0.0, 0.0])  # P(s_t = . | s_u = 0), walking t down from u
            for t in range(u - 1, -1, -1):
                cond = cond @ R[t]
                pj = on[u] * cond[0]
                if pj != 0:
                    sum_h += pj * (np.outer(dp[t], dp[u]) + np.outer(dp[u], dp[t]))
    sum_h /= S * variance
    sum_d /= S * variance
    out = sum_h - np.outer(sum_d, sum_d)
    out[0, 0] += (1 + (_ln(spot[0]) - mu_b - 1) / (sigma_b * sigma_b)) / (spot[0] * spot[0])
    out[1, 1] += (1 + (_ln(spot[1]) - mu_blur - 1) / (sigma_blur * sigma_blur)) / (spot[1] * spot[1])
    return out


# ---- the reference's own code (compiled here) --------------------------------

def ref_available() -> bool:
    return REF_LIB_PATH.exists()


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def ref():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(str(REF_LIB_PATH))
        dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        bp = ctypes.POINTER(ctypes.c_ubyte)
        d, i = ctypes.c_double, ctypes.c_int
        L.ref_spot_intensity.argtypes = [ip, i, dp, i, d, dp]
        L.ref_gibbs_trace.argtypes = [dp, dp, ip, ip, i, i, i, dp, dp, d, bp, dp, dp, dp]
        L.ref_gibbs_run.argtypes = [dp, dp, ip, ip, i, i, i, dp, dp, d, i, i, i, bp, dp]
        L.ref_free_energy.argtypes = [dp, ip, dp, ip, ip, i, i, i, dp, dp, d, d, d, d, d, d, i, i, i, dp]
        L.ref_free_energy.restype = d
        L.ref_spot_hessian.argtypes = [dp, dp, ip, i, i, i, dp, dp, dp, d, d, d, d, d, d, i, i, dp]
        L.ref_free_energy_hessian_draws.argtypes = [dp, ip, dp, i, i, i, i, i, bp, dp, d, d, d, d, d, d, dp]
        _ref = L
    return _ref


def ref_spot_intensity(pixels, spots, z_factor):
    px = np.ascontiguousarray(pixels, np.int32)
    sp = np.ascontiguousarray(spots, np.float64).reshape(-1, 5)
    out = np.empty((len(sp), len(px)))
    ref().ref_spot_intensity(_p(px, ctypes.c_int), len(px), _p(sp, ctypes.c_double), len(sp), z_factor,
                             _p(out, ctypes.c_double))
    return out


def ref_trace(pix, si, moff, midx, A, pi, variance, states):
    pix = np.ascontiguousarray(pix, np.float64)
    si = np.ascontiguousarray(si, np.float64)
    F, P = pix.shape
    K = len(si)
    moff = np.ascontiguousarray(moff, np.int32)
    midx = np.ascontiguousarray(midx, np.int32) if len(midx) else np.zeros(1, np.int32)
    st = np.ascontiguousarray(states, np.uint8)
    A = np.ascontiguousarray(A, np.float64).reshape(9)
    pi = np.ascontiguousarray(pi, np.float64)
    lp, filt, post = np.empty((K, F, 2)), np.empty((K, F, 3)), np.empty((K, F, 3))
    ref().ref_gibbs_trace(_p(pix, ctypes.c_double), _p(si, ctypes.c_double), _p(moff, ctypes.c_int),
                          _p(midx, ctypes.c_int), K, F, P, _p(A, ctypes.c_double), _p(pi, ctypes.c_double), variance,
                          _p(st, ctypes.c_ubyte), _p(lp, ctypes.c_double), _p(filt, ctypes.c_double),
                          _p(post, ctypes.c_double))
    return lp, filt, post


def ref_run(pix, si, moff, midx, A, pi, variance, sweeps, n_draws, seed, want_int=False):
    pix = np.ascontiguousarray(pix, np.float64)
    si = np.ascontiguousarray(si, np.float64)
    F, P = pix.shape
    K = len(si)
    moff = np.ascontiguousarray(moff, np.int32)
    midx = np.ascontiguousarray(midx, np.int32) if len(midx) else np.zeros(1, np.int32)
    A = np.ascontiguousarray(A, np.float64).reshape(9)
    pi = np.ascontiguousarray(pi, np.float64)
    st = np.empty((n_draws, K, F), np.uint8)
    ints = np.empty((n_draws, F, P)) if want_int else None
    ref().ref_gibbs_run(_p(pix, ctypes.c_double), _p(si, ctypes.c_double), _p(moff, ctypes.c_int),
                        _p(midx, ctypes.c_int), K, F, P, _p(A, ctypes.c_double), _p(pi, ctypes.c_double), variance,
                        sweeps, n_draws, seed, _p(st, ctypes.c_ubyte),
                        _p(ints, ctypes.c_double) if want_int else None)
    return st, ints


def ref_free_energy(pix, pixels, spots, moff, midx, A, pi, variance, z_factor, mu_b, sigma_b, mu_blur, sigma_blur,
                    samples, sweeps, seed):
    pix = np.ascontiguousarray(pix, np.float64)
    F, P = pix.shape
    px = np.ascontiguousarray(pixels, np.int32)
    sp = np.ascontiguousarray(spots, np.float64).reshape(-1, 5)
    moff = np.ascontiguousarray(moff, np.int32)
    midx = np.ascontiguousarray(midx, np.int32) if len(midx) else np.zeros(1, np.int32)
    A = np.ascontiguousarray(A, np.float64).reshape(9)
    pi = np.ascontiguousarray(pi, np.float64)
    res = np.empty(samples)
    v = ref().ref_free_energy(_p(pix, ctypes.c_double), _p(px, ctypes.c_int), _p(sp, ctypes.c_double),
                              _p(moff, ctypes.c_int), _p(midx, ctypes.c_int), len(sp), F, P, _p(A, ctypes.c_double),
                              _p(pi, ctypes.c_double), variance, z_factor, mu_b, sigma_b, mu_blur, sigma_blur,
                              samples, sweeps, seed, _p(res, ctypes.c_double))
    return v, res


def ref_spot_hessian(bg, pix, pixels, spot, A, pi, variance, z_factor, mu_b, sigma_b, mu_blur, sigma_blur,
                     bs_iterations, seed):
    """The reference's sampled_background_spot_hessian_ffbs (one thread, its
    MT19937 seeded by simple_seed(seed)); entry [4][3] is indeterminate."""
    bg = np.ascontiguousarray(bg, np.float64)
    pix = np.ascontiguousarray(pix, np.float64)
    S, F, P = bg.shape
    px = np.ascontiguousarray(pixels, np.int32)
    sp = np.ascontiguousarray(spot, np.float64)
    A = np.ascontiguousarray(A, np.float64).reshape(9)
    pi = np.ascontiguousarray(pi, np.float64)
    out = np.empty((5, 5))
    ref().ref_spot_hessian(_p(bg, ctypes.c_double), _p(pix, ctypes.c_double), _p(px, ctypes.c_int), S, F, P,
                           _p(sp, ctypes.c_double), _p(A, ctypes.c_double), _p(pi, ctypes.c_double), variance, z_factor,
                           mu_b, sigma_b, mu_blur, sigma_blur, bs_iterations, seed, _p(out, ctypes.c_double))
    return out


def ref_free_energy_hessian_draws(pix, pixels, spots, spot, states, ints, variance, z_factor, mu_b, sigma_b, mu_blur,
                                  sigma_blur):
    pix = np.ascontiguousarray(pix, np.float64)
    F, P = pix.shape
    px = np.ascontiguousarray(pixels, np.int32)
    sp = np.ascontiguousarray(spots, np.float64).reshape(-1, 5)
    st = np.ascontiguousarray(states, np.uint8)
    ints = np.ascontiguousarray(ints, np.float64)
    out = np.empty((5, 5))
    ref().ref_free_energy_hessian_draws(_p(pix, ctypes.c_double), _p(px, ctypes.c_int), _p(sp, ctypes.c_double),
                                        len(sp), F, P, spot, len(st), _p(st, ctypes.c_ubyte), _p(ints, ctypes.c_double),
                                        variance, z_factor, mu_b, sigma_b, mu_blur, sigma_blur,
                                        _p(out, ctypes.c_double))
    return out


# ---- the C++ port (oracle/gibbs_port.cpp) -------------------------------------

_port = None


def port():
    global _port
    if _port is None:
        from oracle import threeb as T3
        T3.build()
        L = ctypes.CDLL(str(T3.LIB_PATH))
        dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        bp = ctypes.POINTER(ctypes.c_ubyte)
        d, i = ctypes.c_double, ctypes.c_int
        L.port_gibbs_run.argtypes = [dp, dp, ip, ip, i, i, i, dp, dp, d, i, i, i, bp, dp]
        L.port_optimise_pass.argtypes = [dp, ip, i, i, dp, ip, i, i, i, i, dp, d, dp, dp, d, d, d, d, d, d, i, i, i,
                                         dp]
        L.port_spot_hessian.argtypes = [dp, dp, ip, i, i, i, dp, d, d, dp, dp, d, d, d, d, i, i, i, dp]
        _port = L
    return _port


def port_run(pix, si, moff, midx, A, pi, variance, sweeps, n_draws, seed, want_int=False):
    pix = np.ascontiguousarray(pix, np.float64)
    si = np.ascontiguousarray(si, np.float64)
    F, P = pix.shape
    K = len(si)
    moff = np.ascontiguousarray(moff, np.int32)
    midx = np.ascontiguousarray(midx, np.int32) if len(midx) else np.zeros(1, np.int32)
    A = np.ascontiguousarray(A, np.float64).reshape(9)
    pi = np.ascontiguousarray(pi, np.float64)
    st = np.empty((n_draws, K, F), np.uint8)
    ints = np.empty((n_draws, F, P)) if want_int else None
    port().port_gibbs_run(_p(pix, ctypes.c_double), _p(si, ctypes.c_double), _p(moff, ctypes.c_int),
                          _p(midx, ctypes.c_int), K, F, P, _p(A, ctypes.c_double), _p(pi, ctypes.c_double), variance,
                          sweeps, n_draws, seed, _p(st, ctypes.c_ubyte),
                          _p(ints, ctypes.c_double) if want_int else None)
    return st, ints


def port_pass(pix, pixels, spots, pass_index, main_samples, sweeps, cg_max_iterations, limit, extra_radius, A, pi,
              variance, z_factor, mu_b, sigma_b, mu_blur, sigma_blur, seed, nthreads=16, max_spots=-1):
    """(spots after the pass, (seconds in the sampler, seconds in the optimiser))."""
    pix = np.ascontiguousarray(pix, np.float64)
    F, P = pix.shape
    px = np.ascontiguousarray(pixels, np.int32)
    sp = np.ascontiguousarray(spots, np.float64).reshape(-1, 5).copy()
    lim = np.ascontiguousarray(limit, np.float64)
    A = np.ascontiguousarray(A, np.float64).reshape(9)
    pi = np.ascontiguousarray(pi, np.float64)
    n = ctypes.c_int(len(sp))
    sec = np.zeros(2)
    rc = port().port_optimise_pass(_p(pix, ctypes.c_double), _p(px, ctypes.c_int), F, P, _p(sp, ctypes.c_double),
                                   ctypes.byref(n), pass_index, main_samples, sweeps, cg_max_iterations,
                                   _p(lim, ctypes.c_double), extra_radius, _p(A, ctypes.c_double),
                                   _p(pi, ctypes.c_double), variance, z_factor, mu_b, sigma_b, mu_blur, sigma_blur,
                                   seed, nthreads, max_spots, _p(sec, ctypes.c_double))
    assert rc == 0
    return sp[:n.value].copy(), (float(sec[0]), float(sec[1]))


def port_spot_hessian(bg, pix, pixels, spot, A, pi, variance, z_factor, mu_b, sigma_b, mu_blur, sigma_blur,
                      bs_iterations, seed, nthreads=16):
    """The port of sampled_background_spot_hessian_ffbs (threads over samples,
    MT19937 per thread)."""
    bg = np.ascontiguousarray(bg, np.float64)
    pix = np.ascontiguousarray(pix, np.float64)
    S, F, P = bg.shape
    px = np.ascontiguousarray(pixels, np.int32)
    sp = np.ascontiguousarray(spot, np.float64)
    A = np.ascontiguousarray(A, np.float64).reshape(9)
    pi = np.ascontiguousarray(pi, np.float64)
    out = np.empty((5, 5))
    port().port_spot_hessian(_p(bg, ctypes.c_double), _p(pix, ctypes.c_double), _p(px, ctypes.c_int), S, F, P,
                             _p(sp, ctypes.c_double), z_factor, variance, _p(A, ctypes.c_double),
                             _p(pi, ctypes.c_double), mu_b, sigma_b, mu_blur, sigma_blur, bs_iterations, seed, nthreads,
                             _p(out, ctypes.c_double))
    return out
