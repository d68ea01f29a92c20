"""The oracle is pinned to the reference (CPU only).

tests/golden/golden.npz holds outputs of the reference's own GradientCalc
sources compiled as host code (tests/golden/make_golden.py). The FP32 port in
oracle/ must reproduce them bit for bit; the FP64 oracle must agree with them to
the reference's own FP32 rounding. Where oracle/_ref is built (the build
container), fresh random cases are also run through the reference directly.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from tests.parity import rel_linf

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden.npz"


def _golden():
    g = np.load(GOLDEN)
    return g, json.loads(bytes(g["meta"]).decode())


def _conf(O, kw):
    kw = dict(kw)
    if "block_size" in kw:
        kw["block_size"] = tuple(kw["block_size"])
    return O.make_conf(**kw)


def _run(O, m, x, dtype):
    conf = _conf(O, m["conf"])
    if m["kind"] == "legacy":
        return O.legacy(x, conf, dtype=dtype, fill=0.0)
    return O.srrf_region(x, conf, dtype=dtype)


def test_fp32_port_reproduces_reference_bits(oracle_mod):
    g, meta = _golden()
    for m in meta:
        x = g[m["input"]].astype(np.float32)
        got = _run(oracle_mod, m, x, np.float32)
        ref = g["ref_" + m["name"]]
        assert np.array_equal(np.isnan(got), np.isnan(ref)), m["name"]
        fin = ~np.isnan(ref)
        assert np.array_equal(got[fin].view(np.uint32), ref[fin].view(np.uint32)), m["name"]


def test_fp64_oracle_agrees_with_reference(oracle_mod):
    g, meta = _golden()
    for m in meta:
        x = g[m["input"]].astype(np.float32)
        got = _run(oracle_mod, m, x, np.float64)
        ref = g["ref_" + m["name"]]
        assert np.array_equal(np.isnan(got), np.isnan(ref)), m["name"]
        # the reference's FP32 arithmetic (absolute magnified coordinates) is the error here
        assert rel_linf(ref, got) < 2e-5, m["name"]
        stored = g["oracle_" + m["name"]]
        assert rel_linf(stored, got) < 1e-6, m["name"]


def test_oracle_against_reference_build_random_cases(oracle_mod):
    if oracle_mod.ref_lib() is None:
        pytest.skip("oracle/_ref not built (reference sources absent)")
    rng = np.random.default_rng(3)
    cases = [(7, 8, 9, 10, 2, 3, 1, 2, 1), (9, 8, 8, 8, 2, 3, 1, 4, 1), (5, 7, 8, 9, 3, 1, 1, 2, 0),
             (6, 8, 8, 8, 2, 0, 1, 2, 1), (6, 8, 8, 8, 2, 2, 1, 2, 0), (11, 7, 7, 8, 2, 3, 1, 3, 1)]
    for (T, D, H, W, m, meth, itc, order, smooth) in cases:
        x = (rng.poisson(100, size=(T, D, H, W)) + 40 * rng.random((T, D, H, W))).astype(np.float32)
        c = oracle_mod.make_conf(mag=m, method=meth, itc=itc, trac_order=order, gradient_smooth=smooth,
                                 x_range=1, y_range=1, z_range=1)
        ref = oracle_mod.ref_block(x, c)
        got = oracle_mod.srrf_region(x, c, dtype=np.float32)
        assert np.array_equal(np.isnan(got), np.isnan(ref))
        fin = ~np.isnan(ref)
        assert np.array_equal(got[fin].view(np.uint32), ref[fin].view(np.uint32))


def _trac_known(rad, inten, order, itc):
    """Independent restatement of calculateACRF (kernel.cu:423-555) for one
    series, in Python floats."""
    rad = list(rad) + [0.0] * 8
    T = len(inten)
    mean = sum(rad[:T]) / T
    iw = sum(rad[t] * inten[t] for t in range(T)) / T
    acc = dict(ABCD=0.0, ABC=0.0, CD=0.0, AC=0.0, BD=0.0, AD=0.0, BC=0.0)

    def level(n):
        ab = 0.0
        for t in range(n - order):
            a, b = rad[t] - mean, rad[t + 1] - mean
            ab += a * b
            if order == 3:
                acc["ABC"] += a * b * (rad[t + 2] - mean)
            if order == 4:
                c, d = rad[t + 2] - mean, rad[t + 3] - mean
                acc["ABCD"] += a * b * c * d
                acc["CD"] += c * d
                acc["AC"] += a * c
                acc["BD"] += b * d
                acc["AD"] += a * d
                acc["BC"] += b * c
            if itc:
                v = 0.0
                if t * order < n:
                    for j in range(order):
                        src = t * order + j
                        v += (0.0 if src == t else rad[src]) / order
                rad[t] = v
        if order == 3:
            return abs(acc["ABC"])
        if order == 4:
            return abs(acc["ABCD"] - ab * acc["CD"] - acc["AC"] * acc["BD"] - acc["AD"] * acc["BC"])
        return abs(ab)

    if not itc:
        out = level(T) / T
    else:
        out, n = 0.0, T
        while n > order:
            out += level(n) / n
            n //= order
    return iw * out


def test_temporal_reductions_known_answers(oracle_mod):
    O = oracle_mod
    rad = [1.0, 2.0, 3.0, 4.0, 5.0, 6.0]
    one = [1.0] * 6
    # TRAC-2, ITC 0: AB over t < T-2 around mean 3.5 = 3.75 + 0.75 - 0.25 + 0.75 = 5; /T, x IW (3.5)
    assert O.temporal(O.make_conf(method=3, itc=0, trac_order=2), np.array(rad), np.array(one)) == pytest.approx(
        5.0 / 6 * 3.5)
    # TRA with intensity weighting
    inten = [2.0, 0.5, 1.0, 1.0, 0.0, 3.0]
    assert O.temporal(O.make_conf(method=1), np.array(rad), np.array(inten)) == pytest.approx(
        sum(r * i for r, i in zip(rad, inten)) / 6)
    # TRM seeded with 0: all negative gives 0
    assert O.temporal(O.make_conf(method=0, intensity_w=0), -np.array(rad), np.array(one)) == 0.0
    # TRPPM counts every pair once: ((sum r+)^2 + sum r+^2) / 2 / (T(T+1)/2), x mean I
    r = np.array([1.0, -2.0, 3.0])
    pos = np.maximum(r, 0)
    want = ((pos.sum() ** 2 + (pos ** 2).sum()) / 2) / 6 * np.mean([1.0, 1.0, 1.0])
    assert O.temporal(O.make_conf(method=2), r, np.ones(3)) == pytest.approx(want)
    # ITC=1 with its carry-over and binning quirks, several orders and lengths
    rng = np.random.default_rng(0)
    for order in (2, 3, 4):
        for T in (9, 12, 17, 30):
            rr = rng.normal(size=T)
            ii = rng.random(T)
            for itc in (0, 1):
                got = O.temporal(O.make_conf(method=3, itc=itc, trac_order=order), rr, ii)
                assert got == pytest.approx(_trac_known(rr, ii, order, itc), rel=1e-12, abs=1e-12)


def special_inputs():
    """Inputs at the edges of the domain, shared with the GPU tests: flat and
    all-zero series (every gradient 0, so every sample is the reference's
    0/0 = NaN), structure along one axis only (gradients exactly parallel to
    ring axes), and float series with NaN (and one with +Inf) voxels at least 3 voxels from
    every face (the reference's one-past-row read at the window edge can then
    never reach them). Returns [(name, x [T][D][H][W] float32, config)]."""
    rng = np.random.default_rng(17)
    smooth = dict(gradient_smooth=1, x_range=1, y_range=1, z_range=1)
    out = []
    out.append(("flat", np.full((4, 8, 9, 10), 100.0, np.float32), dict(mag=2, method=1, **smooth)))
    out.append(("zeros", np.zeros((3, 8, 8, 8), np.float32), dict(mag=3, method=3, itc=0, trac_order=2, **smooth)))
    xs = 100.0 + 30.0 * np.sin(0.7 * np.arange(12))
    ramp_x = np.broadcast_to(xs, (5, 8, 9, 12)).astype(np.float32).copy()
    ramp_x *= (1.0 + 0.1 * np.arange(5))[:, None, None, None].astype(np.float32)
    out.append(("along_x_tra", ramp_x, dict(mag=2, method=1, **smooth)))
    out.append(("along_x_trm_central", ramp_x, dict(mag=2, method=0, gradient_smooth=0)))
    zs = 80.0 + 25.0 * np.cos(0.9 * np.arange(9))
    ramp_z = np.broadcast_to(zs[None, :, None, None], (6, 9, 8, 10)).astype(np.float32).copy()
    ramp_z *= (1.0 + 0.05 * np.arange(6))[:, None, None, None].astype(np.float32)
    out.append(("along_z_trac2_m442", ramp_z, dict(mag=(4, 4, 2), method=3, itc=0, trac_order=2, **smooth)))
    x = (rng.poisson(100, size=(5, 10, 10, 11)) + 20 * rng.random((5, 10, 10, 11))).astype(np.float32)
    x[1, 4, 5, 6] = np.nan
    out.append(("nan_tra", x, dict(mag=2, method=1, **smooth)))
    out.append(("nan_trac2", x, dict(mag=2, method=3, itc=0, trac_order=2, **smooth)))
    out.append(("nan_trm_mag3", x, dict(mag=3, method=0, **smooth)))
    x = x.copy()
    x[3, 6, 3, 4] = np.inf
    out.append(("inf_tra", x, dict(mag=2, method=1, **smooth)))
    return out


@pytest.mark.parametrize("case", [c[0] for c in special_inputs()])
def test_oracle_special_inputs_against_reference_build(oracle_mod, case):
    """The FP32 port reproduces the reference build bit for bit, NaN masks
    included, on the special inputs."""
    if oracle_mod.ref_lib() is None:
        pytest.skip("oracle/_ref not built (reference sources absent)")
    name, x, kw = next(c for c in special_inputs() if c[0] == case)
    c = oracle_mod.make_conf(**kw)
    if len(set(np.atleast_1d(kw["mag"]).tolist())) != 1:
        pytest.skip("the reference has one magnification for all axes")
    ref = oracle_mod.ref_block(x, c)
    got = oracle_mod.srrf_region(x, c, dtype=np.float32)
    assert np.array_equal(np.isnan(got), np.isnan(ref)), name
    fin = ~np.isnan(ref)
    assert np.array_equal(got[fin].view(np.uint32), ref[fin].view(np.uint32)), name
    if name in ("flat", "zeros"):
        assert np.isnan(ref).all()
    if name.startswith(("nan", "inf")) and kw["method"] != 0:  # TRM's fmaxf drops NaN
        assert 0 < np.isnan(ref).mean() < 1
