"""3B spot gradient on the GPU (rfba_3b_spot_gradient) against the FP64 oracle
(pinned to the reference's headers in tests/test_threeb_cpu.py). Both compute
in FP64; the GPU sums each frame's voxels in a tree instead of in sequence and
uses CUDA's exp/log, so the gradient agrees to 1e-9 of its largest component
and every sample's log probability to 1e-12 (relative)."""
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
