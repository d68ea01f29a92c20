"""3B's model modification and fit loop on the GPU (rfba_3b_modify_model,
rfba_3b_fit; FitSpots::try_modifying_model and FitSpots::run,
RFBA Main/multispot5.cc:1840-2278).

The modification is a stochastic accept / reject between two models, so the
checks are behavioural on blocks whose answer is clear: a bright spot missing
from an empty model is added at the spot, a spurious spot in empty space is
removed while the real one stays, and the fit loop reports its steps in
order and stops when asked.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A = [[0.16, 0.84, 0.0], [0.495, 0.495, 0.01], [0.0, 0.0, 1.0]]
PI = [0.5, 0.5, 0.0]


@pytest.fixture(scope="module")
def ctx():
    from rfba_gb300 import srrf
    c = srrf.Context(0)
    yield c
    c.close()


def one_spot_block(seed, F=30, n=9, bright=40.0):
    """One bright blinking spot (blur 1) near the middle of an n^3 block, data
    normalised as 3B takes it (no background, unit noise): (data [F][P], pixels
    [P][3], the true centre)."""
    rng = np.random.default_rng(seed)
    zz, yy, xx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    pixels = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], 1).astype(np.int32)
    c = np.array([n / 2 - 0.3, n / 2 + 0.2, n / 2 - 0.6])
    d = pixels - c
    shape = bright / np.sqrt(2 * np.pi) * np.exp(-(d * d).sum(1) / 2)
    on = rng.random(F) < 0.6
    pix = on[:, None] * shape[None] + rng.normal(0, 1, (F, len(pixels)))
    return pix, pixels, c


def _model():
    from rfba_gb300 import srrf
    return srrf.ThreeBModel.make(A, PI, variance=1.0, z_factor=1.0, mu_brightness=3.5, sigma_brightness=1.0,
                                 mu_blur=0.0, sigma_blur=0.1)


def _params(**kw):
    from rfba_gb300 import srrf
    lim = 0.5 * np.array([np.sqrt((np.exp(1.0) - 1) * np.exp(2 * 3.5 + 1.0)), 1, 1, 1, 1])
    d = dict(main_passes=1, main_samples=6, opt_samples=8, opt_attempts=3, opt_hess_inner_samples=200,
             h_outer_samples=12, h_inner_samples=200, thermo_samples=200, add_remove_tries=2)
    d.update(kw)
    return srrf.ThreeBFitParams.make(lim, **d)


def test_empty_model_gains_the_spot(ctx):
    """A proposal placed near the spot converges onto it and is kept; one placed
    where there is no signal cannot be optimised (flat position curvature: the
    Hessian is not negative definite) or leaves the allowed area, and the
    original, empty model stays."""
    pix, pixels, c = one_spot_block(1)
    kept = 0
    for seed in range(6):
        got, rec = ctx.modify_model_3b(_model(), pix, pixels, np.zeros((0, 5)), _params(), seed=seed)
        print(f"[3B modify] add, seed {seed}: kept {rec['kept']}, bad Hessian {rec['bad_hessian']}, "
              f"spot {np.round(rec['spot'], 2)}, E2 - E1 {rec['model2_energy'] - rec['model1_energy']:.1f}")
        assert rec["added"] == 1 and rec["evaluations"] > 0
        if rec["kept"] == 2:
            kept += 1
            assert len(got) == 1 and rec["model2_energy"] > rec["model1_energy"]
            assert np.linalg.norm(got[0, 2:] - c) < 0.1 and abs(got[0, 1] - 1.0) < 0.05
        else:
            assert len(got) == 0 and (rec["bad_hessian"] == 1 or rec["zero_prior"] == 1)
    assert kept >= 1


def test_srrf_guided_proposals_land_on_the_spot(ctx):
    """add_guide = 1: a proposal's position is drawn from the SRRF map (GetPoint),
    so with the map peaked at the spot every proposal converges onto it and
    is kept, where uniform placement mostly missed it."""
    pix, pixels, c = one_spot_block(1)
    mag, n = 2, 9
    zz, yy, xx = np.meshgrid(np.arange(n * mag), np.arange(n * mag), np.arange(n * mag), indexing="ij")
    pos = np.stack([xx, yy, zz], -1) / mag
    guide = np.exp(-((pos - c) ** 2).sum(-1) / (2 * 0.4 ** 2)).astype(np.float32)
    for seed in range(4):
        got, rec = ctx.modify_model_3b(_model(), pix, pixels, np.zeros((0, 5)), _params(guide=guide, guide_mag=mag),
                                       seed=seed)
        print(f"[3B modify] guided, seed {seed}: kept {rec['kept']}, spot {np.round(rec['spot'], 2)}")
        assert rec["added"] == 1 and rec["kept"] == 2
        assert np.linalg.norm(got[0, 2:] - c) < 0.1


def test_extra_spot_on_an_explained_spot_is_rejected(ctx):
    """With the data's spot already in the model every proposal is an addition
    (one spot); one that converges (a negative definite Hessian) finds nothing
    the model lacks, and the free-energy comparison keeps the model as it was."""
    pix, pixels, c = one_spot_block(1)
    real = np.array([[39.74, 1.0, 4.19, 4.7, 3.9]])
    compared = 0
    for seed in range(12):
        got, rec = ctx.modify_model_3b(_model(), pix, pixels, real, _params(), seed=seed)
        assert rec["added"] == 1
        np.testing.assert_array_equal(got, real) if rec["kept"] == 1 else None
        if not rec["bad_hessian"] and not rec["zero_prior"]:
            compared += 1
            p2 = rec["model2_energy"] + rec["occam"] + rec["position_log_prior"]
            print(f"[3B modify] extra spot, seed {seed}: p2 - p1 {p2 - rec['model1_energy']:.2f}, "
                  f"mobile {np.round(rec['spot'], 2)}")
            assert rec["kept"] == 1 and p2 <= rec["model1_energy"]
        if compared >= 2:
            break
    assert compared >= 1


def test_removal_proposals_keep_the_data_explained(ctx):
    """Two spots on one: a removal proposal may keep either model, but no try
    leaves the data without a spot on it."""
    pix, pixels, c = one_spot_block(2)
    real = np.array([40.0, 1.0, *(c + 0.1)])
    dup = np.array([40.0, 1.0, *(c + [0.8, -0.3, 0.2])])
    removals = 0
    for seed in range(8):
        got, rec = ctx.modify_model_3b(_model(), pix, pixels, np.stack([real, dup]), _params(), seed=seed)
        print(f"[3B modify] duplicate, seed {seed}: added {rec['added']} kept {rec['kept']} -> {len(got)} spots")
        assert min(np.linalg.norm(s[2:] - c) for s in got) < 1.0
        removals += rec["added"] == 0
    assert removals >= 1


def test_fit_reports_steps_and_stops(ctx):
    pix, pixels, c = one_spot_block(4)
    start = np.array([[30.0, 1.1, *(c + [0.4, -0.3, 0.3])]])
    steps = []

    def progress(it, step, spots):
        steps.append((it, step, len(spots)))
        return False

    prm = _params(main_passes=2, add_remove_tries=2)
    got = ctx.fit_3b(_model(), pix, pixels, start, prm, iterations=2, seed=5, progress=progress)
    assert [s[:2] for s in steps] == [(0, 0), (0, 1), (0, 2), (0, 3), (1, 0), (1, 1), (1, 2), (1, 3)]
    assert min(np.linalg.norm(s[2:] - c) for s in got) < 0.2
    steps.clear()
    ctx.fit_3b(_model(), pix, pixels, got, prm, iterations=2, seed=5, progress=lambda *a: steps.append(a) or True)
    assert len(steps) == 1
