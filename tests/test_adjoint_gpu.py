"""The CUDA adjoint (rfba_srrf_forward_shifted / rfba_srrf_backward) against
the FP64 CPU adjoint of the oracle and against FP64 central differences.

Objective L = -||map||_2 over the finite map voxels, so dL/dmap = -map/||map||.
"""
import numpy as np
import pytest

from tests.parity import assert_parity, rel_linf

pytestmark = pytest.mark.gpu

SHIPPED = dict(gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)


def _objective(m):
    f = np.where(np.isfinite(m), m, 0.0).astype(np.float64)
    return -np.sqrt(np.sum(f * f))


def _gmap(m):
    f = np.where(np.isfinite(m), m, 0.0).astype(np.float64)
    return np.where(np.isfinite(m), -f / np.sqrt(np.sum(f * f)), 0.0)


def _case(seed, T, D, H, W, drift=0.3):
    from rfba_gb300 import synth
    scene = synth.make_scene(seed, T, (W, H, D), 10)
    x = synth.render(scene, (W, H, D), seed, np.float32)
    sh = np.random.default_rng(seed).normal(0, drift, size=(T, 3)).astype(np.float32)
    return x, sh


def _gpu(ctx, cfg, x, sh):
    import torch
    xd = torch.from_numpy(x).cuda()
    sd = torch.from_numpy(sh).cuda() if sh is not None else None
    m = ctx.forward_shifted(cfg, xd, sd)
    torch.cuda.synchronize()
    mh = m.cpu().numpy()
    g = torch.from_numpy(_gmap(mh).astype(np.float32)).cuda()
    din, dsh = ctx.backward(cfg, xd, sd, g)
    torch.cuda.synchronize()
    return mh, din.cpu().numpy(), (dsh.cpu().numpy() if dsh is not None else None)


CASES = [
    ("trac2_iw_drift", dict(mag=2, method=3, itc=0, trac_order=2, **SHIPPED), (7, 9, 10, 11), True),
    ("tra_iw_drift", dict(mag=2, method=1, **SHIPPED), (6, 9, 9, 10), True),
    ("trac4_renorm", dict(mag=2, method=3, itc=0, trac_order=4, renormalize=1, **SHIPPED), (9, 8, 9, 9), True),
    ("trac3_mag3_nodrift_poscon", dict(mag=3, method=3, itc=0, trac_order=3, remove_con=1, **SHIPPED), (7, 7, 8, 8),
     False),
    ("trac2_aniso_nosmooth", dict(mag=(2, 2, 1), method=3, itc=0, trac_order=2), (8, 9, 9, 10), True),
    ("trac2_mag442_deep_tiles", dict(mag=(4, 4, 2), method=3, itc=0, trac_order=2, **SHIPPED), (5, 9, 7, 8), True),
    ("trm_iw_drift", dict(mag=2, method=0, **SHIPPED), (6, 9, 9, 10), True),
    ("trppm_iw_drift", dict(mag=2, method=2, **SHIPPED), (7, 9, 10, 9), True),
    ("trppm_no_iw_renorm", dict(mag=(2, 2, 1), method=2, intensity_w=0, renormalize=1, **SHIPPED), (6, 8, 9, 9),
     False),
    ("trac2_itc1_shipped_drift", dict(mag=2, method=3, itc=1, trac_order=2, **SHIPPED), (13, 9, 9, 10), True),
    ("trac3_itc1_no_iw", dict(mag=2, method=3, itc=1, trac_order=3, intensity_w=0, **SHIPPED), (14, 8, 9, 9), True),
    ("trac4_itc1_mag442", dict(mag=(4, 4, 2), method=3, itc=1, trac_order=4, **SHIPPED), (21, 7, 7, 8), False),
]


@pytest.mark.parametrize("name,kw,shape,drift", CASES, ids=[c[0] for c in CASES])
def test_adjoint_matches_fp64_adjoint(ctx, oracle_mod, name, kw, shape, drift):
    from rfba_gb300 import srrf
    O = oracle_mod
    cfg = srrf.Config.make(**kw)
    oc = O.make_conf(**kw)
    x, sh = _case(11 + len(name), *shape)
    if not drift:
        sh = None
    m, din, dsh = _gpu(ctx, cfg, x, sh)
    mo = O.forward_shifted(x, oc, sh)
    assert_parity(m, mo, 1e-4, name + " forward")
    _, din_o, dsh_o = O.adjoint(x, oc, _gmap(mo), sh)
    e_in = rel_linf(din, din_o)
    msg = f"[adjoint] {name}: dL/dI rel L-inf {e_in:.2e}"
    assert e_in < 2e-4, msg
    if drift:
        e_sh = rel_linf(dsh, dsh_o)
        msg += f", dL/dshift rel L-inf {e_sh:.2e}"
        assert e_sh < 2e-4, msg
    print(msg)


def test_adjoint_against_central_differences(ctx, oracle_mod):
    """h = 1e-3 central differences of the FP64 forward at 200 random input
    voxels and every shift."""
    from rfba_gb300 import srrf
    O = oracle_mod
    kw = dict(mag=2, method=3, itc=0, trac_order=2, **SHIPPED)
    cfg = srrf.Config.make(**kw)
    oc = O.make_conf(**kw)
    x, sh = _case(5, 6, 8, 9, 10, drift=0.15)
    _, din, dsh = _gpu(ctx, cfg, x, sh)
    rng = np.random.default_rng(0)
    T, D, H, W = x.shape
    # voxels inside the volume whose gradient is not negligible
    idx = np.argwhere(np.abs(din) > 1e-3 * np.abs(din).max())
    pick = idx[rng.choice(len(idx), size=min(200, len(idx)), replace=False)]
    h = 1e-3
    fd, an = [], []
    for (t, z, y, xx) in pick:
        xp = x.copy()
        xm = x.copy()
        xp[t, z, y, xx] += h
        xm[t, z, y, xx] -= h
        step = float(xp[t, z, y, xx]) - float(xm[t, z, y, xx])
        fd.append((_objective(O.forward_shifted(xp, oc, sh)) - _objective(O.forward_shifted(xm, oc, sh))) / step)
        an.append(din[t, z, y, xx])
    for t in range(T):
        for a in range(3):
            sp = sh.astype(np.float64).copy()
            sm = sh.astype(np.float64).copy()
            sp[t, a] += h
            sm[t, a] -= h
            fd.append((_objective(O.forward_shifted(x, oc, sp)) - _objective(O.forward_shifted(x, oc, sm))) / (2 * h))
            an.append(dsh[t, a])
    fd, an = np.array(fd), np.array(an)
    scale = np.abs(fd).max()
    err = np.abs(fd - an) / scale
    print(f"[adjoint] central differences: {len(fd)} points, max |fd - adjoint| / max|fd| = {err.max():.2e}")
    assert err.max() < 5e-3
    assert np.median(np.abs(fd - an) / np.maximum(np.abs(fd), 1e-12 * scale)) < 1e-2


def test_backward_in_slices_matches_resident(ctx, oracle_mod):
    """With a scratch budget too small for the whole radiality stack, the
    forward runs in z slices and the backward recomputes each slice's stacks
    before its adjoint; the gradients equal the single-slice ones (up to the
    order of the float atomics that add the tiles' contributions)."""
    import torch
    from rfba_gb300 import srrf
    kw = dict(mag=2, method=3, itc=0, trac_order=2, **SHIPPED)
    cfg = srrf.Config.make(**kw)
    x, sh = _case(23, 6, 12, 10, 9, drift=0.2)
    m, din, dsh = _gpu(ctx, cfg, x, sh)
    small = srrf.Context(0, 6 * 20 * 18 * 8 * 4 * 2)   # about one 4-row z slab of the 24-deep map
    try:
        m2, din2, dsh2 = _gpu(small, cfg, x, sh)
    finally:
        small.close()
    assert np.array_equal(np.isnan(m), np.isnan(m2)) and np.allclose(np.nan_to_num(m), np.nan_to_num(m2), rtol=0,
                                                                      atol=0)
    assert rel_linf(din2, din) < 1e-5
    assert rel_linf(dsh2, dsh) < 1e-5


def test_backward_after_time_batched_forward(ctx):
    """A drift-corrected TRA forward whose series runs in time batches in one
    spatial pass keeps only its last batch's stacks: the backward must not
    reuse them, it recomputes the stacks (in z slices) and gives the gradients
    of the resident path (to the order of the float atomics)."""
    import torch
    from rfba_gb300 import srrf
    kw = dict(mag=2, method=1, intensity_w=1, **SHIPPED)
    cfg = srrf.Config.make(**kw)
    T, D, H, W = 60, 8, 9, 10
    x, sh = _case(29, T, D, H, W, drift=0.2)
    m, din, dsh = _gpu(ctx, cfg, x, sh)
    vox = D * H * W * 8
    budget = vox * (25 * 8 + 2 * 4) + 4096   # one batch of 25 plus the TRA state, not all 60 volumes
    assert budget < vox * T * 8
    small = srrf.Context(0, budget)
    try:
        xd = torch.from_numpy(x).cuda()
        sd = torch.from_numpy(sh).cuda()
        m2 = small.forward_shifted(cfg, xd, sd)
        torch.cuda.synchronize()
        assert small.last_time_batches() == (25, 3) and small.last_passes() == 1
        m2 = m2.cpu().numpy()
        g = torch.from_numpy(_gmap(m2).astype(np.float32)).cuda()
        din2, dsh2 = small.backward(cfg, xd, sd, g)
        torch.cuda.synchronize()
        din2, dsh2 = din2.cpu().numpy(), dsh2.cpu().numpy()
    finally:
        small.close()
    assert np.array_equal(np.isnan(m), np.isnan(m2))
    assert rel_linf(m2, m) < 1e-5
    assert rel_linf(din2, din) < 1e-4
    assert rel_linf(dsh2, dsh) < 1e-4


def test_automatic_batches_keep_the_state_for_the_backward(ctx):
    """TRAC with ITC 0 on a series whose stacks exceed the budget: the drift-
    corrected forward runs in batches of 25 volumes in the z slices the backward
    will use and keeps every slice's carried state; the backward that follows
    reuses it (batched, no state pass) and gives the resident path's gradients."""
    import torch
    from rfba_gb300 import srrf
    kw = dict(mag=2, method=3, itc=0, trac_order=2, intensity_w=1, **SHIPPED)
    cfg = srrf.Config.make(**kw)
    T, D, H, W = 60, 8, 9, 10
    x, sh = _case(30, T, D, H, W, drift=0.2)
    m, din, dsh = _gpu(ctx, cfg, x, sh)
    vox = D * H * W * 8
    budget = vox * 300
    assert budget < vox * T * 8
    small = srrf.Context(0, budget)
    try:
        xd = torch.from_numpy(x).cuda()
        sd = torch.from_numpy(sh).cuda()
        m2 = small.forward_shifted(cfg, xd, sd)
        torch.cuda.synchronize()
        assert small.last_time_batches() == (25, 3)
        m2 = m2.cpu().numpy()
        g = torch.from_numpy(_gmap(m2).astype(np.float32)).cuda()
        din2, dsh2 = small.backward(cfg, xd, sd, g)
        torch.cuda.synchronize()
        din2, dsh2 = din2.cpu().numpy(), dsh2.cpu().numpy()
    finally:
        small.close()
    assert np.array_equal(np.isnan(m), np.isnan(m2))
    assert rel_linf(m2, m) < 1e-5
    assert rel_linf(din2, din) < 1e-4
    assert rel_linf(dsh2, dsh) < 1e-4


def _random_adjoint_case(i):
    rng = np.random.default_rng(3000 + i)
    mag = tuple(int(v) for v in rng.integers(1, 5, size=3))
    method = int(rng.choice([1, 3]))
    kw = dict(mag=mag, method=method, itc=0, trac_order=int(rng.integers(2, 5)),
              gradient_smooth=int(rng.integers(0, 2)), main_range=1, x_range=int(rng.integers(0, 2)),
              y_range=int(rng.integers(0, 2)), z_range=int(rng.integers(0, 2)),
              axes_in_ring=int(rng.integers(3, 7)), ring_radius=float(rng.choice([0.4, 0.5, 0.7])),
              renormalize=int(rng.integers(0, 2)), remove_con=int(rng.integers(0, 2)),
              intensity_w=int(rng.integers(0, 2)))
    kw["ring_radius"] = min(kw["ring_radius"], 0.45 * (1 + min(mag)))
    shape = (int(rng.integers(5, 9)),) + tuple(int(v) for v in rng.integers(7, 11, size=3))
    return kw, shape


@pytest.mark.parametrize("i", range(8))
def test_random_adjoint_matches_fp64_adjoint(ctx, oracle_mod, i):
    """Seeded random configurations (per-axis magnification 1-4, TRA or TRAC-2/3/4,
    ranges, smoothing, ring, renormalisation, positivity, intensity weighting),
    with drift, against the oracle's FP64 adjoint."""
    from rfba_gb300 import srrf
    O = oracle_mod
    kw, shape = _random_adjoint_case(i)
    cfg = srrf.Config.make(**kw)
    oc = O.make_conf(**kw)
    x, sh = _case(500 + i, *shape, drift=0.25)
    m, din, dsh = _gpu(ctx, cfg, x, sh)
    mo = O.forward_shifted(x, oc, sh)
    assert_parity(m, mo, 1e-4, f"random {i} forward")
    if not np.isfinite(mo).any():
        pytest.skip("volume smaller than the interpolation window at this magnification")
    _, din_o, dsh_o = O.adjoint(x, oc, _gmap(mo), sh)
    e_in, e_sh = rel_linf(din, din_o), rel_linf(dsh, dsh_o)
    msg = f"[adjoint] random {i} {kw} {shape}: dL/dI {e_in:.2e}, dL/dshift {e_sh:.2e}"
    assert e_in < 2e-4 and e_sh < 2e-4, msg
    print(msg)
