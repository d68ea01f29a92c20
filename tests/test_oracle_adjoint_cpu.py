"""The oracle's FP64 adjoint (oracle.adjoint) against central differences of
the oracle's own FP64 forward, on the CPU: the reference the GPU backward is
checked against is itself checked here, before any GPU is involved.

Objective L = -||map||_2 over the finite voxels (dL/dmap = -map/||map||).
Inputs are float32, so an input step is the exact difference of the two
perturbed float32 values; shifts are FP64.
"""
import numpy as np
import pytest

SHIPPED = dict(gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)


def _objective(m):
    f = np.where(np.isfinite(m), m, 0.0)
    return -np.sqrt(np.sum(f * f))


def _gmap(m):
    f = np.where(np.isfinite(m), m, 0.0)
    return np.where(np.isfinite(m), -f / np.sqrt(np.sum(f * f)), 0.0)


CASES = [
    ("tra_iw", dict(mag=2, method=1, **SHIPPED), (5, 8, 8, 9)),
    ("trac2", dict(mag=2, method=3, itc=0, trac_order=2, **SHIPPED), (6, 8, 9, 8)),
    ("trac3_aniso", dict(mag=(2, 2, 1), method=3, itc=0, trac_order=3, gradient_smooth=0), (6, 8, 8, 9)),
    ("trac4_renorm", dict(mag=2, method=3, itc=0, trac_order=4, renormalize=1, **SHIPPED), (7, 8, 8, 8)),
    ("tra_no_iw_mag3", dict(mag=3, method=1, intensity_w=0, **SHIPPED), (5, 7, 7, 8)),
    ("trm_iw", dict(mag=2, method=0, **SHIPPED), (5, 8, 8, 9)),
    ("trppm_iw", dict(mag=2, method=2, **SHIPPED), (6, 8, 9, 8)),
    ("trppm_no_iw_poscon", dict(mag=2, method=2, intensity_w=0, remove_con=1, **SHIPPED), (5, 8, 8, 8)),
    ("trac2_itc1", dict(mag=2, method=3, itc=1, trac_order=2, **SHIPPED), (11, 8, 8, 8)),
    ("trac3_itc1_no_iw", dict(mag=2, method=3, itc=1, trac_order=3, intensity_w=0, **SHIPPED), (13, 8, 8, 8)),
    ("trac4_itc1", dict(mag=2, method=3, itc=1, trac_order=4, **SHIPPED), (21, 7, 7, 8)),
]


@pytest.mark.parametrize("name,kw,shape", CASES, ids=[c[0] for c in CASES])
def test_oracle_adjoint_matches_central_differences(oracle_mod, name, kw, shape):
    from rfba_gb300 import synth
    O = oracle_mod
    oc = O.make_conf(**kw)
    T, D, H, W = shape
    scene = synth.make_scene(40 + len(name), T, (W, H, D), 8)
    x = synth.render(scene, (W, H, D), 40 + len(name), np.float32)
    sh = np.random.default_rng(len(name)).normal(0, 0.2, size=(T, 3))
    m = O.forward_shifted(x, oc, sh)
    assert np.isfinite(m).any()
    _, din, dsh = O.adjoint(x, oc, _gmap(m), sh)
    rng = np.random.default_rng(1)
    idx = np.argwhere(np.abs(din) > 1e-3 * np.abs(din).max())
    pick = idx[rng.choice(len(idx), size=min(25, len(idx)), replace=False)]
    fd, an = [], []
    for (t, z, y, xx) in pick:
        xp, xm = x.copy(), x.copy()
        h = max(1e-2, 1e-4 * abs(float(x[t, z, y, xx])))
        xp[t, z, y, xx] += h
        xm[t, z, y, xx] -= h
        step = float(xp[t, z, y, xx]) - float(xm[t, z, y, xx])
        fd.append((_objective(O.forward_shifted(xp, oc, sh)) - _objective(O.forward_shifted(xm, oc, sh))) / step)
        an.append(din[t, z, y, xx])
    for t in range(T):
        for a in range(3):
            sp, sm = sh.copy(), sh.copy()
            sp[t, a] += 1e-4
            sm[t, a] -= 1e-4
            fd.append((_objective(O.forward_shifted(x, oc, sp)) - _objective(O.forward_shifted(x, oc, sm))) / 2e-4)
            an.append(dsh[t, a])
    fd, an = np.array(fd), np.array(an)
    scale = np.abs(fd).max()
    err = np.abs(fd - an) / scale
    print(f"[oracle adjoint] {name}: max |fd - adjoint| / max|fd| = {err.max():.2e}")
    assert err.max() < 1e-3, (name, err.max())
    assert np.median(np.abs(fd - an) / np.maximum(np.abs(fd), 1e-12 * scale)) < 1e-4, name
