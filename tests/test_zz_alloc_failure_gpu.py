"""Injected allocation failure through the C-ABI on a GPU.

RFBA_TEST_ALLOC_FAIL=k makes the context's k-th scratch allocation after the
variable is set fail as an out-of-memory would (rfba_gb300/csrc/devbuf.h). For
every k that a call reaches, the call must return RFBA_ERR_NOMEM with the
buffer's name in rfba_last_error, and the next call on the same context, with
the variable cleared, must succeed and give the map (or gradients) of a context
that never failed. Collected after the other GPU tests (only the
static-scratch test comes later), so a run stopping at the first failure has
run them first.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _series(seed, T, D, H, W, dtype=np.uint16):
    from rfba_gb300 import synth
    scene = synth.make_scene(seed, T, (W, H, D), 12)
    return synth.render(scene, (W, H, D), seed, dtype)


def _inject(monkeypatch, k, call):
    """Run call() with the k-th allocation failing; the error, or None when the
    call made fewer than k allocations."""
    from rfba_gb300 import srrf
    monkeypatch.setenv("RFBA_TEST_ALLOC_FAIL", str(k))
    try:
        call()
        return None
    except srrf.RfbaError as e:
        return e
    finally:
        monkeypatch.delenv("RFBA_TEST_ALLOC_FAIL")


def test_forward_reports_nomem_and_recovers(monkeypatch):
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=(2, 2, 2), method=3, itc=0, trac_order=2, gradient_smooth=1, x_range=1, y_range=1,
                           z_range=1)
    x = _series(41, 10, 9, 12, 14)
    clean = srrf.Context(0)
    try:
        ref = clean.forward(cfg, x)
    finally:
        clean.close()
    names = []
    for k in range(1, 40):
        ctx = srrf.Context(0)  # created before the variable is set: its own allocations are not counted
        try:
            err = _inject(monkeypatch, k, lambda: ctx.forward(cfg, x))
            if err is None:
                break
            assert err.status == -3, str(err)
            assert "RFBA_TEST_ALLOC_FAIL" in str(err)
            names.append(str(err).split("): ", 1)[1].split(":", 1)[0])
            got = ctx.forward(cfg, x)  # same context, variable cleared
            np.testing.assert_array_equal(got, ref)
        finally:
            ctx.close()
    assert len(set(names)) >= 3, names  # several distinct scratch buffers were made to fail


def test_backward_reports_nomem_and_recovers(monkeypatch):
    import torch
    from rfba_gb300 import srrf
    torch.cuda.set_device(0)
    cfg = srrf.Config.make(mag=2, method=3, itc=0, trac_order=2, gradient_smooth=1, x_range=1, y_range=1, z_range=1)
    x = torch.from_numpy(_series(43, 6, 10, 10, 10, np.float32)).cuda()
    shifts = (torch.rand((6, 3), generator=torch.Generator().manual_seed(5)) * 0.4 - 0.2).cuda()

    def run(ctx):
        m = ctx.forward_shifted(cfg, x, shifts)
        g = torch.nan_to_num(m, nan=0.0)
        din, dsh = ctx.backward(cfg, x, shifts, g)
        torch.cuda.synchronize()
        return m.cpu().numpy(), din.cpu().numpy(), dsh.cpu().numpy()

    clean = srrf.Context(0)
    try:
        ref = run(clean)
    finally:
        clean.close()
    failures = 0
    for k in range(1, 60):
        ctx = srrf.Context(0)
        try:
            err = _inject(monkeypatch, k, lambda: run(ctx))
            if err is None:
                break
            assert err.status == -3, str(err)
            failures += 1
            got = run(ctx)
            np.testing.assert_array_equal(got[0], ref[0])
            for a, b in zip(got[1:], ref[1:]):  # float atomics in the adjoint: equal to rounding
                scale = max(float(np.abs(b).max()), 1e-30)
                assert float(np.abs(a - b).max()) <= 1e-5 * scale
        finally:
            ctx.close()
    assert failures >= 3
