"""Failure detection without a GPU fault: the radiality kernel's bounded
input-staging wait is made to run out (RFBA_TEST_TMA_STALL=1 leaves out the
copy request the wait is for, so nothing completes it), the kernel records the
timeout in the context's status word and leaves, and the call reports
RFBA_ERR_TIMEOUT; the same context then computes the same map as before.
Each stalled call waits about two seconds (the wait's one-second limit, then a
bounded drain)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TIMEOUT = -5


def _series():
    from rfba_gb300 import synth
    # W = 16 u16 voxels: 32-byte rows, so the input is staged by TMA
    scene = synth.make_scene(21, 3, (16, 12, 10), 8)
    return synth.render(scene, (16, 12, 10), 21, np.uint16)


def test_staging_timeout_reported_and_context_recovers(monkeypatch):
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=2, method=1, gradient_smooth=1, x_range=1, y_range=1, z_range=1)
    x = _series()
    ctx = srrf.Context(0)
    try:
        good = ctx.forward(cfg, x)
        monkeypatch.setenv("RFBA_TEST_TMA_STALL", "1")
        with pytest.raises(srrf.RfbaError) as ei:
            ctx.forward(cfg, x)
        assert ei.value.status == TIMEOUT
        assert "bounded device wait" in str(ei.value)
        monkeypatch.delenv("RFBA_TEST_TMA_STALL")
        again = ctx.forward(cfg, x)
        assert np.array_equal(np.isnan(good), np.isnan(again))
        assert np.array_equal(np.nan_to_num(good), np.nan_to_num(again))
    finally:
        ctx.close()


def test_staging_timeout_on_device_pointers_reported_by_check(monkeypatch):
    import torch
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=2, method=3, itc=0, trac_order=2, gradient_smooth=1, x_range=1, y_range=1,
                           z_range=1)
    x = _series()
    ctx = srrf.Context(0)
    try:
        xd = torch.from_numpy(x.view(np.int16)).cuda()
        good = ctx.forward(cfg, xd)
        ctx.check()
        good = good.cpu().numpy()
        monkeypatch.setenv("RFBA_TEST_TMA_STALL", "1")
        ctx.forward(cfg, xd)  # asynchronous: returns before the kernel has run
        with pytest.raises(srrf.RfbaError) as ei:
            ctx.check()
        assert ei.value.status == TIMEOUT
        monkeypatch.delenv("RFBA_TEST_TMA_STALL")
        again = ctx.forward(cfg, xd)
        ctx.check()  # the failure was reported once; nothing new
        again = again.cpu().numpy()
        assert np.array_equal(np.isnan(good), np.isnan(again))
        assert np.array_equal(np.nan_to_num(good), np.nan_to_num(again))
    finally:
        ctx.close()
