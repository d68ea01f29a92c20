"""Drift refinement driver (rfba_gb300.drift) on the GPU: a run interrupted
after two iterations and resumed from its checkpoint ends where an
uninterrupted run ends, and the objective improves. The adjoint's scatter adds
in float atomics, so the two runs agree to rounding, not bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_resume_from_checkpoint_matches_uninterrupted(ctx, tmp_path):
    import torch
    from rfba_gb300 import drift, srrf, synth
    scene = synth.make_scene(31, 6, (14, 13, 12), 12, drift_sigma=0.2)
    x = synth.render(scene, (14, 13, 12), 31, np.float32)
    cfg = srrf.Config.make(mag=2, method=3, itc=0, trac_order=2, gradient_smooth=1, x_range=1, y_range=1,
                           z_range=1)
    xd = torch.from_numpy(x).cuda()
    start = np.full((6, 3), 0.5, np.float32)
    full, m_full = drift.refine_drift(ctx, cfg, xd, 4, start=start)
    ck = tmp_path / "drift.npz"
    part, _ = drift.refine_drift(ctx, cfg, xd, 2, start=start, checkpoint=ck)
    assert drift.DriftState.load(ck).it == 2
    rest, m_rest = drift.refine_drift(ctx, cfg, xd, 4, start=start, checkpoint=ck, resume=True)
    torch.cuda.synchronize()
    assert rest.it == 4 and drift.DriftState.load(ck).it == 4
    assert np.allclose(rest.shifts, full.shifts, rtol=0, atol=1e-4)
    L0 = float(drift.objective(ctx.forward_shifted(cfg, xd, torch.from_numpy(start).cuda())))
    assert float(drift.objective(m_rest)) < L0
    assert abs(float(drift.objective(m_rest)) - float(drift.objective(m_full))) <= 1e-4 * abs(L0)
