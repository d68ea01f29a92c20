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


@pytest.mark.parametrize("kind,p", [("lp", 8.0), ("kurtosis", 4.0)])
def test_refinement_with_other_objectives(ctx, kind, p):
    """refine_drift minimises whichever objective's gradient it is given: with
    make_objective's peak-weighted and scale-free objectives (border left out)
    the objective after a few steps is below its start."""
    import torch
    from rfba_gb300 import drift, srrf, synth
    scene = synth.make_scene(33, 6, (16, 15, 14), 14, drift_sigma=0.2)
    x = synth.render(scene, (16, 15, 14), 33, np.float32)
    cfg = srrf.Config.make(mag=2, method=3, itc=0, trac_order=2, gradient_smooth=1, x_range=1, y_range=1,
                           z_range=1)
    xd = torch.from_numpy(x).cuda()
    value, grad = drift.make_objective(kind, p, border=4)
    start = np.full((6, 3), 0.5, np.float32)
    L0 = float(value(ctx.forward_shifted(cfg, xd, torch.from_numpy(start).cuda())))
    st, m = drift.refine_drift(ctx, cfg, xd, 5, start=start, lr=0.01, grad_fn=grad)
    torch.cuda.synchronize()
    assert st.it == 5 and np.isfinite(st.shifts).all()
    assert float(value(m)) < L0
