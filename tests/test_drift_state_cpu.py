"""Drift-refinement state file (CPU): save/load round trip, atomic replace."""
import numpy as np

from rfba_gb300.drift import DriftState


def test_state_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    st = DriftState(rng.normal(size=(7, 3)).astype(np.float32), rng.normal(size=(7, 3)).astype(np.float32),
                    rng.random((7, 3)).astype(np.float32), 5)
    p = tmp_path / "drift.npz"
    st.save(p)
    back = DriftState.load(p)
    assert back.it == 5
    for a in ("shifts", "m", "v"):
        assert np.array_equal(getattr(back, a), getattr(st, a))
    # a second save replaces the file whole and leaves no temporary behind
    st.it = 6
    st.save(p)
    assert DriftState.load(p).it == 6
    assert sorted(q.name for q in tmp_path.iterdir()) == ["drift.npz"]


def test_objective_gradients_match_autograd():
    """make_objective's closed-form dL/dmap equals torch autograd of its value,
    with zeros on NaN voxels and in the left-out border."""
    import pytest
    torch = pytest.importorskip("torch")
    from rfba_gb300 import drift
    g = torch.Generator().manual_seed(3)
    m = torch.randn((10, 12, 14), generator=g)
    m[4, 5, 6] = float("nan")
    for kind, border in [("l2", 0), ("l2", 2), ("lp", 0), ("lp", 3), ("kurtosis", 0), ("kurtosis", 2)]:
        value, grad = drift.make_objective(kind, 8.0, border)
        got = grad(m).double()
        leaf = torch.nan_to_num(m).double().requires_grad_(True)
        value(torch.where(torch.isnan(m), torch.full_like(leaf, float("nan")), leaf)).backward()
        want = torch.where(torch.isnan(m), torch.zeros_like(got), leaf.grad)
        assert float((got - want).abs().max()) <= 1e-6 * float(want.abs().max()), (kind, border)
        assert float(got[4, 5, 6]) == 0.0
        if border:
            assert float(got[:border].abs().max()) == 0.0 and float(got[..., -border:].abs().max()) == 0.0
    value, grad = drift.make_objective("l2")
    assert float(value(m)) == float(drift.objective(m))
    assert float((grad(m) - drift.grad_map(m)).abs().max()) <= 1e-6
