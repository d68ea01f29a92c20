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
