"""CPU: checkpoint format of the phase optimiser (phi, Adam moments, step)."""
import numpy as np

from openol_gb300.optim import load_state, make_targets, save_state


def test_state_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    sd = {"phi": rng.random((16, 16)).astype(np.float32), "m": rng.random((16, 16)).astype(np.float32),
          "v": rng.random((16, 16)).astype(np.float32), "t": np.int64(17)}
    save_state(tmp_path / "s.npz", sd)
    back = load_state(tmp_path / "s.npz")
    for k in sd:
        assert np.array_equal(back[k], sd[k])


def test_targets_are_seeded_and_sparse():
    a = make_targets(128, 128, 3, seed=4)
    b = make_targets(128, 128, 3, seed=4)
    assert np.array_equal(a, b)
    frac = np.count_nonzero(a) / a.size
    assert 0.04 < frac < 0.06
    assert a.max() <= 1.0 and a.min() >= 0.0
