"""The learned surrogate: CPU check of the coarse error metric (the
network's oracle is tested in test_fno_oracle.py)."""
import numpy as np
import pytest

from spatialpy_gb300 import surrogate as SG


def test_coarse_error_metric():
    n, block = 16, 8
    rng = np.random.default_rng(1)
    ref = rng.uniform(1, 2, (3, 2, n * n, 3))
    assert np.all(SG.rel_error(ref, ref, n, block) == 0)
    noisy = ref * (1 + 0.5 * rng.standard_normal(ref.shape))
    # voxel noise averages out over 8 x 8 blocks
    assert np.all(SG.rel_error(noisy, ref, n, block) < 0.1)
    assert np.all(SG.rel_error(1.1 * ref, ref, n, block) == pytest.approx(0.1))


class _FakeSurrogate:
    """Stands in for Surrogate.predict: two members around a given field."""

    def __init__(self, field, spread):
        self.cfg = SG.SweepConfig(n=8)
        self.field, self.spread = field, spread

    def predict(self, params):
        m = self.field
        self.last_members = [(m * (1 + s), m) for s in (self.spread, -self.spread)]
        return m, m, 0.01


def test_sweep_accounting_and_spread_gate():
    rng = np.random.default_rng(2)
    ref = rng.uniform(1, 2, (4, 2, 64, 3))
    pred = ref.copy()
    pred[1] *= 1.05                       # one point 5 % off in the mean and variance
    # members agree to 0.5 % -> the gate accepts every point, one of them wrongly
    s = SG.sweep(_FakeSurrogate(pred, 0.005), np.zeros((4, 5)), ref, ref, 10.0, block=8)
    assert s["accepted"] == 3
    assert s["surrogate_plus_fallback_s"] == pytest.approx(0.01 + 10.0 / 4)
    assert s["speedup"] == pytest.approx(10.0 / (0.01 + 2.5))
    assert s["gated_accepted"] == 4 and s["gated_within_threshold"] == 3
    # members disagree by 3 % -> the gate sends every point to the SSA
    s = SG.sweep(_FakeSurrogate(pred, 0.03), np.zeros((4, 5)), ref, ref, 10.0, block=8)
    assert s["gated_accepted"] == 0
    assert s["gated_seconds"] == pytest.approx(10.01)
