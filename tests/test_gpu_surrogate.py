"""The learned surrogate on the GPU: trained on SSA ensembles from the
engine, it must predict held-out parameter points better than the
parameter-blind baseline (the training-set average), and a sweep answered by
surrogate + SSA fallback must be faster than the plain SSA sweep."""
import numpy as np
import pytest

from spatialpy_gb300 import surrogate as SG

pytestmark = pytest.mark.gpu


def test_surrogate_learns_and_speeds_up_a_sweep():
    pytest.importorskip("torch")
    cfg = SG.SweepConfig(n=16, molecules=300, t_end=2.0, num_times=4, trajectories=16)
    rng = np.random.default_rng(7)
    train_p = SG.sample_parameters(64, rng)
    test_p = SG.sample_parameters(16, rng)
    tm, tv, _ = SG.ssa_moments(train_p, cfg, seed0=10)
    hm, hv, ssa_s = SG.ssa_moments(test_p, cfg, seed0=100000)
    sur = SG.Surrogate(cfg, width=32, modes=6, layers=4)
    loss = sur.fit(train_p, tm, tv, epochs=200)
    pm, pv, _ = sur.predict(test_p)
    err = SG.rel_error(pm, hm, cfg.n, 8)
    base = SG.rel_error(np.broadcast_to(tm.mean(0), hm.shape), hm, cfg.n, 8)
    assert np.median(err) < 0.5 * np.median(base), (err, base, loss)
    summary = SG.sweep(sur, test_p, hm, hv, ssa_s, threshold=0.10)
    assert summary["inference_s"] < ssa_s
    assert summary["surrogate_plus_fallback_s"] <= ssa_s
