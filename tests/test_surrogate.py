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
