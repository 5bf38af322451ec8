"""The learned surrogate: CPU checks of the network's gradients (finite
differences in double precision) and of the coarse error metric."""
import numpy as np
import pytest

from spatialpy_gb300 import surrogate as SG


def test_fno_gradients_match_finite_differences():
    torch = pytest.importorskip("torch")
    torch.manual_seed(0)
    net = SG.build_fno(width=4, modes=2, layers=2, in_ch=3, out_ch=2, cond=2).double()
    x = torch.randn(2, 3, 8, 8, dtype=torch.float64, requires_grad=True)
    c = torch.randn(2, 2, dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(lambda a, b: net(a, b).sum(dim=(2, 3)), (x, c), eps=1e-6,
                                    atol=1e-5, rtol=1e-4)
    # and the parameters' gradients
    w = net.spec[0].w1
    loss = net(x, c).pow(2).mean()
    g, = torch.autograd.grad(loss, w)
    k = (1, 2, 1, 0, 1)
    with torch.no_grad():
        w[k] += 1e-6
        up = net(x, c).pow(2).mean()
        w[k] -= 2e-6
        dn = net(x, c).pow(2).mean()
        w[k] += 1e-6
    assert float(g[k]) == pytest.approx(float((up - dn) / 2e-6), rel=1e-4, abs=1e-8)


def test_coarse_error_metric():
    n, block = 16, 8
    rng = np.random.default_rng(1)
    ref = rng.uniform(1, 2, (3, 2, n * n, 3))
    assert np.all(SG.rel_error(ref, ref, n, block) == 0)
    noisy = ref * (1 + 0.5 * rng.standard_normal(ref.shape))
    # voxel noise averages out over 8 x 8 blocks
    assert np.all(SG.rel_error(noisy, ref, n, block) < 0.1)
    assert np.all(SG.rel_error(1.1 * ref, ref, n, block) == pytest.approx(0.1))
