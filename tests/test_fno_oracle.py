"""The surrogate network's double-precision oracle (oracle/fno_oracle.py)
against automatic differentiation of its FFT formulation (PyTorch, float64),
finite differences and torch.optim.Adam; the parameter layout and the bf16
rounding the kernels use."""
import numpy as np
import pytest
import torch

from oracle import fno_oracle as FO
from spatialpy_gb300 import fno as F
from tests import fno_torch_ref as TR

SHAPE = F.FnoShape(n=8, width=4, modes=2, layers=2, in_ch=3, out_ch=2, cond=3, hidden=5,
                   max_batch=4)


def _case(shape=SHAPE, B=3, shared=False, seed=1):
    rng = np.random.default_rng(seed)
    flat = F.init_params(shape, seed).astype(np.float64)
    P = F.unpack(shape, flat)
    for k in range(shape.layers):      # spectral weights large enough to matter
        P[f"spec_w{k}"] *= 8.0
    xs = (shape.in_ch, shape.n, shape.n) if shared else (B, shape.in_ch, shape.n, shape.n)
    x = rng.standard_normal(xs)
    cond = rng.uniform(-1, 1, (B, shape.cond))
    target = rng.standard_normal((B, shape.out_ch, shape.n, shape.n))
    return flat, P, x, cond, target


def test_layout_covers_every_parameter_once():
    lay = F.param_layout(SHAPE)
    total = lay.pop("_total")[0]
    spans = sorted((off, off + int(np.prod(shp))) for off, shp in lay.values())
    assert spans[0][0] == 0 and spans[-1][1] == total
    assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
    full = F.FnoShape(n=32)
    M = 2 * 12 * 12
    assert F.num_params(full) == (32 * 6 + 32 + 4 * (M * 32 * 32 * 2 + 32 * 32 + 32) + 64 * 6 + 64
                                  + 256 * 64 + 256 + 64 * 32 + 64 + 6 * 64 + 6)


@pytest.mark.parametrize("shared", [False, True])
def test_oracle_matches_autograd(shared):
    s = SHAPE
    flat, P, x, cond, target = _case(shared=shared)
    out, cache = FO.forward(P, x, cond, s.n, s.modes, s.layers)
    loss, dout = FO.mse(out, target)
    G = FO.backward(P, cache, dout, s.n, s.modes, s.layers)
    tl, tout, TG = TR.loss_and_grads(P, x, cond, target, s.n, s.modes, s.layers)
    np.testing.assert_allclose(out, tout, rtol=1e-11, atol=1e-12)
    assert abs(loss - tl) <= 1e-12 * abs(tl)
    for k, g in TG.items():
        scale = np.abs(g).max() + 1e-30
        assert np.abs(G[k] - g).max() <= 1e-10 * scale, k


def test_oracle_matches_finite_differences():
    s = SHAPE
    flat, P, x, cond, target = _case(B=2)
    out, cache = FO.forward(P, x, cond, s.n, s.modes, s.layers)
    _, dout = FO.mse(out, target)
    G = FO.backward(P, cache, dout, s.n, s.modes, s.layers)
    rng = np.random.default_rng(7)
    eps = 1e-6
    for name in ("spec_w0", "spec_w1", "lin_w1", "film1_w", "film2_b", "lift_w", "proj1_b"):
        arr = P[name].reshape(-1)
        for j in rng.choice(arr.size, 3, replace=False):
            old = arr[j]
            arr[j] = old + eps
            lp = FO.mse(FO.forward(P, x, cond, s.n, s.modes, s.layers)[0], target)[0]
            arr[j] = old - eps
            lm = FO.mse(FO.forward(P, x, cond, s.n, s.modes, s.layers)[0], target)[0]
            arr[j] = old
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - G[name].reshape(-1)[j]) <= 1e-6 * max(1.0, abs(fd)), (name, j)


def test_adam_matches_torch():
    rng = np.random.default_rng(3)
    p = rng.standard_normal(50)
    tp = torch.tensor(p.copy(), requires_grad=True)
    opt = torch.optim.Adam([tp], lr=2e-3)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    for t in range(1, 6):
        g = rng.standard_normal(50)
        tp.grad = torch.tensor(g)
        opt.step()
        p, m, v = FO.adam(p, g, m, v, t, 2e-3)
    np.testing.assert_allclose(p, tp.detach().numpy(), rtol=1e-12, atol=1e-14)


def test_bf16_rounding_is_nearest_even():
    rng = np.random.default_rng(4)
    a = np.concatenate([rng.standard_normal(1000).astype(np.float32) * 10.0 ** rng.integers(-8, 8, 1000),
                        np.float32([0.0, -0.0, 1.0, 1.00390625, 1.01171875, 65504.0])])
    want = torch.tensor(a).to(torch.bfloat16).float().numpy()
    np.testing.assert_array_equal(F.bf16_round(a), want)


def test_oracle_matches_autograd_at_the_sweep_shape():
    """The shape the surrogate sweep trains (32 x 32, width 32, 12 modes,
    4 layers), two samples, one input shared by the batch."""
    s = F.FnoShape(n=32, max_batch=2)
    flat, P, x, cond, target = _case(s, B=2, shared=True, seed=5)
    out, cache = FO.forward(P, x, cond, s.n, s.modes, s.layers)
    loss, dout = FO.mse(out, target)
    G = FO.backward(P, cache, dout, s.n, s.modes, s.layers)
    tl, tout, TG = TR.loss_and_grads(P, x, cond, target, s.n, s.modes, s.layers)
    np.testing.assert_allclose(out, tout, rtol=1e-10, atol=1e-12)
    for k, g in TG.items():
        assert np.abs(G[k] - g).max() <= 1e-9 * (np.abs(g).max() + 1e-30), k
