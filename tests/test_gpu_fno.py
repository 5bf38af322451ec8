"""The surrogate network's kernels (csrc/fno.cu through the sp_fno_* C ABI)
against the double-precision oracle (oracle/fno_oracle.py): forward values,
every parameter's gradient, the Adam step, the graph-replayed training step,
and training on a small problem.

The kernels compute with bf16 weights and fp32 arithmetic; the oracle is fed
the same bf16-rounded weights and computes in float64.  Tolerances: forward
outputs within 2e-4 of the output's largest magnitude; each gradient tensor
within 2e-3 of its largest magnitude; Adam within 1e-6 relative."""
import numpy as np
import pytest

from oracle import fno_oracle as FO
from spatialpy_gb300 import fno as F

pytestmark = pytest.mark.gpu

SMALL = F.FnoShape(n=16, width=8, modes=4, layers=2, in_ch=3, out_ch=2, cond=3, hidden=16,
                   max_batch=8)
FULL = F.FnoShape(n=32, width=32, modes=12, layers=4, in_ch=6, out_ch=6, cond=6, hidden=64,
                  max_batch=8)


def _torch():
    return pytest.importorskip("torch")


def _case(shape, B, shared, seed=1):
    rng = np.random.default_rng(seed)
    flat = F.init_params(shape, seed)
    P = F.unpack(shape, flat)
    for k in range(shape.layers):
        P[f"spec_w{k}"] *= 8.0
    xs = (shape.in_ch, shape.n, shape.n) if shared else (B, shape.in_ch, shape.n, shape.n)
    x = rng.standard_normal(xs).astype(np.float32)
    cond = rng.uniform(-1, 1, (B, shape.cond)).astype(np.float32)
    target = rng.standard_normal((B, shape.out_ch, shape.n, shape.n)).astype(np.float32)
    return flat, x, cond, target


def _oracle(shape, flat, x, cond, target):
    P = {k: v.astype(np.float64) for k, v in F.unpack(shape, F.bf16_round(flat)).items()}
    out, cache = FO.forward(P, x.astype(np.float64), cond.astype(np.float64), shape.n,
                            shape.modes, shape.layers)
    loss, dout = FO.mse(out, target.astype(np.float64))
    G = FO.backward(P, cache, dout, shape.n, shape.modes, shape.layers)
    return out, loss, G


@pytest.mark.parametrize("shape,shared", [(SMALL, False), (SMALL, True), (FULL, True)])
def test_forward_and_gradients_match_oracle(shape, shared):
    torch = _torch()
    B = 4
    flat, x, cond, target = _case(shape, B, shared)
    net = F.FnoNet(shape, params=flat)
    dx, dc, dt = (torch.tensor(a, device="cuda") for a in (x, cond, target))
    out = net.forward(dx, dc)
    net.backward(dt)
    got_out = out.cpu().numpy()
    got_loss = net.loss()
    G = F.unpack(shape, net.get_grads())
    o_out, o_loss, o_G = _oracle(shape, flat, x, cond, target)
    assert np.abs(got_out - o_out).max() <= 2e-4 * np.abs(o_out).max()
    assert got_loss == pytest.approx(o_loss, rel=1e-4)
    for k, g in o_G.items():
        scale = np.abs(g).max()
        assert np.abs(G[k] - g).max() <= 2e-3 * scale + 1e-12, (k, np.abs(G[k] - g).max(), scale)
    net.close()


def test_shared_input_equals_per_sample_input():
    torch = _torch()
    flat, x, cond, _ = _case(SMALL, 4, True)
    net = F.FnoNet(SMALL, params=flat)
    a = net.forward(torch.tensor(x, device="cuda"), torch.tensor(cond, device="cuda")).cpu()
    xb = np.ascontiguousarray(np.broadcast_to(x, (4,) + x.shape))
    b = net.forward(torch.tensor(xb, device="cuda"), torch.tensor(cond, device="cuda")).cpu()
    assert torch.equal(a, b)


def test_adam_step_matches_oracle():
    torch = _torch()
    flat, x, cond, target = _case(SMALL, 4, False)
    net = F.FnoNet(SMALL, params=flat)
    p = flat.astype(np.float64)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    dx, dc, dt = (torch.tensor(a, device="cuda") for a in (x, cond, target))
    for t in range(1, 4):
        net.forward(dx, dc)
        net.backward(dt)
        g = net.get_grads().astype(np.float64)
        net.adam(1e-3)
        p, m, v = FO.adam(p, g, m, v, t, 1e-3)
        got = net.get_params().astype(np.float64)
        assert np.abs(got - p).max() <= 1e-6 * max(1.0, np.abs(p).max())
        p = got          # continue from the device's fp32 values


def test_graph_training_step_equals_separate_calls():
    torch = _torch()
    rows = 6
    flat, x, cond, target = _case(SMALL, rows, False)
    dx, dc, dt = (torch.tensor(a, device="cuda") for a in (x, cond, target))
    a = F.FnoNet(SMALL, params=flat)
    b = F.FnoNet(SMALL, params=flat)
    for idx in (np.array([4, 1, 3], np.int32), np.array([0, 5, 2], np.int32),
                np.array([2, 2, 4], np.int32)):
        a.train_step(dx, dc, dt, idx, 2e-3)          # captured once, then replayed
        ii = torch.tensor(idx.astype(np.int64), device="cuda")
        b.forward(dx[ii].contiguous(), dc[ii].contiguous())
        b.backward(dt[ii].contiguous())
        b.adam(2e-3)
        np.testing.assert_array_equal(a.get_params(), b.get_params())
        assert a.loss() == b.loss()


def test_training_reduces_the_loss():
    torch = _torch()
    shape = F.FnoShape(n=16, width=16, modes=4, layers=2, in_ch=3, out_ch=2, cond=2, hidden=32,
                       max_batch=16)
    rng = np.random.default_rng(5)
    rows = 64
    xs = np.linspace(0, 1, shape.n)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    grid = np.stack([X, Y, np.sin(2 * np.pi * X)]).astype(np.float32)
    cond = rng.uniform(-1, 1, (rows, 2)).astype(np.float32)
    tgt = np.stack([np.stack([c[0] * np.sin(2 * np.pi * X) + c[1] * Y,
                              c[1] * np.cos(2 * np.pi * Y)]) for c in cond]).astype(np.float32)
    dg, dc, dt = (torch.tensor(a, device="cuda") for a in (grid, cond, tgt))
    net = F.FnoNet(shape, seed=3)
    net.forward(dg, dc[:16])
    net.backward(dt[:16])
    first = net.loss()
    for e in range(150):
        perm = rng.permutation(rows).astype(np.int32)
        for k in range(0, rows, 16):
            net.train_step(dg, dc, dt, perm[k:k + 16], 3e-3)
    net.forward(dg, dc[:16])
    net.backward(dt[:16])
    assert net.loss() < 0.05 * first, (first, net.loss())
