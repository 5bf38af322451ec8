"""PyTorch formulation of the surrogate network with FFTs (torch.fft.rfft2 /
irfft2 on the truncated spectrum) and autograd: the independent reference the
double-precision oracle (oracle/fno_oracle.py) is pinned against."""
from __future__ import annotations

import numpy as np
import torch


def forward(P: dict, x, cond, n: int, m: int, layers: int):
    """P: named torch tensors (the layout of spatialpy_gb300.fno.param_layout)."""
    B = cond.shape[0]
    if x.dim() == 3:
        x = x.expand(B, -1, -1, -1)
    C = P["lin_w0"].shape[0]
    gelu = torch.nn.functional.gelu

    def pw(W, b, f):
        return torch.einsum("oi,bixy->boxy", W, f) + b[None, :, None, None]

    hid = gelu(cond @ P["film1_w"].T + P["film1_b"])
    g = (hid @ P["film2_w"].T + P["film2_b"]).reshape(B, layers, 2, C)
    h = pw(P["lift_w"], P["lift_b"], x)
    for k in range(layers):
        w = torch.view_as_complex(P[f"spec_w{k}"].contiguous()).reshape(2 * m, m, C, C)
        hf = torch.fft.rfft2(h)                                   # [B, C, n, n//2+1]
        out = torch.zeros(B, C, n, n // 2 + 1, dtype=hf.dtype)
        out[:, :, :m, :m] = torch.einsum("bixy,xyio->boxy", hf[:, :, :m, :m], w[:m])
        out[:, :, n - m:, :m] = torch.einsum("bixy,xyio->boxy", hf[:, :, n - m:, :m], w[m:])
        s = torch.fft.irfft2(out, s=(n, n))
        u = s + pw(P[f"lin_w{k}"], P[f"lin_b{k}"], h)
        h = gelu(u * (1.0 + g[:, k, 0, :, None, None]) + g[:, k, 1, :, None, None])
    a = gelu(pw(P["proj1_w"], P["proj1_b"], h))
    return pw(P["proj2_w"], P["proj2_b"], a)


def loss_and_grads(named: dict, x: np.ndarray, cond: np.ndarray, target: np.ndarray, n, m,
                   layers):
    """MSE and its gradients (float64) by autograd."""
    P = {k: torch.tensor(v, dtype=torch.float64, requires_grad=True) for k, v in named.items()}
    out = forward(P, torch.tensor(x, dtype=torch.float64), torch.tensor(cond, dtype=torch.float64),
                  n, m, layers)
    loss = torch.mean((out - torch.tensor(target, dtype=torch.float64)) ** 2)
    loss.backward()
    return float(loss.detach()), out.detach().numpy(), {k: t.grad.numpy() for k, t in P.items()}
