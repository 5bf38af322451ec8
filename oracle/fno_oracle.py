"""TEST INFRASTRUCTURE: double-precision restatement of the surrogate
network's forward pass, its hand-derived backward pass and Adam, the checker
for the kernels of ``spatialpy_gb300/csrc/fno.cu``.

Only ``tests/`` and ``__graft_entry__.smoke()`` use it.  The network has no
counterpart in the reference; the oracle itself is pinned against automatic
differentiation of an FFT-based formulation of the same network
(``tests/test_fno_oracle.py``).

Parameters come as the dict of named arrays ``spatialpy_gb300.fno.unpack``
returns (float64 copies of the values the kernels use).  Fields are
[batch][channel][n][n].  The truncated DFTs are written as explicit sums:

  analysis  F[kxi, ky] = s[ky] sum_{x,y} f[x, y] exp(-2 pi i (kx x + ky y) / n)
  synthesis f[x, y]    = sum_{kxi,ky} s[ky] Re(F[kxi, ky] exp(+2 pi i (kx x + ky y) / n))

with kx = kxi for kxi < modes and n - 2 modes + kxi above; the forward
spectral convolution uses s = 1 for the analysis and s = c_ky / n^2
(c_0 = 1, c_ky = 2) for the synthesis, which is numpy's irfft2 of the
truncated spectrum.  Each is the other's adjoint with the same s.

Gradients of complex quantities are dRe + i dIm, so for Y = X W:
dX = dY conj(W)^T and dW = conj(X)^T dY.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_d(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def _bases(n: int, m: int):
    kx = np.concatenate([np.arange(m), np.arange(n - m, n)])
    ky = np.arange(m)
    x = np.arange(n)
    Ex = np.exp(-2j * np.pi * np.outer(kx, x) / n)     # [2m, n]
    Ey = np.exp(-2j * np.pi * np.outer(ky, x) / n)     # [m, n]
    c = np.where(ky == 0, 1.0, 2.0) / (n * n)
    return Ex, Ey, c


def analysis(f, n, m, scale=None):
    """[..., n, n] -> [..., 2m * m] complex."""
    Ex, Ey, _ = _bases(n, m)
    F = np.einsum("ax,by,...xy->...ab", Ex, Ey, f)
    if scale is not None:
        F = F * scale[None, :]
    return F.reshape(*F.shape[:-2], -1)


def synthesis(F, n, m, scale=None):
    """[..., 2m * m] complex -> [..., n, n] real."""
    Ex, Ey, _ = _bases(n, m)
    F = F.reshape(*F.shape[:-1], 2 * m, m)
    if scale is not None:
        F = F * scale[None, :]
    return np.real(np.einsum("ax,by,...ab->...xy", np.conj(Ex), np.conj(Ey), F))


def _spec(P, k):
    w = P[f"spec_w{k}"]
    return w[..., 0] + 1j * w[..., 1]                  # [M, C_in, C_out]


def _pw(W, b, f):
    """pointwise layer on [B, C, n, n] fields."""
    out = np.einsum("oi,bixy->boxy", W, f)
    return out if b is None else out + b[None, :, None, None]


def forward(P: dict, x: np.ndarray, cond: np.ndarray, n: int, m: int, layers: int):
    """Returns (out [B, out_ch, n, n], cache for backward)."""
    B = cond.shape[0]
    if x.ndim == 3:
        x = np.broadcast_to(x, (B,) + x.shape)
    C = P["lin_w0"].shape[0]
    _, _, c = _bases(n, m)
    hid_pre = cond @ P["film1_w"].T + P["film1_b"]
    hid = gelu(hid_pre)
    g = (hid @ P["film2_w"].T + P["film2_b"]).reshape(B, layers, 2, C)
    h = [_pw(P["lift_w"], P["lift_b"], x)]
    X, U = [], []
    for k in range(layers):
        Xk = analysis(h[k], n, m)                                  # [B, C, M]
        Yk = np.einsum("biq,qio->boq", Xk, _spec(P, k))
        s = synthesis(Yk, n, m, c)
        u = s + _pw(P[f"lin_w{k}"], P[f"lin_b{k}"], h[k])
        z = u * (1.0 + g[:, k, 0, :, None, None]) + g[:, k, 1, :, None, None]
        X.append(Xk)
        U.append(u)
        h.append(gelu(z))
    q = _pw(P["proj1_w"], P["proj1_b"], h[-1])
    a = gelu(q)
    out = _pw(P["proj2_w"], P["proj2_b"], a)
    cache = dict(x=x, cond=cond, hid_pre=hid_pre, hid=hid, g=g, h=h, X=X, U=U, q=q, a=a)
    return out, cache


def mse(out, target):
    """(loss, d loss / d out) of the mean squared error."""
    d = out - target
    return float(np.mean(d * d)), 2.0 * d / d.size


def backward(P: dict, cache: dict, dout: np.ndarray, n: int, m: int, layers: int) -> dict:
    """Gradient of every named parameter, given d loss / d out."""
    G = {}
    _, _, c = _bases(n, m)
    ones = np.ones(m)
    h, X, U, g = cache["h"], cache["X"], cache["U"], cache["g"]
    a, q = cache["a"], cache["q"]
    G["proj2_w"] = np.einsum("boxy,bixy->oi", dout, a)
    G["proj2_b"] = dout.sum(axis=(0, 2, 3))
    dq = np.einsum("oi,boxy->bixy", P["proj2_w"], dout) * gelu_d(q)
    G["proj1_w"] = np.einsum("boxy,bixy->oi", dq, h[-1])
    G["proj1_b"] = dq.sum(axis=(0, 2, 3))
    dh = np.einsum("oi,boxy->bixy", P["proj1_w"], dq)
    dg = np.zeros_like(g)
    for k in reversed(range(layers)):
        g0 = g[:, k, 0, :, None, None]
        g1 = g[:, k, 1, :, None, None]
        u = U[k]
        dz = dh * gelu_d(u * (1.0 + g0) + g1)
        du = dz * (1.0 + g0)
        dg[:, k, 0] = (dz * u).sum(axis=(2, 3))
        dg[:, k, 1] = dz.sum(axis=(2, 3))
        G[f"lin_w{k}"] = np.einsum("boxy,bixy->oi", du, h[k])
        G[f"lin_b{k}"] = du.sum(axis=(0, 2, 3))
        dh_k = np.einsum("oi,boxy->bixy", P[f"lin_w{k}"], du)
        dY = analysis(du, n, m, c)                                 # adjoint of the synthesis
        dW = np.einsum("biq,boq->qio", np.conj(X[k]), dY)
        G[f"spec_w{k}"] = np.stack([dW.real, dW.imag], axis=-1)
        dX = np.einsum("boq,qio->biq", dY, np.conj(_spec(P, k)))
        dh = dh_k + synthesis(dX, n, m, ones)                      # adjoint of the analysis
    G["lift_w"] = np.einsum("boxy,bixy->oi", dh, cache["x"])
    G["lift_b"] = dh.sum(axis=(0, 2, 3))
    dgf = dg.reshape(dg.shape[0], -1)
    G["film2_w"] = dgf.T @ cache["hid"]
    G["film2_b"] = dgf.sum(axis=0)
    dpre = (dgf @ P["film2_w"]) * gelu_d(cache["hid_pre"])
    G["film1_w"] = dpre.T @ cache["cond"]
    G["film1_b"] = dpre.sum(axis=0)
    return G


def adam(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (PyTorch's form): returns (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    denom = np.sqrt(v) / np.sqrt(1 - b2 ** t) + eps
    return p - (lr / (1 - b1 ** t)) * m / denom, m, v
