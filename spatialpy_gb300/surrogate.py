"""Learned surrogate beside the exact SSA: a FiLM-conditioned Fourier neural
operator that predicts per-voxel ensemble mean and variance over a parameter
sweep, trained on ensembles the GPU engine generates, with the SSA as the
fallback wherever its held-out error exceeds a threshold.

Workload (reduced from the full sweep: see ``SweepConfig``): the RDME network
of the 3-D bench (A + B -> C, C -> A + B, 0 -> A on x < 0.1, C -> 0) on a 2-D
n x n lattice; the parameters (k_f, k_r, k_birth, D_A = D_B, D_C) are drawn
log-uniformly within one decade of the base values; the targets are the
per-voxel mean and variance of A, B, C at the output times.

The network (``FNO``): input channels are the voxel coordinates, the
initial counts and the birth-region mask; a pointwise lift to ``width``
channels; ``layers`` Fourier layers, each a spectral convolution on the
lowest ``modes`` x ``modes`` frequencies plus a pointwise linear map, with
FiLM scale and shift from an MLP on (log parameters, time) and GELU; a
pointwise projection to 6 channels (means and log-variances).  Weights are
kept in fp32 and the forward runs under bf16 autocast, so matrix products
take bf16 operands with fp32 accumulation.

The learned part runs on PyTorch operations (cuBLAS GEMMs and cuFFT under
torch); the SSA it stands in for is this engine's own kernels.

Error and fallback: the SSA estimate of a point is noisy (a few molecules per
voxel), so errors are measured on coarse-grained fields: the mean over
``block`` x ``block`` voxel blocks, relative L2 over species, times and
blocks, for the means and the variances.  A sweep point whose surrogate
error on the held-out check exceeds ``threshold`` is answered by the SSA.
"""
from __future__ import annotations

import dataclasses
import math
import time

import numpy as np

from . import scenario as S


@dataclasses.dataclass
class SweepConfig:
    n: int = 32                 # lattice edge (n x n voxels)
    molecules: int = 1000       # initial A and B, each, scattered
    t_end: float = 4.0
    num_times: int = 8          # output times t_end / num_times * k, k = 1..num_times
    trajectories: int = 32      # SSA ensemble per parameter point
    seed: int = 5


BASE = {"k_f": 1e-3, "k_r": 0.1, "k_birth": 5.0, "D_A": 1e-2, "D_C": 1e-3}
NAMES = list(BASE)


def sample_parameters(n: int, rng) -> np.ndarray:
    """[n, 5] parameter points, each log-uniform within one decade of BASE."""
    base = np.array([BASE[k] for k in NAMES])
    return base * 10.0 ** rng.uniform(-1.0, 1.0, (n, len(NAMES)))


def point_scenario(p, cfg: SweepConfig) -> S.Scenario:
    k_f, k_r, k_b, d_a, d_c = (float(v) for v in p)
    return S.config_rdme_3d(n=cfg.n, dims=2, D=(d_a, d_a, d_c), k_f=k_f, k_r=k_r, k_birth=k_b,
                            nA=cfg.molecules, nB=cfg.molecules, t_end=cfg.t_end,
                            num_points=cfg.num_times + 1, dt=cfg.t_end / cfg.num_times,
                            seed=cfg.seed)


def ssa_moments(params: np.ndarray, cfg: SweepConfig, seed0: int = 1000):
    """GPU SSA ensembles of every parameter point in one engine run (one
    instance per point).  Returns (mean, var) [P, T, N, 3] over the output
    times after t = 0, and the device seconds."""
    from .engine import Engine
    scs = [point_scenario(p, cfg) for p in params]
    P, J = len(scs), cfg.trajectories
    inst = np.repeat(np.arange(P, dtype=np.int32), J)
    seeds = np.arange(seed0, seed0 + P * J, dtype=np.uint64)
    with Engine(scs) as eng:
        res = eng.run(seeds, instance=inst, want_counts=False, want_moments=True)
        ms = eng.profile()["total_ms"]
    mean, var = [], []
    for m in res["moments"]:
        s1 = m[1:, :, :, 0].astype(np.float64)
        s2 = m[1:, :, :, 1].astype(np.float64)
        mu = s1 / J
        mean.append(mu)
        var.append(np.maximum(s2 / J - mu * mu, 0.0) * J / (J - 1))
    return np.array(mean), np.array(var), ms / 1e3


def coarse(field: np.ndarray, n: int, block: int) -> np.ndarray:
    """[..., N, S] voxel fields -> [..., (n/block)^2, S] block means."""
    lead = field.shape[:-2]
    S_ = field.shape[-1]
    f = field.reshape(*lead, n // block, block, n // block, block, S_)
    return f.mean(axis=(-4, -2)).reshape(*lead, -1, S_)


def rel_error(pred: np.ndarray, ref: np.ndarray, n: int, block: int = 8) -> np.ndarray:
    """Per point relative L2 error of coarse-grained fields [P, T, N, S]."""
    a, b = coarse(pred, n, block), coarse(ref, n, block)
    P = a.shape[0]
    num = np.sqrt(((a - b) ** 2).reshape(P, -1).sum(1))
    den = np.sqrt((b ** 2).reshape(P, -1).sum(1))
    return num / np.maximum(den, 1e-30)


# ---------------------------------------------------------------------------
# the network
# ---------------------------------------------------------------------------
def _torch():
    import torch
    return torch


def build_fno(width: int = 32, modes: int = 12, layers: int = 4, in_ch: int = 6,
              out_ch: int = 6, cond: int = 6):
    torch = _torch()
    nn = torch.nn

    class Spectral(nn.Module):
        def __init__(self):
            super().__init__()
            scale = 1.0 / (width * width)
            self.w1 = nn.Parameter(scale * torch.randn(width, width, modes, modes, 2))
            self.w2 = nn.Parameter(scale * torch.randn(width, width, modes, modes, 2))

        def forward(self, x):
            b, c, h, w = x.shape
            # the FFT runs in fp32 (or fp64) whatever the autocast dtype
            xr = x if x.dtype in (torch.float32, torch.float64) else x.float()
            xf = torch.fft.rfft2(xr)
            out = torch.zeros(b, width, h, w // 2 + 1, dtype=xf.dtype, device=x.device)
            w1 = torch.view_as_complex(self.w1).to(xf.dtype)
            w2 = torch.view_as_complex(self.w2).to(xf.dtype)
            out[:, :, :modes, :modes] = torch.einsum("bixy,ioxy->boxy", xf[:, :, :modes, :modes], w1)
            out[:, :, -modes:, :modes] = torch.einsum("bixy,ioxy->boxy", xf[:, :, -modes:, :modes], w2)
            return torch.fft.irfft2(out, s=(h, w))

    class FNO(nn.Module):
        def __init__(self):
            super().__init__()
            self.lift = nn.Conv2d(in_ch, width, 1)
            self.spec = nn.ModuleList([Spectral() for _ in range(layers)])
            self.lin = nn.ModuleList([nn.Conv2d(width, width, 1) for _ in range(layers)])
            self.film = nn.Sequential(nn.Linear(cond, 64), nn.GELU(), nn.Linear(64, 2 * width * layers))
            self.proj = nn.Sequential(nn.Conv2d(width, 64, 1), nn.GELU(), nn.Conv2d(64, out_ch, 1))

        def forward(self, x, c):
            h = self.lift(x)
            g = self.film(c).view(c.shape[0], len(self.spec), 2, -1, 1, 1)
            for k, (sp, li) in enumerate(zip(self.spec, self.lin)):
                h = sp(h) + li(h)
                h = h * (1.0 + g[:, k, 0]) + g[:, k, 1]
                h = torch.nn.functional.gelu(h)
            return self.proj(h)

    return FNO()


class Surrogate:
    """FNO surrogate of the ensemble mean and variance of a parameter sweep."""

    def __init__(self, cfg: SweepConfig, device: str = "cuda", width: int = 32, modes: int = 12,
                 layers: int = 4, seed: int = 0):
        torch = _torch()
        torch.manual_seed(seed)
        self.cfg = cfg
        self.device = device
        self.modes = min(modes, cfg.n // 2)
        self.net = build_fno(width, self.modes, layers).to(device)
        sc = point_scenario(np.array([BASE[k] for k in NAMES]), cfg)
        n = cfg.n
        xy = sc.x[:, :2].reshape(n, n, 2)
        u0 = sc.u0.astype(np.float64).reshape(n, n, 3)
        mask = (sc.type == 2).reshape(n, n, 1).astype(np.float64)
        grid = np.concatenate([xy, u0 / max(1.0, u0.max()), mask], axis=2)   # [n,n,6]
        self.grid = torch.tensor(grid.transpose(2, 0, 1)[None], dtype=torch.float32, device=device)
        self.times = np.arange(1, cfg.num_times + 1) * (cfg.t_end / cfg.num_times)
        self.scale = None

    def _cond(self, params: np.ndarray):
        torch = _torch()
        base = np.array([BASE[k] for k in NAMES])
        lp = np.log10(params / base)                           # [-1, 1]
        P, T = len(params), len(self.times)
        c = np.concatenate([np.repeat(lp, T, axis=0),
                            np.tile(self.times / self.cfg.t_end, P)[:, None]], axis=1)
        return torch.tensor(c, dtype=torch.float32, device=self.device)

    def _targets(self, mean, var):
        torch = _torch()
        P, T, N, S_ = mean.shape
        n = self.cfg.n
        y = np.concatenate([mean / self.scale, np.log1p(var) / np.log1p(self.scale)], axis=3)
        y = y.reshape(P * T, n, n, 2 * S_).transpose(0, 3, 1, 2)
        return torch.tensor(np.ascontiguousarray(y), dtype=torch.float32, device=self.device)

    def fit(self, params, mean, var, epochs: int = 300, lr: float = 2e-3, batch: int = 64):
        """Train on SSA ensemble moments; returns the final training loss."""
        torch = _torch()
        self.scale = float(max(mean.max(), 1.0))
        c = self._cond(params)
        y = self._targets(mean, var)
        opt = torch.optim.Adam(self.net.parameters(), lr=lr)
        sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, epochs)
        n = y.shape[0]
        loss = torch.tensor(0.0)
        for _ in range(epochs):
            perm = torch.randperm(n, device=self.device)
            for k in range(0, n, batch):
                idx = perm[k:k + batch]
                with torch.autocast("cuda", dtype=torch.bfloat16):
                    out = self.net(self.grid.expand(len(idx), -1, -1, -1), c[idx])
                loss = torch.mean((out.float() - y[idx]) ** 2)
                opt.zero_grad(set_to_none=True)
                loss.backward()
                opt.step()
            sched.step()
        return float(loss.detach())

    def predict(self, params):
        """(mean, var) [P, T, N, 3] and the device seconds of inference."""
        torch = _torch()
        c = self._cond(params)
        n = self.cfg.n
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.no_grad(), torch.autocast("cuda", dtype=torch.bfloat16):
            out = self.net(self.grid.expand(c.shape[0], -1, -1, -1), c).float()
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        out = out.cpu().numpy().transpose(0, 2, 3, 1).reshape(len(params), len(self.times), n * n, 6)
        mean = np.maximum(out[..., :3] * self.scale, 0.0)
        var = np.maximum(np.expm1(out[..., 3:] * math.log1p(self.scale)), 0.0)
        return mean, var, sec


def sweep(surrogate: Surrogate, params, ssa_mean, ssa_var, ssa_seconds: float,
          threshold: float = 0.02, block: int = 8):
    """Surrogate answers with SSA fallback where the coarse error of the mean
    or the variance exceeds ``threshold``; returns a summary dict."""
    cfg = surrogate.cfg
    pm, pv, inf_s = surrogate.predict(params)
    em = rel_error(pm, ssa_mean, cfg.n, block)
    ev = rel_error(pv, ssa_var, cfg.n, block)
    ok = (em <= threshold) & (ev <= threshold)
    P = len(params)
    fallback_s = ssa_seconds * (P - ok.sum()) / P
    return {"points": P, "accepted": int(ok.sum()), "err_mean_median": float(np.median(em)),
            "err_var_median": float(np.median(ev)), "inference_s": inf_s,
            "ssa_s": ssa_seconds, "surrogate_plus_fallback_s": inf_s + fallback_s,
            "speedup": ssa_seconds / (inf_s + fallback_s), "threshold": threshold}
