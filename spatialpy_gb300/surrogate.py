"""Learned surrogate beside the exact SSA: a FiLM-conditioned Fourier neural
operator that predicts per-voxel ensemble mean and variance over a parameter
sweep, trained on ensembles the GPU engine generates, with the SSA as the
fallback wherever its held-out error exceeds a threshold.

Workload (reduced from the full sweep: see ``SweepConfig``): the RDME network
of the 3-D bench (A + B -> C, C -> A + B, 0 -> A on x < 0.1, C -> 0) on a 2-D
n x n lattice; the parameters (k_f, k_r, k_birth, D_A = D_B, D_C) are drawn
log-uniformly within one decade of the base values; the targets are the
per-voxel mean and variance of A, B, C at the output times.

The network (``spatialpy_gb300.fno``, kernels in ``csrc/fno.cu``): input
channels are the voxel coordinates, the initial counts and the birth-region
mask; a pointwise lift to ``width`` channels; ``layers`` Fourier layers, each
a spectral convolution on the lowest ``modes`` x ``modes`` frequencies plus a
pointwise linear map, with FiLM scale and shift from an MLP on (log
parameters, time) and GELU; a pointwise projection to 6 channels (means and
log-variances).  Forward, backward and Adam are this library's own kernels,
with bf16 weights and fp32 accumulation; PyTorch only holds device memory.

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
# the network: csrc/fno.cu through spatialpy_gb300.fno
# ---------------------------------------------------------------------------
class Surrogate:
    """FNO surrogate of the ensemble mean and variance of a parameter sweep."""

    def __init__(self, cfg: SweepConfig, device: str = "cuda", width: int = 32, modes: int = 12,
                 layers: int = 4, seed: int = 0, batch: int = 64, members: int = 1):
        """``members`` networks with seeds seed, seed+1, ... are trained
        independently; predictions are their average."""
        import torch
        from .fno import FnoNet, FnoShape
        self.torch = torch
        self.cfg = cfg
        self.device = device
        self.batch = batch
        n = cfg.n
        self.shape = FnoShape(n=n, width=width, modes=min(modes, n // 2), layers=layers,
                              in_ch=6, out_ch=6, cond=len(NAMES) + 1, hidden=64, max_batch=batch)
        self.nets = [FnoNet(self.shape, seed=seed + j) for j in range(members)]
        self.seed = seed
        sc = point_scenario(np.array([BASE[k] for k in NAMES]), cfg)
        xy = sc.x[:, :2].reshape(n, n, 2)
        u0 = sc.u0.astype(np.float64).reshape(n, n, 3)
        mask = (sc.type == 2).reshape(n, n, 1).astype(np.float64)
        grid = np.concatenate([xy, u0 / max(1.0, u0.max()), mask], axis=2)   # [n,n,6]
        self.grid = torch.tensor(np.ascontiguousarray(grid.transpose(2, 0, 1)),
                                 dtype=torch.float32, device=device)          # shared input
        self.times = np.arange(1, cfg.num_times + 1) * (cfg.t_end / cfg.num_times)
        self.scale = None

    def _cond(self, params: np.ndarray):
        base = np.array([BASE[k] for k in NAMES])
        lp = np.log10(params / base)                           # [-1, 1]
        T = len(self.times)
        c = np.concatenate([np.repeat(lp, T, axis=0),
                            np.tile(self.times / self.cfg.t_end, len(params))[:, None]], axis=1)
        return self.torch.tensor(c, dtype=self.torch.float32, device=self.device)

    def _targets(self, mean, var):
        P, T, N, S_ = mean.shape
        n = self.cfg.n
        y = np.concatenate([mean / self.scale, np.log1p(var) / np.log1p(self.scale)], axis=3)
        y = y.reshape(P * T, n, n, 2 * S_).transpose(0, 3, 1, 2)
        return self.torch.tensor(np.ascontiguousarray(y), dtype=self.torch.float32,
                                 device=self.device)

    def fit(self, params, mean, var, epochs: int = 300, lr: float = 2e-3):
        """Train every member on SSA ensemble moments (Adam, cosine
        learning-rate schedule, minibatches of ``batch`` rows); returns the
        members' mean final loss and sets ``train_seconds``."""
        torch = self.torch
        self.scale = float(max(mean.max(), 1.0))
        c = self._cond(params)
        y = self._targets(mean, var)
        rows = y.shape[0]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        losses = []
        for j, net in enumerate(self.nets):
            rng = np.random.default_rng(self.seed + j)
            for e in range(epochs):
                lr_e = lr * 0.5 * (1.0 + math.cos(math.pi * e / epochs))
                perm = rng.permutation(rows).astype(np.int32)
                for k in range(0, rows, self.batch):
                    net.train_step(self.grid, c, y, perm[k:k + self.batch], lr_e)
            losses.append(net.loss())
        self.train_seconds = time.perf_counter() - t0
        return float(np.mean(losses))

    def predict(self, params):
        """(mean, var) [P, T, N, 3] and the device seconds of inference."""
        torch = self.torch
        c = self._cond(params)
        n = self.cfg.n
        outs = [torch.empty(c.shape[0], 6, n, n, dtype=torch.float32, device=self.device)
                for _ in self.nets]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for net, out in zip(self.nets, outs):
            for k in range(0, c.shape[0], self.batch):
                net.forward(self.grid, c[k:k + self.batch], out=out[k:k + self.batch])
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        members = [self._fields(o.cpu().numpy(), len(params)) for o in outs]
        self.last_members = members
        out = np.mean([o.cpu().numpy() for o in outs], axis=0)
        mean, var = self._fields(out, len(params))
        return mean, var, sec

    def _fields(self, out, P):
        n = self.cfg.n
        out = out.transpose(0, 2, 3, 1).reshape(P, len(self.times), n * n, 6)
        mean = np.maximum(out[..., :3] * self.scale, 0.0)
        var = np.maximum(np.expm1(out[..., 3:] * math.log1p(self.scale)), 0.0)
        return mean, var


def sweep(surrogate: Surrogate, params, ssa_mean, ssa_var, ssa_seconds: float,
          threshold: float = 0.02, block: int = 8):
    """Surrogate answers with SSA fallback where the coarse error of the mean
    or the variance against the held-out SSA ensemble exceeds ``threshold``
    (the SSA judges every point; only the fallback points' share of its time
    is charged to the surrogate).  Returns a summary dict.

    With several members it also reports a gate that needs no SSA: accept a
    point when the members' spread around their average (the same coarse
    metric) is at most ``threshold / 2`` for the mean and the variance; the
    summary gives how many points it accepts, how many of those are within
    ``threshold`` of the SSA, and the time with the SSA answering the rest."""
    cfg = surrogate.cfg
    pm, pv, inf_s = surrogate.predict(params)
    em = rel_error(pm, ssa_mean, cfg.n, block)
    ev = rel_error(pv, ssa_var, cfg.n, block)
    ok = (em <= threshold) & (ev <= threshold)
    P = len(params)
    fallback_s = ssa_seconds * (P - ok.sum()) / P
    out = {"points": P, "accepted": int(ok.sum()), "err_mean_median": float(np.median(em)),
           "err_var_median": float(np.median(ev)), "inference_s": inf_s,
           "ssa_s": ssa_seconds, "surrogate_plus_fallback_s": inf_s + fallback_s,
           "speedup": ssa_seconds / (inf_s + fallback_s), "threshold": threshold}
    members = getattr(surrogate, "last_members", [])
    if len(members) > 1:
        sm = np.mean([rel_error(m, pm, cfg.n, block) for m, _ in members], axis=0)
        sv = np.mean([rel_error(v, pv, cfg.n, block) for _, v in members], axis=0)
        gate = (sm <= threshold / 2) & (sv <= threshold / 2)
        gs = inf_s + ssa_seconds * (P - gate.sum()) / P
        out.update({"gated_accepted": int(gate.sum()),
                    "gated_within_threshold": int((gate & ok).sum()),
                    "gated_seconds": gs, "gated_speedup": ssa_seconds / gs})
    return out
