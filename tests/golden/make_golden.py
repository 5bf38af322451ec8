"""Generate the golden fixtures in tests/golden/ from the compiled reference engine.

Run where the SpatialPy reference sources exist (they are compiled by
oracle/build_ref.sh into oracle/_ref/):

    python tests/golden/make_golden.py

Fixtures (all inputs are rebuilt by spatialpy_gb300.scenario builders with the
parameters stored alongside):

* neighbors.npz      reference neighbour sets, dist, dWdr and D_ij
                     (particle.cpp:150-294 via the ANN kd-tree) for several
                     domains, sorted by neighbour index per particle
* nsm_birth_death.npz  1,000-trajectory reference ensembles of the spatial
                     birth-death model, stock and rescaled-selection engine:
                     per-output mean/variance of the total and per-voxel
                     means at the last output
* nsm_rdme_small.npz   the A+B<->C, 0->A, C->0 network on a 6^3 lattice,
                     400 trajectories per engine variant, per-species totals
* sdpd_small.npz     reference SDPD dam-break states after 1, 5, 21, 41 steps
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from spatialpy_gb300 import scenario as S  # noqa: E402


def neighbor_domains():
    rng = np.random.default_rng(11)
    doms = {
        "bd2d_10": S.config_birth_death_2d(),
        "rdme3d_6": S.config_rdme_3d(n=6, nA=50, nB=50),
        "dam_8": S.config_dam_break(spacing_div=8, num_steps=10),
    }
    # irregular point clouds (exercise non-lattice distances and ties)
    for dim, n, h in ((2, 300, 0.08), (3, 500, 0.15)):
        x = np.zeros((n, 3))
        x[:, :dim] = rng.random((n, dim))
        base = S.config_birth_death_2d()
        sc = base.copy(x=x, type=np.ones(n), mass=rng.uniform(0.5, 2.0, n),
                       rho=rng.uniform(50, 150, n), nu=np.ones(n), fixed=np.ones(n),
                       u0=np.zeros((n, 1)), dimension=dim, h=h)
        doms[f"cloud{dim}d_{n}"] = sc
    # 1-D line: the reference's 1-D kernel constant is `5 / 4 * h` = h
    x = np.zeros((40, 3))
    x[:, 0] = np.linspace(0, 1, 40)
    base = S.config_birth_death_2d()
    doms["line_40"] = base.copy(x=x, type=np.ones(40), mass=1.0, rho=40.0, nu=1.0, fixed=1,
                                u0=np.zeros((40, 1)), dimension=1, h=S.find_h(x))
    return doms


def sorted_lists(cnt, idx, dist, dw, dij):
    n, k = idx.shape
    o_idx = np.full((n, k), -1, np.int32)
    o = [np.zeros((n, k)) for _ in range(3)]
    for i in range(n):
        c = cnt[i]
        order = np.argsort(idx[i, :c], kind="stable")
        o_idx[i, :c] = idx[i, :c][order]
        for a, src in zip(o, (dist, dw, dij)):
            a[i, :c] = src[i, :c][order]
    return o_idx, o[0], o[1], o[2]


def _ens_worker(args):
    name, variant, seeds, kw = args
    sc = getattr(S, name)(**kw)
    tots, vox, ev = [], [], []
    for s in seeds:
        out, e = oracle.ref_nsm(sc, int(s), variant)
        tots.append(out.sum(axis=1))           # [T, S]
        vox.append(out[-1])                    # [N, S]
        ev.append(e)
    return np.array(tots), np.array(vox), np.array(ev)


def ensemble(name, variant, ntraj, seed0, kw, procs=8):
    seeds = np.arange(seed0, seed0 + ntraj, dtype=np.uint64)
    chunks = np.array_split(seeds, procs)
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        parts = pool.map(_ens_worker, [(name, variant, c, kw) for c in chunks])
    tots = np.concatenate([p[0] for p in parts])
    vox = np.concatenate([p[1] for p in parts])
    ev = np.concatenate([p[2] for p in parts])
    return tots, vox, ev


def main():
    if not oracle.reference_available():
        if not oracle.build_reference():
            raise SystemExit("reference engine sources are not available here")
    # 1. neighbour lists
    fx = {}
    for key, sc in neighbor_domains().items():
        cnt, idx, dist, dw, dij = oracle.ref_neighbors(sc, 1024)
        k = int(cnt.max())
        i2, d2, w2, j2 = sorted_lists(cnt, idx[:, :k], dist[:, :k], dw[:, :k], dij[:, :k])
        fx[f"{key}/x"] = sc.x
        fx[f"{key}/mass"] = sc.mass
        fx[f"{key}/rho"] = sc.rho
        fx[f"{key}/dim"] = np.int32(sc.dimension)
        fx[f"{key}/h"] = np.float64(sc.h)
        fx[f"{key}/count"] = cnt
        fx[f"{key}/idx"] = i2
        fx[f"{key}/dist"] = d2
        fx[f"{key}/dWdr"] = w2
        fx[f"{key}/Dij"] = j2
    np.savez_compressed(os.path.join(HERE, "neighbors.npz"), **fx)
    print("neighbors.npz:", len(fx) // 10, "domains")

    # 2. birth-death ensembles
    out = {}
    for variant in ("", "_exact"):
        tots, vox, ev = ensemble("config_birth_death_2d", variant, 1000, 20260101, {})
        tag = variant.strip("_") or "stock"
        out[f"{tag}/total_mean"] = tots[:, :, 0].mean(0)
        out[f"{tag}/total_var"] = tots[:, :, 0].var(0, ddof=1)
        out[f"{tag}/voxel_mean_last"] = vox[:, :, 0].mean(0)
        out[f"{tag}/voxel_var_last"] = vox[:, :, 0].var(0, ddof=1)
        out[f"{tag}/events_mean"] = ev.mean(0)
        out[f"{tag}/ntraj"] = np.int32(len(tots))
        print("birth-death", tag, tots[:, -1, 0].mean(), ev.mean(0))
    np.savez_compressed(os.path.join(HERE, "nsm_birth_death.npz"), **out)

    # 3. small 3-D RDME network
    kw = dict(n=6, nA=300, nB=300, t_end=10.0, num_points=11, dt=1.0)
    out = {"kw_n": np.int32(6), "kw_nA": np.int32(300), "kw_nB": np.int32(300)}
    for variant in ("", "_exact"):
        tots, vox, ev = ensemble("config_rdme_3d", variant, 400, 777, kw)
        tag = variant.strip("_") or "stock"
        out[f"{tag}/total_mean"] = tots.mean(0)          # [T, S]
        out[f"{tag}/total_var"] = tots.var(0, ddof=1)
        out[f"{tag}/events_mean"] = ev.mean(0)
        out[f"{tag}/ntraj"] = np.int32(len(tots))
        print("rdme", tag, tots[:, -1].mean(0), ev.mean(0))
    np.savez_compressed(os.path.join(HERE, "nsm_rdme_small.npz"), **out)

    # 4. SDPD
    sc = S.config_dam_break(spacing_div=8, num_steps=41)
    out = {"spacing_div": np.int32(8)}
    for nsteps in (1, 5, 21, 41):
        x, v, rho = oracle.ref_sdpd(sc, nsteps)
        out[f"{nsteps}/x"] = x
        out[f"{nsteps}/v"] = v
        out[f"{nsteps}/rho"] = rho
    np.savez_compressed(os.path.join(HERE, "sdpd_small.npz"), **out)
    print("sdpd_small.npz written")


if __name__ == "__main__":
    main()
