"""Generate the golden fixtures in tests/golden/ from the compiled reference engine.

Run where the SpatialPy reference is present ($SPATIALPY_REFERENCE or its
pip install in baseline/_ref; its engine is compiled by oracle/build_ref.sh
into oracle/_ref/), optionally naming the fixtures to write:

    python tests/golden/make_golden.py [neighbors] [bd] [rdme] [rdme40] [sdpd] [pins] [coupled] [vtk]

Fixtures (all inputs are rebuilt by spatialpy_gb300.scenario builders with the
parameters stored alongside):

* neighbors.npz      reference neighbour sets, dist, dWdr and D_ij
                     (particle.cpp:150-294 via the ANN kd-tree) for several
                     domains, sorted by neighbour index per particle
* nsm_birth_death.npz  10,000-trajectory reference ensembles of the spatial
                     birth-death model (100 voxels, t = 0..10), stock and
                     rescaled-selection engine: per-output mean/variance of
                     the total, and per voxel and output the mean, variance
                     and fourth central moment
* nsm_rdme_small.npz   the A+B<->C, 0->A, C->0 network on a 6^3 lattice,
                     400 trajectories per engine variant, per-species totals
* nsm_rdme40.npz     the bench's 40^3 model (64,000 voxels, A+B<->C, 0->A,
                     C->0; 10,000 A and 10,000 B), rescaled selection, 1,000
                     trajectories over t = 0..5: per-output mean/variance of
                     the species totals, and per voxel and species the sums
                     of x, x^2, x^3, x^4 over the trajectories at t = 1 and 5
* sdpd_small.npz     reference SDPD dam-break states after 1, 5, 21, 41 steps
* pins.npz           the deterministic chemistry on a static lattice
                     (tests/chem_cases.py pinned_chem) and on the moving dam
                     break (tests/coupled_cases.py dam_break_chem): the
                     concentrations at every output; the dam break with flow
                     boundary conditions (chem_cases.flow_bcs): x, v, rho
                     after 1, 5, 21, 41 steps
* nsm_coupled.npz    2,000-trajectory ensembles of the moving dam break with
                     species (coupled_cases.dam_break_species, 1,368
                     particles, network "full", 60 steps), stock and rescaled
                     selection: per particle and output the mean, variance
                     and fourth central moment of the counts, the totals'
                     mean and variance, and the mean event counts
* vtk_ref.npz        outputN.vtk files written by the engine's own VTK writer
                     (output.cpp) for three runs (the birth-death lattice; the
                     pinned chemistry case with C[] and D[] fields; the moving
                     dam break with species), with the full-precision state
                     each file was written from
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


def _moment_worker(args):
    name, variant, seeds, kw, outs = args
    sc = getattr(S, name)(**kw)
    m = None
    tots, ev = [], []
    for s in seeds:
        out, e = oracle.ref_nsm(sc, int(s), variant)
        x = out[list(outs)].astype(np.float64)               # [len(outs), N, S]
        p = [x, x * x, x * x * x, x * x * x * x]
        m = p if m is None else [a + b for a, b in zip(m, p)]
        tots.append(out.sum(axis=1))
        ev.append(e)
    return m, np.array(tots), np.array(ev)


def moment_ensemble(name, variant, ntraj, seed0, kw, outs, procs=None):
    """Sums over ntraj reference trajectories of x, x^2, x^3, x^4 at the
    outputs `outs` ([len(outs), N, S] each), the per-trajectory totals
    [ntraj, T, S] and event counts [ntraj, 2]."""
    procs = procs or os.cpu_count() or 1
    seeds = np.arange(seed0, seed0 + ntraj, dtype=np.uint64)
    chunks = [c for c in np.array_split(seeds, procs) if len(c)]
    with mp.get_context("spawn").Pool(len(chunks)) as pool:
        parts = pool.map(_moment_worker, [(name, variant, c, kw, outs) for c in chunks])
    m = [sum(p[0][k] for p in parts) for k in range(4)]
    return m, np.concatenate([p[1] for p in parts]), np.concatenate([p[2] for p in parts])


def central_moments(m, n):
    """mean, variance (ddof=1) and fourth central moment from raw sums."""
    mu = m[0] / n
    e2, e3, e4 = m[1] / n, m[2] / n, m[3] / n
    var = (e2 - mu * mu) * n / (n - 1)
    m4 = e4 - 4 * mu * e3 + 6 * mu * mu * e2 - 3 * mu ** 4
    return mu, var, m4


def _coupled_worker(args):
    variant, seeds, kw = args
    sys.path.insert(0, os.path.dirname(HERE))
    from coupled_cases import dam_break_species
    sc = dam_break_species(**kw)
    m, tots, ev = None, [], []
    for s in seeds:
        out, e = oracle.ref_coupled(sc, int(s), variant)
        x = out.astype(np.float64)
        p = [x, x * x, x * x * x, x * x * x * x]
        m = p if m is None else [a + b for a, b in zip(m, p)]
        tots.append(out.sum(axis=1))
        ev.append(e)
    return m, np.array(tots), np.array(ev)


def vtk_cases():
    sys.path.insert(0, os.path.dirname(HERE))
    from chem_cases import pinned_chem
    from coupled_cases import dam_break_species
    return {"bd": (S.config_birth_death_2d(t_end=2.0, num_points=3), ["A"]),
            "chem": (pinned_chem(), ["A", "B"]),
            "dam": (dam_break_species(spacing_div=8, num_steps=10, num_outputs=2,
                                      network="decay"), ["S"])}


def _vtk_worker(key):
    import tempfile
    sc, names = vtk_cases()[key]
    with tempfile.TemporaryDirectory() as d:
        st = oracle.ref_vtk_run(sc, 11, names, d)
        files = [open(os.path.join(d, f"output{k}.vtk"), "rb").read()
                 for k in range(len(sc.output_steps))]
        bbox = open(os.path.join(d, "output0_boundingBox.vtk"), "rb").read()
    return st, files, bbox


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
    want = set(sys.argv[1:]) or {"neighbors", "bd", "rdme", "rdme40", "sdpd"}
    if not oracle.reference_available():
        if not oracle.build_reference():
            raise SystemExit("reference engine sources are not available here")
    if "neighbors" in want:
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

    if "bd" in want:   # birth-death ensembles, per-voxel moments at every output
        out = {}
        sc = S.config_birth_death_2d()
        outs = tuple(range(len(sc.output_steps)))
        for variant in ("", "_exact"):
            m, tots, ev = moment_ensemble("config_birth_death_2d", variant, 10000, 20260101, {},
                                          outs)
            n = len(tots)
            mu, var, m4 = central_moments(m, n)
            tag = variant.strip("_") or "stock"
            out[f"{tag}/total_mean"] = tots[:, :, 0].mean(0)
            out[f"{tag}/total_var"] = tots[:, :, 0].var(0, ddof=1)
            out[f"{tag}/voxel_mean"] = mu[..., 0]             # [T, N]
            out[f"{tag}/voxel_var"] = var[..., 0]
            out[f"{tag}/voxel_m4"] = m4[..., 0]
            out[f"{tag}/voxel_mean_last"] = mu[-1, :, 0]
            out[f"{tag}/voxel_var_last"] = var[-1, :, 0]
            out[f"{tag}/events_mean"] = ev.mean(0)
            out[f"{tag}/ntraj"] = np.int32(n)
            print("birth-death", tag, tots[:, -1, 0].mean(), ev.mean(0))
        np.savez_compressed(os.path.join(HERE, "nsm_birth_death.npz"), **out)

    if "rdme" in want:   # small 3-D RDME network
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

    if "rdme40" in want:   # the bench's 40^3 model, per-voxel sums at t = 1 and 5
        kw = dict(t_end=5.0, num_points=6, dt=1.0)
        m, tots, ev = moment_ensemble("config_rdme_3d", "_exact", 1000, 4040, kw, (1, 5))
        assert max(float(a.max()) for a in m) < 65536
        out = {"t_end": np.float64(5.0), "num_points": np.int32(6), "outputs": np.int32([1, 5]),
               "ntraj": np.int32(len(tots)),
               # uint16: the largest sum of x^4 over the 1,000 trajectories is 979
               "sum1": m[0].astype(np.uint16), "sum2": m[1].astype(np.uint16),
               "sum3": m[2].astype(np.uint16), "sum4": m[3].astype(np.uint16),
               "total_mean": tots.mean(0), "total_var": tots.var(0, ddof=1),
               "events_mean": ev.mean(0)}
        np.savez_compressed(os.path.join(HERE, "nsm_rdme40.npz"), **out)
        print("rdme40", tots[:, -1].mean(0), ev.mean(0))

    if "pins" in want:
        sys.path.insert(0, os.path.dirname(HERE))
        from chem_cases import flow_bcs, pinned_chem
        from coupled_cases import dam_break_chem
        out = {"static/C": oracle.ref_chem(pinned_chem()),
               "moving/C": oracle.ref_chem(dam_break_chem())}
        sc = flow_bcs(spacing_div=8, num_steps=41)
        for nsteps in (1, 5, 21, 41):
            x, v, rho = oracle.ref_sdpd(sc, nsteps)
            out[f"bcs/{nsteps}/x"] = x
            out[f"bcs/{nsteps}/v"] = v
            out[f"bcs/{nsteps}/rho"] = rho
        np.savez_compressed(os.path.join(HERE, "pins.npz"), **out)
        print("pins.npz written")

    if "coupled" in want:
        kw = dict(spacing_div=8, num_steps=60, num_outputs=4, network="full")
        out = {}
        procs = os.cpu_count() or 1
        for variant in ("", "_exact"):
            seeds = np.arange(3030, 3030 + 2000, dtype=np.uint64)
            chunks = [c for c in np.array_split(seeds, procs) if len(c)]
            with mp.get_context("spawn").Pool(len(chunks)) as pool:
                parts = pool.map(_coupled_worker, [(variant, c, kw) for c in chunks])
            m = [sum(p[0][k] for p in parts) for k in range(4)]
            tots = np.concatenate([p[1] for p in parts])
            ev = np.concatenate([p[2] for p in parts])
            n = len(tots)
            mu, var, m4 = central_moments(m, n)
            tag = variant.strip("_") or "stock"
            out[f"{tag}/mean"] = mu[..., 0]                   # [T, N]
            out[f"{tag}/var"] = var[..., 0]
            out[f"{tag}/m4"] = m4[..., 0]
            out[f"{tag}/total_mean"] = tots[..., 0].mean(0)
            out[f"{tag}/total_var"] = tots[..., 0].var(0, ddof=1)
            out[f"{tag}/events_mean"] = ev.mean(0)
            out[f"{tag}/ntraj"] = np.int32(n)
            print("coupled", tag, tots[:, -1, 0].mean(), ev.mean(0))
        np.savez_compressed(os.path.join(HERE, "nsm_coupled.npz"), **out)

    if "vtk" in want:
        out = {}
        for key, (sc, names) in vtk_cases().items():
            with mp.get_context("spawn").Pool(1) as pool:      # a fresh file counter
                st, files, bbox = pool.map(_vtk_worker, [key])[0]
            for k, f in enumerate(files):
                out[f"{key}/file{k}"] = np.frombuffer(f, np.uint8)
            out[f"{key}/bbox"] = np.frombuffer(bbox, np.uint8)
            for name, a in st.items():
                out[f"{key}/{name}"] = a
            out[f"{key}/type"] = sc.type
            out[f"{key}/mass"] = sc.mass
            out[f"{key}/names"] = np.array(names)
            out[f"{key}/chem_on"] = np.int32(bool(sc.enable_pde))
        np.savez_compressed(os.path.join(HERE, "vtk_ref.npz"), **out)
        print("vtk_ref.npz written")

    if "sdpd" in want:
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
