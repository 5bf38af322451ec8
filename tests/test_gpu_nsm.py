"""GPU NSM parity: libspgpu trajectories against the oracle and the reference.

The GPU engine and the oracle (oracle/sp_oracle.c) consume the same Philox
streams and round every double-precision operation alike, so counts must be
identical event for event (bit-exact integer parity).  Against the compiled
reference engine (mt19937_64 streams) parity is statistical: ensemble means
and variances inside 99% bands of the reference ensembles in tests/golden/.
"""
import numpy as np
import pytest

from spatialpy_gb300 import abi
from spatialpy_gb300 import scenario as S

from .conftest import golden

pytestmark = pytest.mark.gpu


def _engine(scs, **kw):
    from spatialpy_gb300.engine import Engine
    return Engine(scs, **kw)


def _dimer_model():
    sc = S.config_birth_death_2d(n=6, count=40, t_end=4.0, num_points=5)
    rate, kind, reac, allowed, jcN, irN, prN = S.mass_action(
        ["A", "B"],
        [(5.0, {}, {"A": 1}, None), (0.02, {"A": 2}, {"B": 1}, None),
         (0.3, {"B": 1}, {"A": 2}, None), (0.05, {"A": 1, "B": 1}, {}, None)], 1)
    u0 = np.zeros((sc.num_particles, 2), np.uint32)
    u0[:, 0] = sc.u0[:, 0]
    u0[3, 1] = 7
    return sc.copy(species=["A", "B"], rxn_rate=rate, rxn_kind=kind, rxn_reactants=reac,
                   rxn_allowed=allowed, jcN=jcN, irN=irN, prN=prN,
                   diffusion=np.array([[0.2], [0.05]]), u0=u0, name="dimer")


def _restricted_model():
    """Two types; species A may not enter type 2; birth only in type 2."""
    sc = S.config_rdme_3d(n=5, nA=60, nB=60, t_end=5.0, num_points=6, dims=2)
    diff = sc.diffusion.copy()
    diff[0, 1] = 0.0          # D(A, type 2) = 0: no A moves into type 2
    return sc.copy(diffusion=diff, name="restricted")


CASES = {
    "birth_death": lambda: S.config_birth_death_2d(),
    "rdme3d_6": lambda: S.config_rdme_3d(n=6, nA=300, nB=300, t_end=10.0, num_points=11),
    "rdme2d_12": lambda: S.config_rdme_3d(n=12, nA=200, nB=150, t_end=6.0, num_points=7, dims=2),
    "dimer": _dimer_model,
    "restricted": _restricted_model,
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("selection", [abi.SP_SELECT_EXACT, abi.SP_SELECT_REFERENCE])
def test_trajectories_bitexact_vs_oracle(oracle_lib, case, selection):
    sc = CASES[case]()
    seeds = np.arange(1000, 1008, dtype=np.uint64) * 7919
    with _engine(sc) as eng:
        res = eng.run(seeds, selection=selection)
    assert res["rc"] == abi.SP_OK, res.get("error")
    for j, s in enumerate(seeds):
        out, ev, st = oracle_lib.nsm_trajectory(sc, int(s), selection)
        assert st == 0
        np.testing.assert_array_equal(res["counts"][j], out, err_msg=f"{case} traj {j}")
        np.testing.assert_array_equal(res["events"][j], ev)


def _wide_model():
    """10 species, 12 reactions: runs the generic (shared-table) kernel."""
    sc = S.config_birth_death_2d(n=5, count=0, t_end=3.0, num_points=4)
    sp = [f"X{i}" for i in range(10)]
    rx = [(2.0, {}, {"X0": 1}, None)]
    for i in range(9):
        rx.append((0.5, {f"X{i}": 1}, {f"X{i+1}": 1}, None))
    rx.append((0.01, {"X9": 2}, {"X0": 1}, None))
    rx.append((0.002, {"X3": 1, "X7": 1}, {}, None))
    rate, kind, reac, allowed, jcN, irN, prN = S.mass_action(sp, rx, 1)
    u0 = np.zeros((sc.num_particles, 10), np.uint32)
    u0[:, 0] = 3
    u0[7, 5] = 20
    return sc.copy(species=sp, rxn_rate=rate, rxn_kind=kind, rxn_reactants=reac,
                   rxn_allowed=allowed, jcN=jcN, irN=irN, prN=prN,
                   diffusion=np.linspace(0.05, 0.5, 10).reshape(10, 1), u0=u0, name="wide")


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("case", ["rdme3d_6", "dimer", "wide", "birth_death", "restricted"])
def test_kernel_variants_bitexact(oracle_lib, case, variant):
    sc = _wide_model() if case == "wide" else CASES[case]()
    seeds = np.arange(4, dtype=np.uint64) + 424242
    with _engine(sc, nsm_variant=variant) as eng:
        res = eng.run(seeds, selection=abi.SP_SELECT_EXACT)
    assert res["rc"] == abi.SP_OK, res.get("error")
    for j, s in enumerate(seeds):
        out, ev, _ = oracle_lib.nsm_trajectory(sc, int(s), 0)
        np.testing.assert_array_equal(res["counts"][j], out)
        np.testing.assert_array_equal(res["events"][j], ev)


_ORACLE_RUNS = {}


def _oracle_run(oracle_lib, key, sc, seed, selection):
    k = (key, seed, selection)
    if k not in _ORACLE_RUNS:
        _ORACLE_RUNS[k] = oracle_lib.nsm_trajectory(sc, seed, selection)
    return _ORACLE_RUNS[k]


@pytest.mark.parametrize("variant", [2, 4, 5])
@pytest.mark.parametrize("selection", [abi.SP_SELECT_EXACT, abi.SP_SELECT_REFERENCE])
@pytest.mark.parametrize("n,dims", [(16, 3), (64, 2)])
def test_batch_kernel_bitexact_large_domain(oracle_lib, n, dims, selection, variant):
    """Speculative batches on 4,096-voxel domains (one warp and 32 events,
    two warps and 64, four warps and 128 per trajectory) equal the
    sequential oracle event for event (both selection rules)."""
    t_end = 2.0 if dims == 3 else 0.2
    sc = S.config_rdme_3d(n=n, nA=3000, nB=2500, t_end=t_end, num_points=5, dt=t_end / 4,
                          dims=dims)
    seeds = np.arange(6, dtype=np.uint64) + 99173
    with _engine(sc, nsm_variant=variant) as eng:
        res = eng.run(seeds, selection=selection)
        kernel = eng.profile()["kernel"]
    assert kernel == {2: "nsm_advance_batch", 4: "nsm_advance_batchw2",
                      5: "nsm_advance_batchw4"}[variant]
    assert res["rc"] == abi.SP_OK, res.get("error")
    for j, s in enumerate(seeds):
        out, ev, _ = _oracle_run(oracle_lib, (n, dims), sc, int(s), selection)
        np.testing.assert_array_equal(res["events"][j], ev)
        np.testing.assert_array_equal(res["counts"][j], out)


@pytest.mark.parametrize("variant", [2, 4, 5])
def test_batch_kernel_birth_death_large(oracle_lib, variant):
    sc = S.config_birth_death_2d(n=64, count=3000, k_birth=2000.0, D=1e-4, t_end=0.5,
                                 num_points=3, dt=0.25)
    seeds = np.arange(4, dtype=np.uint64) + 5
    with _engine(sc, nsm_variant=variant) as eng:
        res = eng.run(seeds)
    for j, s in enumerate(seeds):
        out, ev, _ = _oracle_run(oracle_lib, "bd64", sc, int(s), 0)
        np.testing.assert_array_equal(res["events"][j], ev)
        np.testing.assert_array_equal(res["counts"][j], out)


def test_stepwise_run_equals_run():
    sc = S.config_rdme_3d(n=6, nA=300, nB=300, t_end=10.0, num_points=11)
    seeds = np.arange(16, dtype=np.uint64) + 5
    with _engine(sc) as eng:
        a = eng.run(seeds, want_moments=True)
        eng.start(seeds, want_counts=True, want_moments=True)
        for _ in range(10):
            eng.advance(1)
        b = eng.finish()
    for x, y in zip(a["counts"], b["counts"]):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(a["moments"][0], b["moments"][0])
    np.testing.assert_array_equal(a["events"], b["events"])


def test_budget_exhaustion_resumes_exactly(oracle_lib):
    """A tiny per-launch event budget forces many resumable exits
    (SP_TRAJ_BUDGET_EXHAUSTED); the host relaunches and the trajectory is
    unchanged."""
    sc = S.config_birth_death_2d(n=6, count=50, t_end=3.0, num_points=4)
    seeds = np.arange(3, dtype=np.uint64) + 77
    with _engine(sc, event_budget=17) as eng:
        res = eng.run(seeds)
    assert res["rc"] == abi.SP_OK
    for j, s in enumerate(seeds):
        out, ev, _ = oracle_lib.nsm_trajectory(sc, int(s), 0)
        np.testing.assert_array_equal(res["counts"][j], out)


def test_uneven_batch_bitexact(oracle_lib):
    scs = [S.config_birth_death_2d(n=7, count=30),
           S.config_birth_death_2d(n=23, count=300, k_birth=3.0),
           S.config_birth_death_2d(n=2, count=5, D=1.0)]
    inst = np.array([1, 0, 2, 1, 1, 0, 2, 2], np.int32)
    seeds = np.arange(50, 58, dtype=np.uint64)
    with _engine(scs) as eng:
        res = eng.run(seeds, instance=inst, want_moments=True)
    assert res["rc"] == abi.SP_OK, res.get("error")
    for j, s in enumerate(seeds):
        out, ev, _ = oracle_lib.nsm_trajectory(scs[inst[j]], int(s), 0)
        np.testing.assert_array_equal(res["counts"][j], out)
        np.testing.assert_array_equal(res["events"][j], ev)
    # moments are exact integer sums over each instance's trajectories
    for i in range(3):
        xs = np.array([res["counts"][j] for j in range(len(seeds)) if inst[j] == i], np.int64)
        np.testing.assert_array_equal(res["moments"][i][..., 0], xs.sum(0))
        np.testing.assert_array_equal(res["moments"][i][..., 1], (xs * xs).sum(0))


def test_rerun_is_bit_identical():
    sc = S.config_rdme_3d(n=6, nA=300, nB=300, t_end=10.0, num_points=11)
    seeds = np.arange(32, dtype=np.uint64) + 99
    with _engine(sc) as eng:
        a = eng.run(seeds)
        b = eng.run(seeds)
    for x, y in zip(a["counts"], b["counts"]):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(a["events"], b["events"])


def test_output0_is_u0_and_empty_domain():
    sc = S.config_birth_death_2d(count=0, k_birth=0.0)
    with _engine(sc) as eng:
        res = eng.run(np.arange(4, dtype=np.uint64))
    for c in res["counts"]:
        assert c.sum() == 0
    assert res["events"].sum() == 0
    sc = S.config_birth_death_2d()
    with _engine(sc) as eng:
        res = eng.run(np.arange(4, dtype=np.uint64))
    for c in res["counts"]:
        np.testing.assert_array_equal(c[0], sc.u0)      # test_solver.py:127-131


def test_neighbors_bitexact(oracle_lib):
    fx = golden("neighbors.npz")
    keys = sorted({k.split("/")[0] for k in fx.files})
    for key in keys:
        base = S.config_birth_death_2d()
        x = fx[f"{key}/x"]
        n = x.shape[0]
        sc = base.copy(x=x, type=np.ones(n), mass=fx[f"{key}/mass"], rho=fx[f"{key}/rho"],
                       nu=np.ones(n), fixed=np.ones(n), u0=np.zeros((n, 1)),
                       dimension=int(fx[f"{key}/dim"]), h=float(fx[f"{key}/h"]))
        kmax = 256
        with _engine(sc) as eng:
            cnt, idx, dist, dw, dij = eng.neighbors(0, kmax)
        o = oracle_lib.neighbors(sc, kmax)
        # identical lists and order against the oracle
        np.testing.assert_array_equal(cnt, o[0], err_msg=key)
        for a, b in zip((idx, dist, dw, dij), o[1:]):
            np.testing.assert_array_equal(a, b, err_msg=key)
        # identical sets and values against the reference engine
        np.testing.assert_array_equal(cnt, fx[f"{key}/count"], err_msg=key)
        for i in range(n):
            c = cnt[i]
            order = np.argsort(idx[i, :c], kind="stable")
            np.testing.assert_array_equal(idx[i, :c][order], fx[f"{key}/idx"][i, :c])
            for a, name in ((dist, "dist"), (dw, "dWdr"), (dij, "Dij")):
                np.testing.assert_array_equal(a[i, :c][order], fx[f"{key}/{name}"][i, :c],
                                              err_msg=f"{key}:{name}:{i}")


def test_ddiag_bitexact(oracle_lib):
    for sc in (_restricted_model(), S.config_rdme_3d(n=6, nA=10, nB=10)):
        with _engine(sc) as eng:
            dd = eng.ddiag(0)
        cnt, idx, dist, dw, dij = oracle_lib.neighbors(sc, 64)
        odd, _ = oracle_lib.diffusion_tables(sc, cnt, idx, dij)
        np.testing.assert_array_equal(dd, odd)


def test_birth_death_exact_statistics():
    """1,000 trajectories: the total follows the immigration-death law
    mean(t) = 100 (k_b V / k_d with V = 1 and 100 initial molecules) and
    var(t) = 100 e^{-t/10}(1-e^{-t/10}) + 100 (1-e^{-t/10})."""
    sc = S.config_birth_death_2d()
    n = 1000
    with _engine(sc) as eng:
        tot = np.array([c.sum(axis=(1, 2)) for c in
                        eng.run(np.arange(n, dtype=np.uint64) + 20260101)["counts"]])
    t = sc.output_times()
    q = np.exp(-0.1 * t)
    var = 100 * q * (1 - q) + 100 * (1 - q)
    mean = tot.mean(0)
    # 99% joint bands over the 10 outputs (99.9% each)
    band = 3.29 * np.sqrt(np.maximum(var, 1e-9) / n)
    assert np.all(np.abs(mean[1:] - 100.0) <= band[1:] + 1e-12), (mean, band)
    sv = tot.var(0, ddof=1)
    vband = 3.29 * var * np.sqrt(2.0 / (n - 1))
    assert np.all(np.abs(sv[1:] - var[1:]) <= vband[1:]), (sv, var)


@pytest.mark.parametrize("tag,selection", [("stock", abi.SP_SELECT_REFERENCE),
                                           ("exact", abi.SP_SELECT_EXACT)])
def test_per_voxel_moments_vs_10000_reference_trajectories(tag, selection):
    """10,000 GPU trajectories of the spatial birth-death model against the
    reference engine's 10,000 (stock engine for the reused-uniform selection,
    rescaled twin for exact selection): per voxel and output (100 x 10
    cells), mean and variance inside 99% bands for at least 97% of the cells
    (99% expected); the total inside 99.9% bands at every output."""
    from .stats import band_fractions, moments_from_samples
    g = golden("nsm_birth_death.npz")
    gn = int(g[f"{tag}/ntraj"])
    assert gn == 10000
    sc = S.config_birth_death_2d()
    n = 10000
    with _engine(sc) as eng:
        res = eng.run(np.arange(n, dtype=np.uint64) + 7, selection=selection)
    cnt = np.array(res["counts"])[..., 0]                     # [n, T, N]
    tot = cnt.sum(-1)
    gm, gv = g[f"{tag}/total_mean"], g[f"{tag}/total_var"]
    se = np.sqrt(tot.var(0, ddof=1) / n + gv / gn)
    assert np.all(np.abs(tot.mean(0) - gm)[1:] <= 3.29 * se[1:]), (tot.mean(0), gm)
    ref = (g[f"{tag}/voxel_mean"], g[f"{tag}/voxel_var"], g[f"{tag}/voxel_m4"], gn)
    fm, fv, cells = band_fractions(moments_from_samples(cnt), ref)
    assert cells == 1000
    assert fm >= 0.97 and fv >= 0.97, (fm, fv)


def _bench_model(t_end, num_points):
    # the bench's workload: 40^3 lattice, A+B<->C, 0->A (x < 0.1), C->0,
    # 10,000 A and 10,000 B scattered once
    return S.config_rdme_3d(t_end=t_end, num_points=num_points, dt=1.0)


@pytest.mark.parametrize("variant", [0, 5])
def test_bench_workload_bitexact(oracle_lib, variant):
    """The bench's own model (64,000 voxels) on the kernel it is timed on:
    the default policy and the forced 4-warp speculative batch kernel give,
    for 6 trajectories over two output intervals (about 180,000 events each),
    the oracle's counts and event numbers exactly."""
    sc = _bench_model(2.0, 3)
    seeds = np.arange(6, dtype=np.uint64) + 20260101
    with _engine(sc, nsm_variant=variant) as eng:
        res = eng.run(seeds)
        kernel = eng.profile()["kernel"]
    assert kernel == "nsm_advance_batchw4", kernel
    for j, s in enumerate(seeds):
        out, ev, _ = oracle_lib.nsm_trajectory(sc, int(s), 0)
        np.testing.assert_array_equal(res["events"][j], ev, err_msg=f"trajectory {j}")
        np.testing.assert_array_equal(res["counts"][j], out, err_msg=f"trajectory {j}")


def test_bench_workload_per_voxel_vs_reference():
    """The bench's model against 1,000 trajectories of the reference engine
    (rescaled selection) over t = 0..5: species totals inside 99.9% bands at
    every output, and per voxel, species and output (t = 1 and 5; 64,000 x 3
    x 2 cells) mean and variance inside 99% bands, from 1,000 GPU
    trajectories summed on the device.  Cells holding fewer than 10 expected
    molecules over an ensemble are discrete and left out (about 150,000
    cells remain); the bar is 97% of cells for means and 96% for variances
    (the sample variance of small counts is skewed: 300 oracle trajectories
    gave 98.7% and 97.8%)."""
    from .stats import band_fractions, moments_from_sums
    g = golden("nsm_rdme40.npz")
    gn = int(g["ntraj"])
    sc = _bench_model(float(g["t_end"]), int(g["num_points"]))
    n = 1000
    with _engine(sc) as eng:
        res = eng.run(np.arange(n, dtype=np.uint64) + 99991, want_counts=False,
                      want_moments=True)
    mom = res["moments"][0].astype(np.float64)                # [T, N, S, 2]
    outs = list(g["outputs"])
    s1, s2 = mom[outs, ..., 0], mom[outs, ..., 1]
    mu = s1 / n
    var = (s2 / n - mu * mu) * n / (n - 1)
    ref = moments_from_sums(g["sum1"], g["sum2"], g["sum3"], g["sum4"], gn)
    fm, fv, cells = band_fractions(ref, (mu, var, None, n), min_count=10)
    assert cells > 100000
    assert fm >= 0.97 and fv >= 0.96, (fm, fv)
    # totals: the mean of the total is the sum of the voxel means; its
    # variance needs per-trajectory totals, which the sums do not give, so
    # the band uses the reference's variance for both sides
    tot = mom[..., 0].sum(axis=1) / n                          # [T, S]
    se = np.sqrt(g["total_var"] / gn + g["total_var"] / n)
    assert np.all(np.abs(tot - g["total_mean"])[1:] <= 3.29 * se[1:] + 1e-9)


def test_exact_mode_matches_rescaled_reference_ensemble():
    g = golden("nsm_rdme_small.npz")
    sc = S.config_rdme_3d(n=6, nA=300, nB=300, t_end=10.0, num_points=11)
    n = 400
    for tag, sel in (("exact", abi.SP_SELECT_EXACT), ("stock", abi.SP_SELECT_REFERENCE)):
        with _engine(sc) as eng:
            res = eng.run(np.arange(n, dtype=np.uint64) + 31337, selection=sel)
        tot = np.array([c.sum(axis=1) for c in res["counts"]])      # [n, T, S]
        m, v = tot.mean(0), tot.var(0, ddof=1)
        gm, gv, gn = g[f"{tag}/total_mean"], g[f"{tag}/total_var"], int(g[f"{tag}/ntraj"])
        se = np.sqrt(v / n + gv / gn)
        assert np.all(np.abs(m - gm)[1:] <= 3.29 * se[1:] + 1e-9), (tag, m, gm)


def test_mixed_kernel_groups_bitexact(oracle_lib):
    """Domains of >= 2,048 voxels go to the speculative batch kernel and the
    others to the sequential kernel, launched concurrently, each group in
    descending order of total propensity; trajectories stay bit-exact."""
    scs = [S.config_birth_death_2d(n=50, count=200, D=0.02, t_end=2.0, num_points=3, dt=1.0),
           S.config_birth_death_2d(n=7, count=30, t_end=2.0, num_points=3, dt=1.0),
           S.config_birth_death_2d(n=64, count=100, D=0.02, t_end=2.0, num_points=3, dt=1.0)]
    inst = np.array([0, 1, 2, 1, 0, 2, 1], np.int32)
    seeds = np.arange(70, 77, dtype=np.uint64)
    with _engine(scs) as eng:
        res = eng.run(seeds, instance=inst)
        assert eng.profile()["kernel"] == "nsm_advance_batch+nsm_advance_small"
    assert res["rc"] == abi.SP_OK, res.get("error")
    for j, s in enumerate(seeds):
        out, ev, _ = oracle_lib.nsm_trajectory(scs[inst[j]], int(s), 0)
        np.testing.assert_array_equal(res["counts"][j], out, err_msg=f"trajectory {j}")
        np.testing.assert_array_equal(res["events"][j], ev)


def test_skewed_ensemble_bitexact(oracle_lib):
    """An ensemble whose largest initial total propensity is at least 8x its
    90th percentile (40 heavy trajectories among 600 light ones on domains
    of 2,304 voxels, and 20 small domains) runs in one group on the 2-warp
    batch kernel, heaviest first: its time is that of its heaviest chains.
    Every trajectory stays bit-exact, small domains included."""
    kw = dict(t_end=0.01, num_points=3, dt=0.005)
    scs = [S.config_birth_death_2d(n=48, count=2000, D=0.5, **kw),    # heavy, 2,304 voxels
           S.config_birth_death_2d(n=48, count=100, D=0.02, **kw),    # light, 2,304 voxels
           S.config_birth_death_2d(n=7, count=30, **kw)]              # small, 49 voxels
    inst = np.array([0] * 40 + [1] * 600 + [2] * 20, np.int32)
    inst = np.random.default_rng(3).permutation(inst)
    seeds = np.arange(900, 900 + len(inst), dtype=np.uint64)
    with _engine(scs) as eng:
        res = eng.run(seeds, instance=inst)
        kernel = eng.profile()["kernel"]
    assert res["rc"] == abi.SP_OK, res.get("error")
    assert kernel == "nsm_advance_batchw2"
    check = [j for j in range(len(inst)) if inst[j] == 0][:10]
    check += [j for j in range(len(inst)) if inst[j] == 1][:12]
    check += [j for j in range(len(inst)) if inst[j] == 2][:6]
    for j in check:
        out, ev, _ = oracle_lib.nsm_trajectory(scs[inst[j]], int(seeds[j]), 0)
        np.testing.assert_array_equal(res["counts"][j], out, err_msg=f"trajectory {j}")
        np.testing.assert_array_equal(res["events"][j], ev)


def test_warp_tuner_keeps_trajectories(oracle_lib):
    """With the default policy a long run tries 4, 2 and 1 warps per
    trajectory on its first intervals and keeps the fastest; the events are
    those of the sequential oracle whichever width runs."""
    sc = S.config_rdme_3d(n=16, nA=3000, nB=2500, t_end=1.0, num_points=11, dt=0.1)
    seeds = np.arange(5, dtype=np.uint64) + 4242
    with _engine(sc) as eng:
        res = eng.run(seeds)
        kernel = eng.profile()["kernel"]
    assert kernel in ("nsm_advance_batch", "nsm_advance_batchw2", "nsm_advance_batchw4")
    for j, s in enumerate(seeds):
        out, ev, _ = oracle_lib.nsm_trajectory(sc, int(s), 0)
        np.testing.assert_array_equal(res["events"][j], ev)
        np.testing.assert_array_equal(res["counts"][j], out)
