"""CPU tests: the oracle restatement pinned against the reference engine's
golden vectors (tests/golden/, generated by make_golden.py from the compiled
reference) and against known answers."""
import math

import numpy as np
import pytest

from spatialpy_gb300 import abi
from spatialpy_gb300 import scenario as S

from .conftest import golden


def test_philox_known_answers(oracle_lib):
    """Random123 known-answer vectors for Philox4x32-10."""
    kat = [
        ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
        ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
        ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
         (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
    ]
    for ctr, key, want in kat:
        assert tuple(int(v) for v in oracle_lib.philox(ctr, key)) == want


def test_host_philox_matches_oracle(oracle_lib):
    from spatialpy_gb300.philox import philox4x32_10
    rng = np.random.default_rng(3)
    for _ in range(50):
        c = rng.integers(0, 2 ** 32, 4, dtype=np.uint64)
        k = rng.integers(0, 2 ** 32, 2, dtype=np.uint64)
        assert tuple(philox4x32_10(*c, *k)) == tuple(int(v) for v in oracle_lib.philox(c, k))


def test_neglog_accuracy(oracle_lib):
    for u in np.concatenate([np.geomspace(2 ** -33, 1 - 1e-12, 400), [0.5, 0.25, 0.7071]]):
        a = oracle_lib.neglog(float(u))
        b = -math.log(float(u))
        assert abs(a - b) <= 4e-16 * max(1.0, abs(b)), (u, a, b)


def test_neighbors_match_reference_golden(oracle_lib):
    fx = golden("neighbors.npz")
    keys = sorted({k.split("/")[0] for k in fx.files})
    assert len(keys) >= 6
    for key in keys:
        base = S.config_birth_death_2d()
        x = fx[f"{key}/x"]
        n = x.shape[0]
        sc = base.copy(x=x, type=np.ones(n), mass=fx[f"{key}/mass"], rho=fx[f"{key}/rho"],
                       nu=np.ones(n), fixed=np.ones(n), u0=np.zeros((n, 1)),
                       dimension=int(fx[f"{key}/dim"]), h=float(fx[f"{key}/h"]))
        cnt, idx, dist, dw, dij = oracle_lib.neighbors(sc, 256)
        np.testing.assert_array_equal(cnt, fx[f"{key}/count"], err_msg=key)
        for i in range(n):
            c = cnt[i]
            # ascending distance, ties by index
            assert np.all(np.diff(dist[i, :c]) >= 0)
            order = np.argsort(idx[i, :c], kind="stable")
            np.testing.assert_array_equal(idx[i, :c][order], fx[f"{key}/idx"][i, :c])
            for a, name in ((dist, "dist"), (dw, "dWdr"), (dij, "Dij")):
                np.testing.assert_array_equal(a[i, :c][order], fx[f"{key}/{name}"][i, :c],
                                              err_msg=f"{key}:{name}")


def _ensemble(sc, n, seed0, selection):
    out, ev, st, _ = oracle_lib_cached().nsm_ensemble(
        sc, np.arange(seed0, seed0 + n, dtype=np.uint64), selection)
    assert st.max() == 0
    return out, ev


_OL = None


def oracle_lib_cached():
    global _OL
    if _OL is None:
        import oracle
        oracle.build()
        _OL = oracle
    return _OL


def test_birth_death_exact_law(oracle_lib):
    """exact selection: immigration-death law mean 100, var 100(1-q)+100q(1-q)."""
    sc = S.config_birth_death_2d()
    n = 1000
    out, _ = _ensemble(sc, n, 20260101, abi.SP_SELECT_EXACT)
    tot = out.sum(axis=(2, 3))
    q = np.exp(-0.1 * sc.output_times())
    var = 100 * q * (1 - q) + 100 * (1 - q)
    assert np.all(np.abs(tot.mean(0)[1:] - 100) <= 3.29 * np.sqrt(var[1:] / n))
    sv = tot.var(0, ddof=1)
    assert np.all(np.abs(sv[1:] - var[1:]) <= 3.29 * var[1:] * np.sqrt(2 / (n - 1)))


@pytest.mark.parametrize("tag,selection", [("stock", abi.SP_SELECT_REFERENCE),
                                           ("exact", abi.SP_SELECT_EXACT)])
def test_birth_death_vs_reference_ensembles(oracle_lib, tag, selection):
    """Oracle ensembles (2,000 trajectories) against the reference's
    10,000-trajectory ensembles (stock engine / rescaled-selection engine):
    the total inside 99.9% bands at every output, mean event counts within
    5%, and per voxel and output the mean and the variance inside 99% bands
    (at least 97% of the 1,000 cells, 99% expected)."""
    from .stats import band_fractions, moments_from_samples
    g = golden("nsm_birth_death.npz")
    sc = S.config_birth_death_2d()
    n = 2000
    out, ev = _ensemble(sc, n, 5, selection)
    tot = out.sum(axis=(2, 3))
    gm, gv, gn = g[f"{tag}/total_mean"], g[f"{tag}/total_var"], int(g[f"{tag}/ntraj"])
    assert gn == 10000
    se = np.sqrt(tot.var(0, ddof=1) / n + gv / gn)
    assert np.all(np.abs(tot.mean(0) - gm)[1:] <= 3.29 * se[1:]), (tot.mean(0), gm)
    np.testing.assert_allclose(ev.mean(0), g[f"{tag}/events_mean"], rtol=0.05)
    ref = (g[f"{tag}/voxel_mean"], g[f"{tag}/voxel_var"], g[f"{tag}/voxel_m4"], gn)
    fm, fv, cells = band_fractions(moments_from_samples(out[..., 0]), ref)
    assert cells == 1000
    assert fm >= 0.97 and fv >= 0.97, (fm, fv)


@pytest.mark.parametrize("tag,selection", [("stock", abi.SP_SELECT_REFERENCE),
                                           ("exact", abi.SP_SELECT_EXACT)])
def test_rdme_vs_reference_ensembles(oracle_lib, tag, selection):
    g = golden("nsm_rdme_small.npz")
    sc = S.config_rdme_3d(n=6, nA=300, nB=300, t_end=10.0, num_points=11)
    n = 400
    out, ev = _ensemble(sc, n, 31337, selection)
    tot = out.sum(axis=2)
    gm, gv, gn = g[f"{tag}/total_mean"], g[f"{tag}/total_var"], int(g[f"{tag}/ntraj"])
    se = np.sqrt(tot.var(0, ddof=1) / n + gv / gn)
    assert np.all(np.abs(tot.mean(0) - gm)[1:] <= 3.29 * se[1:] + 1e-9)
    np.testing.assert_allclose(ev.mean(0), g[f"{tag}/events_mean"], rtol=0.05)


def test_sdpd_oracle_vs_reference_golden(oracle_lib):
    """FP64 SDPD oracle with the reference's neighbour semantics (moved query
    points against start-of-step points; Gauss-Seidel density reads) against
    the compiled engine, and the Jacobi variant used by the GPU."""
    g = golden("sdpd_small.npz")
    sc = S.config_dam_break(spacing_div=int(g["spacing_div"]), num_steps=41)
    for mode in (3, 2):
        st = oracle_lib.SdpdState(sc)
        done = 0
        for nsteps in (1, 5, 21, 41):
            oracle_lib.sdpd(sc, st, nsteps - done, "f64", mode)
            done = nsteps
            rx, rv, rr = g[f"{nsteps}/x"], g[f"{nsteps}/v"], g[f"{nsteps}/rho"]
            assert np.abs(st.x - rx).max() <= 1e-12
            assert np.linalg.norm(st.v - rv) <= 1e-9 * max(np.linalg.norm(rv), 1e-30)
            assert np.abs(st.rho - rr).max() <= 1e-12


def test_sdpd_f32_tracks_f64_over_1000_steps(oracle_lib):
    """The FP32 flow computes in float but stores positions as float pairs
    hi + lo and densities as deviations from rho0.  After 1,000 steps of the
    1,368-particle dam break, against FP64 with the same self-pair rule
    (mode 6), its positions and velocities are within 1e-5 norm-wise
    relative (measured 1.4e-9 and 1.2e-6; plain float storage gave 4.5e-7
    and 2.8e-4).  The state kept between calls makes 25 calls of 40 steps
    equal one call of 1,000."""
    sc = S.config_dam_break(spacing_div=8, num_steps=1000)
    a = oracle_lib.sdpd(sc, oracle_lib.SdpdState(sc), 1000, "f64", 6)
    b = oracle_lib.SdpdState(sc)
    for _ in range(25):
        oracle_lib.sdpd(sc, b, 40, "f32", 6)
    c = oracle_lib.sdpd(sc, oracle_lib.SdpdState(sc), 1000, "f32", 6)
    np.testing.assert_array_equal(b.x, c.x)
    np.testing.assert_array_equal(b.v, c.v)
    assert np.linalg.norm(a.x - b.x) <= 1e-5 * np.linalg.norm(a.x)
    assert np.linalg.norm(a.v - b.v) <= 1e-5 * np.linalg.norm(a.v)
    assert np.abs(a.rho - b.rho).max() <= 1e-6


def test_sdpd_self_pair_rule_is_a_discontinuity(oracle_lib):
    """A moved particle meets its own start-of-step point (the reference
    searches a kd-tree of start-of-step points).  With double positions the
    pair is absent when the step rounds away.  Particle 333 (a corner of the
    fluid block) takes a step of pure rounding noise at step 1 (bounced
    velocity plus half a step of gravity cancel; its background-pressure
    force sums a symmetric neighbourhood): mode 2 (positions, the reference)
    drops its self pair, mode 6 (the step |dt vt|) keeps it.  Both are FP64;
    after 1,000 steps their velocities differ by 1.2e-4, so the flow is
    defined only to that level by this choice, whatever the precision."""
    sc = S.config_dam_break(spacing_div=8, num_steps=1000)
    a = oracle_lib.sdpd(sc, oracle_lib.SdpdState(sc), 2, "f64", 2)
    b = oracle_lib.sdpd(sc, oracle_lib.SdpdState(sc), 2, "f64", 6)
    assert (a.nbr_count[333], b.nbr_count[333]) == (18, 19)
    assert int((a.nbr_count != b.nbr_count).sum()) == 2
    oracle_lib.sdpd(sc, a, 998, "f64", 2)
    oracle_lib.sdpd(sc, b, 998, "f64", 6)
    assert np.linalg.norm(a.v - b.v) > 1e-5 * np.linalg.norm(a.v)


def test_coupled_oracle_flow_and_species(oracle_lib):
    """Moving domain with species (simulate_rdme.cpp:53-68 on a non-static
    domain): the flow part equals the plain SDPD oracle stepped to each
    output; molecules stay in the fluid (walls have D = 0); with diffusion
    only the total is conserved; a rerun repeats every count."""
    from .coupled_cases import dam_break_species
    sc = dam_break_species(network="none", num_steps=41, num_outputs=3)
    seeds = np.arange(3, dtype=np.uint64) + 11
    out, ev, st, px, pr = oracle_lib.coupled_ensemble(sc, seeds)
    assert (st == 0).all() and (ev[:, 1] > 0).all() and (ev[:, 0] == 0).all()
    np.testing.assert_array_equal(out.sum(axis=(2, 3)), sc.u0.sum())
    assert out[:, :, sc.type == 2].sum() == 0
    flow = oracle_lib.SdpdState(sc)
    done = 0
    for k, step in enumerate(sc.output_steps):
        oracle_lib.sdpd(sc, flow, int(step) - done, "f32", 6, kmax=48)
        done = int(step)
        np.testing.assert_array_equal(px[k], flow.x)
        np.testing.assert_array_equal(pr[k], flow.rho)
    out2, ev2, _, _, _ = oracle_lib.coupled_ensemble(sc, seeds)
    np.testing.assert_array_equal(out, out2)
    np.testing.assert_array_equal(ev, ev2)


def test_chemistry_oracle_vs_compiled_reference(oracle_lib):
    """The deterministic chemistry against the compiled engine
    (tests/golden/pins.npz): a static lattice with a concentration boundary
    condition, and the moving dam break (FP64 flow, both neighbour modes):
    concentrations within 1e-12 of the largest at every output (measured
    2.8e-16 and 9e-21).  The cases are ones on which the engine's transposed
    reads of the diffusion matrix and stoichiometry (model.cpp:165, 186)
    agree with the layouts written (tests/chem_cases.py pinned_chem)."""
    from .chem_cases import pinned_chem
    from .coupled_cases import dam_break_chem
    g = golden("pins.npz")
    want = g["static/C"]
    got = oracle_lib.chem_static(pinned_chem())
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    assert np.abs(want[-1] - want[0]).max() > 0.5
    want = g["moving/C"]
    for mode in (2, 3):
        ch = oracle_lib.coupled_ensemble(dam_break_chem(), np.arange(1, dtype=np.uint64),
                                         precision="f64", mode=mode, want_chem=True)[5]
        assert np.abs(ch - want).max() <= 1e-12 * np.abs(want).max()


def test_flow_boundary_conditions_vs_compiled_reference(oracle_lib):
    """The dam break with boundary conditions on v, nu and rho against the
    compiled engine running the same conditions (applyBoundaryConditions as
    boundarycondition.py:121-167 generates it): FP64 oracle states after 1,
    5, 21 and 41 steps within 1e-12 (positions, densities) and 1e-9
    norm-wise (velocities), in the reference's neighbour mode and the GPU's."""
    from .chem_cases import flow_bcs
    g = golden("pins.npz")
    sc = flow_bcs(spacing_div=8, num_steps=41)
    for mode in (3, 2):
        st = oracle_lib.SdpdState(sc)
        done = 0
        for n in (1, 5, 21, 41):
            oracle_lib.sdpd(sc, st, n - done, "f64", mode)
            done = n
            rv = g[f"bcs/{n}/v"]
            assert np.abs(st.x - g[f"bcs/{n}/x"]).max() <= 1e-12
            assert np.linalg.norm(st.v - rv) <= 1e-9 * np.linalg.norm(rv)
            assert np.abs(st.rho - g[f"bcs/{n}/rho"]).max() <= 1e-12


@pytest.mark.parametrize("tag,selection", [("stock", abi.SP_SELECT_REFERENCE),
                                           ("exact", abi.SP_SELECT_EXACT)])
def test_coupled_oracle_vs_reference_ensembles(oracle_lib, tag, selection):
    """Moving dam break with species (1,368 particles, network "full", 60
    steps; FP32 flow as on the GPU) against 2,000 trajectories of the
    compiled engine (stock / rescaled selection): totals inside 99.9% bands
    at every output, mean event counts within 5%, and per particle and
    output mean and variance inside 99% bands (at least 97% / 96% of the
    cells holding 10 or more expected molecules: about 290 cells, the
    particles the molecules reach).  The exact-selection reference is the
    twin that also evaluates a diffusion destination's reactions with the
    destination's own volume, as exact selection does."""
    from .coupled_cases import dam_break_species
    from .stats import band_fractions, moments_from_samples
    g = golden("nsm_coupled.npz")
    gn = int(g[f"{tag}/ntraj"])
    sc = dam_break_species(spacing_div=8, num_steps=60, num_outputs=4, network="full")
    n = 1000
    out, ev, st, _, _ = oracle_lib.coupled_ensemble(sc, np.arange(n, dtype=np.uint64) + 77,
                                                    selection=selection, want_particles=False)
    assert (st == 0).all()
    tot = out[..., 0].sum(-1)
    se = np.sqrt(tot.var(0, ddof=1) / n + g[f"{tag}/total_var"] / gn)
    assert np.all(np.abs(tot.mean(0) - g[f"{tag}/total_mean"])[1:] <= 3.29 * se[1:])
    np.testing.assert_allclose(ev.mean(0), g[f"{tag}/events_mean"], rtol=0.05)
    ref = (g[f"{tag}/mean"], g[f"{tag}/var"], g[f"{tag}/m4"], gn)
    fm, fv, cells = band_fractions(moments_from_samples(out[..., 0]), ref, min_count=10)
    assert cells >= 250          # the molecules start on the top ~10% of the fluid
    assert fm >= 0.97 and fv >= 0.96, (fm, fv)


def test_chem_oracle_conserves_and_integrates(oracle_lib):
    """Deterministic chemistry (model.cpp:151-189): SPH diffusion alone keeps
    the total of C; a zero-order ODE rate k adds k*dt per step to every
    particle of its type; a boundary condition pins its concentrations.""" 
    from .chem_cases import static_chem
    sc = static_chem(reactions="none", bcs=False)
    out = oracle_lib.chem_static(sc)
    tot = out.sum(axis=1)
    np.testing.assert_allclose(tot, np.broadcast_to(tot[0], tot.shape), rtol=1e-12)
    assert np.abs(out[-1] - out[0]).max() > 0.1           # it diffused
    sc2 = static_chem(reactions="birth")
    sc2 = sc2.copy(u0=np.zeros_like(sc2.u0))
    out2 = oracle_lib.chem_static(sc2)
    n1 = int((sc2.type == 1).sum())
    steps = sc2.output_steps
    # the first half step of step 0 has no fluxes yet (simulate.cpp:81), so
    # the total lags k*N1*t by half a step
    want = np.where(steps > 0, 3.0 * n1 * (sc2.dt * steps - 0.5 * sc2.dt), 0.0)
    np.testing.assert_allclose(out2[:, :, 0].sum(axis=1), want, rtol=1e-9)
    top = sc2.x[:, 1] > 0.8
    assert np.all(out2[1:, top, 1] == 4.0)
