"""GPU parity of the moving domain with stochastic species: the SDPD flow
and, every step, the diffusion tables from the flow's lists, the volumes
m/rho and each trajectory's rebuilt event queue (simulate_threads.cpp:
232-281, simulate_rdme.cpp:53-68).  The flow, the tables and the event loop
are each bit-exact with the oracle, so whole runs are compared bit for bit:
counts, event counters and the flow state at every output."""
import numpy as np
import pytest

from spatialpy_gb300 import abi

from .conftest import golden
from .coupled_cases import dam_break_species

pytestmark = pytest.mark.gpu

SEEDS = np.arange(4, dtype=np.uint64) + 20260101


def _run(sc, prec, selection, seeds=SEEDS):
    from spatialpy_gb300.engine import Engine
    with Engine(sc, sdpd_precision=prec) as eng:
        res = eng.run(seeds, selection=selection, want_counts=True, want_particles=True)
        prof = eng.profile()
    assert res["rc"] == abi.SP_OK, res.get("error")
    return res, prof


@pytest.mark.parametrize("network", ["decay", "full"])
@pytest.mark.parametrize("prec,mode", [("f32", 6), ("f64", 2)])
@pytest.mark.parametrize("selection", [abi.SP_SELECT_EXACT, abi.SP_SELECT_REFERENCE])
def test_coupled_bitexact_vs_oracle(oracle_lib, network, prec, mode, selection):
    sc = dam_break_species(network=network)
    res, _ = _run(sc, prec, selection)
    out, ev, st, px, pr = oracle_lib.coupled_ensemble(
        sc, SEEDS, selection=selection, precision=prec, mode=mode, kmax=48)
    assert (st == 0).all()
    np.testing.assert_array_equal(res["events"], ev)
    for j in range(len(SEEDS)):
        np.testing.assert_array_equal(res["counts"][j], out[j], err_msg=f"trajectory {j}")
    x, v, rho = res["particles"][0]
    np.testing.assert_array_equal(x, px)
    np.testing.assert_array_equal(rho, pr)


@pytest.mark.parametrize("prec,mode", [("f32", 6), ("f64", 2)])
def test_coupled_2d_bitexact_vs_oracle(oracle_lib, prec, mode):
    """The flow + species path on a 2-D moving domain (xy-plane dam break,
    708 particles): trajectories, event counts and the flow bit for bit
    against the coupled oracle."""
    sc = dam_break_species(spacing_div=32, network="full", dims=2, molecules=1000)
    res, _ = _run(sc, prec, abi.SP_SELECT_EXACT)
    out, ev, st, px, pr = oracle_lib.coupled_ensemble(
        sc, SEEDS, selection=abi.SP_SELECT_EXACT, precision=prec, mode=mode, kmax=48)
    assert (st == 0).all()
    np.testing.assert_array_equal(res["events"], ev)
    for j in range(len(SEEDS)):
        np.testing.assert_array_equal(res["counts"][j], out[j], err_msg=f"trajectory {j}")
    x, v, rho = res["particles"][0]
    np.testing.assert_array_equal(x, px)
    np.testing.assert_array_equal(rho, pr)


def test_coupled_rerun_and_sequential_kernel(oracle_lib):
    """A second run restarts the flow from its initial state; the
    sequential event kernel gives the trajectories of the speculative batch
    kernels (chosen for these 4,056 voxels)."""
    from spatialpy_gb300.engine import Engine
    sc = dam_break_species(network="full", num_steps=30)
    a, pa = _run(sc, "f32", abi.SP_SELECT_EXACT)
    assert pa["kernel"].startswith("nsm_advance_batch")
    b, _ = _run(sc, "f32", abi.SP_SELECT_EXACT)
    with Engine(sc, nsm_variant=3) as eng:
        c = eng.run(SEEDS, want_counts=True)
        assert eng.profile()["kernel"] == "nsm_advance_small"
    for j in range(len(SEEDS)):
        np.testing.assert_array_equal(a["counts"][j], b["counts"][j])
        np.testing.assert_array_equal(a["counts"][j], c["counts"][j])


def test_coupled_solver_plugin():
    """GpuSolver on a moving domain with species: one Result per trajectory,
    shared flow state, counts only in fluid particles."""
    from spatialpy_gb300.solver import GpuSolver
    sc = dam_break_species(network="decay", num_steps=30)
    r = GpuSolver(sc).run(number_of_trajectories=2, seed=5)
    assert len(r) == 2 and r[0] != r[1]
    pts, data = r[1].read_step(len(sc.output_steps) - 1)
    assert not np.array_equal(pts, sc.x)                    # the flow moved
    assert data["D[S]"][sc.type == 2].sum() == 0
    assert r[0].get_species("S")[0].sum() == sc.u0.sum()


@pytest.mark.parametrize("variant", [4, 5])
def test_coupled_multiwarp_batches(oracle_lib, variant):
    """The coupled run with 2 or 4 warps per trajectory equals the oracle."""
    from spatialpy_gb300.engine import Engine
    sc = dam_break_species(network="full", num_steps=30)
    out, ev, st, _, _ = oracle_lib.coupled_ensemble(sc, SEEDS, want_particles=False)
    with Engine(sc, nsm_variant=variant) as eng:
        res = eng.run(SEEDS, want_counts=True)
    np.testing.assert_array_equal(res["events"], ev)
    for j in range(len(SEEDS)):
        np.testing.assert_array_equal(res["counts"][j], out[j])


@pytest.mark.parametrize("tag,selection", [("stock", abi.SP_SELECT_REFERENCE),
                                           ("exact", abi.SP_SELECT_EXACT)])
def test_coupled_vs_reference_ensembles(tag, selection):
    """4,000 GPU trajectories of the moving dam break with species (FP32
    flow) against 2,000 of the compiled engine, which runs the same flow in
    FP64 with its own random streams: totals inside 99.9% bands at every
    output, mean event counts within 5%, per particle and output mean and
    variance inside 99% bands (at least 97% / 96% of the cells holding 10 or
    more expected molecules: about 290, the particles the molecules reach).
    The exact-selection reference is the twin that also evaluates a
    diffusion destination's reactions with the destination's own volume, as
    exact selection does."""
    from .stats import band_fractions, moments_from_samples
    g = golden("nsm_coupled.npz")
    gn = int(g[f"{tag}/ntraj"])
    sc = dam_break_species(spacing_div=8, num_steps=60, num_outputs=4, network="full")
    n = 4000
    res, _ = _run(sc, "f32", selection, seeds=np.arange(n, dtype=np.uint64) + 4242)
    cnt = np.array(res["counts"])[..., 0]                      # [n, T, N]
    tot = cnt.sum(-1)
    se = np.sqrt(tot.var(0, ddof=1) / n + g[f"{tag}/total_var"] / gn)
    assert np.all(np.abs(tot.mean(0) - g[f"{tag}/total_mean"])[1:] <= 3.29 * se[1:])
    np.testing.assert_allclose(res["events"].mean(0), g[f"{tag}/events_mean"], rtol=0.05)
    ref = (g[f"{tag}/mean"], g[f"{tag}/var"], g[f"{tag}/m4"], gn)
    fm, fv, cells = band_fractions(moments_from_samples(cnt), ref, min_count=10)
    assert cells >= 250          # the molecules start on the top ~10% of the fluid
    assert fm >= 0.97 and fv >= 0.96, (fm, fv)
