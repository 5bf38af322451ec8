"""GPU parity of deterministic chemistry (enable_pde) and boundary
conditions: the concentrations C of a static domain and of a moving one, and
a flow with boundary conditions on v, nu and rho, compared bit for bit with
the oracle (same operations, same order, no FMA contraction)."""
import numpy as np
import pytest

from spatialpy_gb300 import abi
from spatialpy_gb300 import scenario as S

from .chem_cases import flow_bcs, pinned_chem, static_chem
from .conftest import golden
from .coupled_cases import dam_break_chem, dam_break_species

pytestmark = pytest.mark.gpu


def test_static_chemistry_bitexact(oracle_lib):
    from spatialpy_gb300.engine import Engine
    sc = static_chem()
    with Engine(sc) as eng:
        res = eng.run(np.arange(2, dtype=np.uint64) + 3, want_chem=True)
    assert res["rc"] == abi.SP_OK, res.get("error")
    want = oracle_lib.chem_static(sc)
    np.testing.assert_array_equal(res["chem"][0], want)
    assert np.abs(want[-1] - want[0]).max() > 0.5


@pytest.mark.parametrize("prec,mode", [("f32", 6), ("f64", 2)])
def test_flow_boundary_conditions_bitexact(oracle_lib, prec, mode):
    from spatialpy_gb300.engine import Engine
    sc = flow_bcs()
    st = oracle_lib.SdpdState(sc)
    with Engine(sc, sdpd_precision=prec) as eng:
        done = 0
        for n in (1, 7, 30):
            eng.sdpd_advance(n - done)
            oracle_lib.sdpd(sc, st, n - done, prec, mode, kmax=48)
            done = n
            x, v, rho = eng.particles(0)
            np.testing.assert_array_equal(x, st.x, err_msg=f"x step {n}")
            np.testing.assert_array_equal(v, st.v, err_msg=f"v step {n}")
            np.testing.assert_array_equal(rho, st.rho, err_msg=f"rho step {n}")
    held = (sc.type == 1) & (st.x[:, 2] > 0.35)
    vx = float(np.float32(0.2)) if prec == "f32" else 0.2
    assert held.any() and np.all(st.v[held] == np.array([vx, 0.0, 0.0]))


@pytest.mark.parametrize("prec,mode", [("f32", 6), ("f64", 2)])
def test_moving_domain_chemistry_bitexact(oracle_lib, prec, mode):
    from spatialpy_gb300.engine import Engine
    base = dam_break_species(network="full", num_steps=25)
    programs = {}
    rate, kind, reac, allowed, jcN, irN, prN = S.mass_action(
        ["S"], [(0.5, {"S": 1}, {}, None), (2e5, {}, {"S": 1}, [1]),
                (2e-7, {"S": 2}, {}, None)], 2, programs=programs)
    sc = base.copy(enable_pde=True, rxn_rate=rate, rxn_kind=kind, rxn_reactants=reac,
                   rxn_allowed=allowed, jcN=jcN, irN=irN, prN=prN,
                   bc_box=[[-np.inf, 0.2, -np.inf, np.inf, -np.inf, np.inf]], bc_type=[0],
                   bc_target=[3], bc_value=[[7.0, 0, 0]], **programs)
    seeds = np.arange(3, dtype=np.uint64) + 12
    with Engine(sc, sdpd_precision=prec) as eng:
        res = eng.run(seeds, want_chem=True, want_particles=True)
    assert res["rc"] == abi.SP_OK, res.get("error")
    out, ev, st, px, pr, ch = oracle_lib.coupled_ensemble(sc, seeds, precision=prec, mode=mode,
                                                          want_chem=True)
    np.testing.assert_array_equal(res["particles"][0][0], px)
    np.testing.assert_array_equal(res["chem"][0], ch)
    np.testing.assert_array_equal(res["events"], ev)
    for j in range(len(seeds)):
        np.testing.assert_array_equal(res["counts"][j], out[j])


def test_chemistry_vs_compiled_reference():
    """GPU concentrations against the compiled engine (tests/golden/pins.npz):
    the static lattice with a concentration boundary condition and the
    moving dam break with an FP64 flow within 1e-12 of the largest value at
    every output; with the FP32 flow within 1e-7 (the oracle's FP32 run is
    3.8e-9 from the engine)."""
    from spatialpy_gb300.engine import Engine
    g = golden("pins.npz")
    seeds = np.arange(1, dtype=np.uint64) + 3
    with Engine(pinned_chem()) as eng:
        res = eng.run(seeds, want_chem=True)
    assert res["rc"] == abi.SP_OK, res.get("error")
    want = g["static/C"]
    assert np.abs(res["chem"][0] - want).max() <= 1e-12 * np.abs(want).max()
    want = g["moving/C"]
    for prec, tol in (("f64", 1e-12), ("f32", 1e-7)):
        with Engine(dam_break_chem(), sdpd_precision=prec) as eng:
            res = eng.run(seeds, want_chem=True)
        assert res["rc"] == abi.SP_OK, res.get("error")
        assert np.abs(res["chem"][0] - want).max() <= tol * np.abs(want).max(), prec


def test_flow_boundary_conditions_vs_compiled_reference():
    """The FP64 flow with boundary conditions on v, nu and rho against the
    compiled engine after 1, 5, 21 and 41 steps: positions and densities
    within 1e-12, velocities within 1e-9 norm-wise."""
    from spatialpy_gb300.engine import Engine
    g = golden("pins.npz")
    sc = flow_bcs(spacing_div=8, num_steps=41)
    with Engine(sc, sdpd_precision="f64") as eng:
        done = 0
        for n in (1, 5, 21, 41):
            eng.sdpd_advance(n - done)
            done = n
            x, v, rho = eng.particles(0)
            rv = g[f"bcs/{n}/v"]
            assert np.abs(x - g[f"bcs/{n}/x"]).max() <= 1e-12
            assert np.linalg.norm(v - rv) <= 1e-9 * np.linalg.norm(rv)
            assert np.abs(rho - g[f"bcs/{n}/rho"]).max() <= 1e-12
