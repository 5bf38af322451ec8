"""GPU parity of deterministic chemistry (enable_pde) and boundary
conditions: the concentrations C of a static domain and of a moving one, and
a flow with boundary conditions on v, nu and rho, compared bit for bit with
the oracle (same operations, same order, no FMA contraction)."""
import numpy as np
import pytest

from spatialpy_gb300 import abi
from spatialpy_gb300 import scenario as S

from .chem_cases import flow_bcs, static_chem
from .coupled_cases import dam_break_species

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
