"""GPU parity of custom propensity functions: the generic event kernel
evaluates the reaction programs (nsm_prog.cuh) in the oracle's operation
order, so trajectories are compared bit for bit.  The expressions use
arithmetic, integer powers, comparisons, sqrt, a data function and the
particle type, all of which round identically on both sides."""
import numpy as np
import pytest

from spatialpy_gb300 import abi
from spatialpy_gb300 import scenario as S

pytestmark = pytest.mark.gpu


def custom_model(n=12):
    base = S.config_birth_death_2d(n=n, count=60, t_end=4.0, num_points=5, dt=1.0)
    N = base.num_particles
    typ = np.where(base.x[:, 0] < 0.5, 1, 2).astype(np.int32)
    params = {"Vmax": 30.0, "Km": 3.0, "kh": 2.0, "kd": 0.4}
    rxns = [
        ("Vmax * vol / (1.0 + vol)", {}, {"E": 1}, [1]),                     # E birth, type 1
        ("Vmax * E / (Km + E) / Size", {"E": 1}, {"P": 1}, None),            # saturating
        ("kh * P ** 2 / (Km ** 2 + P ** 2) * (P > 1)", {"P": 1}, {}, None),  # Hill removal
        ("kd * sqrt(E) + 0.1 * (sd == 2) * E", {"E": 1}, {}, None),
        (0.05, {"P": 1}, {"E": 1}, None),                                    # mass action
    ]
    programs = {}
    rate, kind, reac, allowed, jcN, irN, prN = S.mass_action(
        ["E", "P"], rxns, 2, params, ["Size"], programs)
    u0 = np.zeros((N, 2), np.uint32)
    u0[:, 0] = np.random.default_rng(2).integers(0, 3, N)
    data = (1.0 + base.x[:, 0] + base.x[:, 1])[None, :]
    return base.copy(type=typ, num_types=2, species=["E", "P"], rxn_rate=rate, rxn_kind=kind,
                     rxn_reactants=reac, rxn_allowed=allowed, jcN=jcN, irN=irN, prN=prN,
                     diffusion=np.array([[0.05, 0.05], [0.02, 0.0]]), u0=u0,
                     data_fn=data, name="custom", **programs)


@pytest.mark.parametrize("selection", [abi.SP_SELECT_EXACT, abi.SP_SELECT_REFERENCE])
def test_custom_propensities_bitexact(oracle_lib, selection):
    from spatialpy_gb300.engine import Engine
    sc = custom_model()
    seeds = np.arange(6, dtype=np.uint64) + 777
    with Engine(sc) as eng:
        res = eng.run(seeds, selection=selection)
        assert eng.profile()["kernel"] == "nsm_advance_generic"
    assert res["rc"] == abi.SP_OK, res.get("error")
    for j, s in enumerate(seeds):
        out, ev, st = oracle_lib.nsm_trajectory(sc, int(s), selection)
        assert st == 0
        np.testing.assert_array_equal(res["events"][j], ev)
        np.testing.assert_array_equal(res["counts"][j], out)
    assert res["events"][:, 0].sum() > 100          # the reactions fired


def test_custom_propensities_on_a_large_domain(oracle_lib):
    """4,096 voxels: custom programs keep the run on the generic kernel."""
    from spatialpy_gb300.engine import Engine
    sc = custom_model(n=64).copy(num_steps=2, dt=0.02,
                                 output_steps=np.array([0, 1, 2], np.int32))
    seeds = np.arange(3, dtype=np.uint64) + 91
    with Engine(sc) as eng:
        res = eng.run(seeds)
    for j, s in enumerate(seeds):
        out, ev, _ = oracle_lib.nsm_trajectory(sc, int(s), 0)
        np.testing.assert_array_equal(res["events"][j], ev)
        np.testing.assert_array_equal(res["counts"][j], out)
