"""CPU tests of the workload builders against the sizes and rules they restate."""
import numpy as np

from spatialpy_gb300 import abi
from spatialpy_gb300 import scenario as S


def test_birth_death_domain():
    sc = S.config_birth_death_2d()
    assert sc.num_particles == 100                      # linspace(0,1,10)^2
    assert np.isclose(sc.h, 2.2 / 9)                    # find_h = 2.2 x spacing
    assert np.allclose(sc.vol, 0.01)
    assert sc.u0.sum() == 100
    assert list(sc.output_steps) == list(range(11)) and sc.num_steps == 10
    assert list(sc.rxn_kind) == [abi.SP_RXN_ZERO, abi.SP_RXN_FIRST]
    assert list(sc.jcN) == [0, 1, 2] and list(sc.prN) == [1, -1]


def test_rdme_3d_domain():
    sc = S.config_rdme_3d(n=10, nA=100, nB=50)
    assert sc.num_particles == 1000
    assert (sc.type == 2).sum() == 100                  # x < 0.1: the first plane
    assert sc.u0[:, 0].sum() == 100 and sc.u0[:, 1].sum() == 50
    # 0 -> A is restricted to type 2
    assert sc.rxn_allowed[2].tolist() == [0, 0, 1]
    assert list(sc.rxn_kind) == [abi.SP_RXN_SECOND, abi.SP_RXN_FIRST, abi.SP_RXN_ZERO,
                                 abi.SP_RXN_FIRST]


def test_dam_break_sizes():
    sc = S.config_dam_break()
    fluid = (sc.fixed == 0).sum()
    assert fluid == 48 * 32 * 32
    assert sc.num_particles - fluid == 70 * 38 * 38 - 64 * 32 * 32      # 35,544 walls
    assert np.isclose(sc.h, 1.5 / 64)
    assert np.allclose(sc.mass, 1.0 / 64 ** 3)
    top = np.nonzero(sc.u0[:, 0])[0]
    assert sc.u0.sum() == 50000 and np.all(sc.fixed[top] == 0)
    assert np.all(sc.x[top, 2] > 0.45)


def test_mass_action_dimer_and_restrictions():
    rate, kind, reac, allowed, jcN, irN, prN = S.mass_action(
        ["A", "B"], [(1.0, {"A": 2}, {"B": 1}, None), (2.0, {"A": 1, "B": 1}, {}, [2])], 2)
    assert list(kind) == [abi.SP_RXN_DIMER, abi.SP_RXN_SECOND]
    assert list(jcN) == [0, 2, 4] and list(irN) == [0, 1, 0, 1] and list(prN) == [-2, 1, -1, -1]
    assert allowed[1].tolist() == [0, 0, 1] and allowed[0].tolist() == [0, 1, 1]


def test_uneven_ensemble_sizes():
    ins = S.config_uneven_ensemble(num_instances=16, seed=4)
    for i, sc in enumerate(ins):
        assert sc.dimension == (2 if i % 2 == 0 else 3)
        assert 400 * 0.5 <= sc.num_particles <= 40000 * 1.5
        assert sc.u0.sum() == 100
