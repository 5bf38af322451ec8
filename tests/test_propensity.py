"""Custom propensity functions: the expression compiler, its programs'
values, the engine's program checks, and model conversion.

The reference compiles a reaction's propensity_function into the generated
C++ (spatialpy/solvers/solver.py:344-373 via build_expression.py:308-324);
here it becomes a stack program evaluated in double by the kernels and the
oracle."""
import ctypes as C
import math

import numpy as np
import pytest

from spatialpy_gb300 import abi
from spatialpy_gb300 import propensity as P
from spatialpy_gb300 import scenario as S

from .refmodels import spatialpy_or_skip

EXPRS = [
    "k1 * A * B / vol",
    "Vmax * A / (Km + A) * vol",
    "k1 * A ** 2 / (Km ** 2 + A ** 2)",
    "k1 * pow(A, 3) + k2 * sqrt(B + 1)",
    "k1 * exp(-A / 10.0) * (B > 2) + (A <= 1 or B == 0) * k2",
    "-k1 * -A + abs(B - 4) * log(A + 1) / (1 + t) + sd",
    "k2 * DomainSize * A",
]
NAMES = {"k1": 0.3, "k2": 1.7, "Vmax": 12.5, "Km": 4.0}


def _py(expr, x, vol, t, sd, data):
    env = dict(NAMES, A=float(x[0]), B=float(x[1]), vol=vol, t=t, sd=float(sd),
               DomainSize=data[0], exp=math.exp, log=math.log, sqrt=math.sqrt, pow=math.pow,
               abs=abs)
    return float(eval(expr, {"__builtins__": {}}, env))  # noqa: S307


@pytest.mark.parametrize("expr", EXPRS)
def test_program_values_equal_python(expr):
    consts = []
    code = P.compile_expression(expr, ["A", "B"], NAMES, consts, ["DomainSize"])
    rng = np.random.default_rng(3)
    for _ in range(50):
        x = rng.integers(0, 20, 2)
        vol, t, sd, data = float(rng.uniform(0.1, 2)), float(rng.uniform(0, 5)), 2, [0.25]
        got = P.evaluate(code, consts, x, vol, t, sd, data)
        want = _py(expr, x, vol, t, sd, data)
        assert got == pytest.approx(want, rel=1e-14, abs=1e-300), expr


def test_integer_powers_are_products():
    consts = []
    code = P.compile_expression("A ** 3", ["A"], {}, consts)
    assert P.POWI in code and P.POW not in code
    assert P.evaluate(code, consts, [7], 1.0) == 7.0 * 7.0 * 7.0


def test_rejects_unknown_names_and_deep_programs():
    with pytest.raises(P.PropensityError):
        P.compile_expression("k * Q", ["A"], {"k": 1.0}, [])
    deep = "A"
    for _ in range(17):
        deep = f"A * ({deep})"     # postfix keeps 18 values on the stack
    with pytest.raises(P.PropensityError):
        P.compile_expression(deep, ["A"], {}, [])


def _custom_scenario(code_words=None, consts=None):
    sc = S.config_birth_death_2d(n=4)
    rate, kind, reac, allowed, jcN, irN, prN = S.mass_action(
        ["Rabbits"], [("2.0 * Rabbits / (1.0 + Rabbits)", {"Rabbits": 1}, {}, None)], 1,
        programs=(fields := {}))
    sc = sc.copy(rxn_rate=rate, rxn_kind=kind, rxn_reactants=reac, rxn_allowed=allowed,
                 jcN=jcN, irN=irN, prN=prN, **fields)
    if code_words is not None:
        sc.rxn_code = np.array(code_words, np.int32)
        sc.rxn_code_off = np.array([0, len(code_words)], np.int64)
    if consts is not None:
        sc.rxn_consts = np.array(consts, np.float64)
    return sc


@pytest.mark.parametrize("words", [
    [P.CONST, 5, P.END],                       # constant index out of range
    [P.X, 3, P.END],                           # species index out of range
    [P.ADD, P.END],                            # underflow
    [P.CONST, 0, P.CONST, 0],                  # no END
    [P.DATA, 0, P.END],                        # no data functions
    [P.CONST, 0] * 17 + [P.ADD] * 16 + [P.END],  # 17 stack values
    [99, P.END],                               # unknown opcode
])
def test_engine_rejects_bad_programs_before_device_work(spgpu_lib, words):
    """sp_create checks every program before any CUDA call (no GPU needed)."""
    sc = _custom_scenario(words, [1.0])
    s = (abi.SpScenario * 1)(abi.scenario_struct(sc))
    h = C.c_void_p()
    rc = spgpu_lib.sp_create(s, 1, None, C.byref(h))
    msg = spgpu_lib.sp_last_error(h).decode()
    spgpu_lib.sp_destroy(h)
    assert rc == abi.SP_E_INVALID and "reaction 0" in msg, msg


def test_oracle_runs_custom_propensities(oracle_lib):
    """The CPU oracle evaluates programs (immigration with a saturating death
    rate); the total stays near its fixed point."""
    sc = _custom_scenario()
    out, ev, st = oracle_lib.nsm_trajectory(sc, 5, 0)
    assert st == 0 and ev.sum() > 0


def test_from_model_custom_propensity_and_data_function():
    """A MinCDE-style reaction (test/models/mincde.py:77-79): a custom
    propensity over a parameter and a data function, restricted to one type."""
    spatialpy = spatialpy_or_skip()

    class Size(spatialpy.DataFunction):
        def __init__(self):
            super().__init__(name="DomainSize")

        def map(self, point):
            return 1.0 + point[0] + 2.0 * point[1]

    model = spatialpy.Model("custom")
    dom = spatialpy.Domain.create_2D_domain(xlim=(0, 1), ylim=(0, 1), numx=6, numy=6,
                                            fixed=True)
    model.add_domain(dom)
    A = spatialpy.Species(name="A", diffusion_coefficient=0.01)
    B = spatialpy.Species(name="B", diffusion_coefficient=0.01)
    model.add_species([A, B])
    model.add_parameter(spatialpy.Parameter(name="sigma", expression=2.5))
    model.add_data_function(Size())
    model.add_reaction(spatialpy.Reaction(name="R1", reactants={A: 1}, products={B: 1},
                                          propensity_function="A * sigma / DomainSize"))
    model.add_reaction(spatialpy.Reaction(name="R2", reactants={B: 1}, products={A: 1},
                                          rate="sigma"))
    model.add_initial_condition(spatialpy.ScatterInitialCondition(A, 40))
    model.timespan(spatialpy.TimeSpan.linspace(t=2, num_points=3, timestep_size=1))
    sc = S.from_model(model)
    assert list(sc.rxn_kind) == [abi.SP_RXN_CUSTOM, abi.SP_RXN_FIRST]
    assert sc.data_fn.shape == (1, sc.num_particles)
    np.testing.assert_allclose(sc.data_fn[0], 1.0 + sc.x[:, 0] + 2.0 * sc.x[:, 1])
    code = sc.rxn_code[sc.rxn_code_off[0]:sc.rxn_code_off[1]]
    for v in (0, 7, sc.num_particles - 1):
        got = P.evaluate(code, sc.rxn_consts, [11, 3], float(sc.vol[v]), 0.0,
                         int(sc.type[v]), sc.data_fn[:, v])
        assert got == pytest.approx(11 * 2.5 / sc.data_fn[0, v], rel=1e-15)
