"""Scenarios with deterministic chemistry (enable_pde) and boundary
conditions, shared by the CPU and GPU tests."""
import numpy as np

from spatialpy_gb300 import scenario as S

INF = np.inf


def static_chem(n=10, reactions="full", bcs=True):
    """2-D n x n static lattice, two types (x < 0.5 is type 1), species A, B
    (D = 0.1 / 0.05), deterministic chemistry on: A + B -> 0 (k 0.02),
    0 -> A on type 1 (k 3), B decays by a custom rate k*B/(1+B); a boundary
    condition holds C[B] = 4 for y > 0.8."""
    base = S.config_birth_death_2d(n=n, count=0, t_end=3.0, num_points=4, dt=0.05)
    N = base.num_particles
    typ = np.where(base.x[:, 0] < 0.5, 1, 2).astype(np.int32)
    rxns = {"full": [(0.02, {"A": 1, "B": 1}, {}, None),
                     (3.0, {}, {"A": 1}, [1]),
                     ("kd * B / (1.0 + B)", {"B": 1}, {}, None)],
            "birth": [(3.0, {}, {"A": 1}, [1])],
            "none": []}[reactions]
    programs = {}
    rate, kind, reac, allowed, jcN, irN, prN = S.mass_action(["A", "B"], rxns, 2, {"kd": 0.7},
                                                             [], programs)
    u0 = np.zeros((N, 2), np.uint32)
    rng = np.random.default_rng(5)
    u0[:, 0] = rng.integers(0, 20, N)
    u0[:, 1] = rng.integers(0, 10, N)
    extra = {}
    if bcs:
        extra = dict(bc_box=[[-INF, INF, 0.8, INF, -INF, INF]], bc_type=[0], bc_target=[3 + 1],
                     bc_value=[[4.0, 0.0, 0.0]])
    return base.copy(type=typ, num_types=2, species=["A", "B"], rxn_rate=rate, rxn_kind=kind,
                     rxn_reactants=reac, rxn_allowed=allowed, jcN=jcN, irN=irN, prN=prN,
                     diffusion=np.array([[0.1, 0.1], [0.05, 0.05]]), u0=u0, enable_pde=True,
                     name="static_chem", **programs, **extra)


def flow_bcs(spacing_div=16, num_steps=30):
    """The dam break with boundary conditions on the flow: fluid particles
    with z > 0.35 get v = (0.2, 0, 0); particles with x < 0.1 get rho = 1.05;
    walls (type 2) with z < 0.1 get nu = 5e-3."""
    sc = S.config_dam_break(spacing_div=spacing_div, num_steps=num_steps)
    return sc.copy(bc_box=[[-INF, INF, -INF, INF, 0.35, INF], [-INF, 0.1, -INF, INF, -INF, INF],
                           [-INF, INF, -INF, INF, -INF, 0.1]],
                   bc_type=[1, 0, 2], bc_target=[0, 2, 1],
                   bc_value=[[0.2, 0.0, 0.0], [1.05, 0, 0], [5e-3, 0, 0]])


def pinned_chem(n=10):
    """Deterministic chemistry that the reference engine can be compared on.
    The engine reads the diffusion matrix type-major and the dense
    stoichiometry reaction-major (model.cpp:165, 186) from arrays written the
    other way round (solver.py:225-231, 269-286); with one particle type and a
    symmetric stoichiometry both reads agree with the layouts.  2-D n x n
    lattice, species A, B (D = 0.1 / 0.05), A -> B (k 0.3), B -> A (k 0.1),
    and a boundary condition holding C[B] = 4 for y > 0.8."""
    base = S.config_birth_death_2d(n=n, count=0, t_end=3.0, num_points=4, dt=0.05)
    N = base.num_particles
    programs = {}
    rate, kind, reac, allowed, jcN, irN, prN = S.mass_action(
        ["A", "B"], [(0.3, {"A": 1}, {"B": 1}, None), (0.1, {"B": 1}, {"A": 1}, None)], 1, {},
        [], programs)
    u0 = np.zeros((N, 2), np.uint32)
    rng = np.random.default_rng(5)
    u0[:, 0] = rng.integers(0, 20, N)
    u0[:, 1] = rng.integers(0, 10, N)
    return base.copy(species=["A", "B"], rxn_rate=rate, rxn_kind=kind, rxn_reactants=reac,
                     rxn_allowed=allowed, jcN=jcN, irN=irN, prN=prN,
                     diffusion=np.array([[0.1], [0.05]]), u0=u0, enable_pde=True,
                     bc_box=[[-INF, INF, 0.8, INF, -INF, INF]], bc_type=[0], bc_target=[3 + 1],
                     bc_value=[[4.0, 0.0, 0.0]], name="pinned_chem", **programs)
