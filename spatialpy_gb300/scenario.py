"""Scenario: the array form of a compiled SpatialPy model, and synthetic builders.

A :class:`Scenario` carries exactly what ``Solver.compile()`` bakes into the
generated C++ model (spatialpy/solvers/solver.py:208-288 input constants,
:312-331 particle inits, :375-419 system config) as numpy arrays, so the GPU
engine needs neither code generation nor a C++ build per model.

``from_model`` converts a ``spatialpy.Model`` (after ``compile_prep``).  The
``config_*`` builders create the benchmark workloads directly, without
spatialpy, with the shapes, sizes and rules of the reference's domain and
reaction builders (cited per function).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import propensity as prop
from .abi import SP_RXN_CUSTOM, SP_RXN_DIMER, SP_RXN_FIRST, SP_RXN_SECOND, SP_RXN_ZERO


@dataclasses.dataclass
class Scenario:
    dimension: int
    x: np.ndarray                 # [N,3] float64
    type: np.ndarray              # [N] int32, 1..num_types
    mass: np.ndarray              # [N] float64
    rho: np.ndarray               # [N] float64
    nu: np.ndarray                # [N] float64
    fixed: np.ndarray             # [N] uint8
    num_types: int
    species: list                 # names
    rxn_rate: np.ndarray          # [R] float64
    rxn_kind: np.ndarray          # [R] int32
    rxn_reactants: np.ndarray     # [R,2] int32
    rxn_allowed: np.ndarray | None  # [R,T+1] uint8
    jcN: np.ndarray               # [R+1] int64
    irN: np.ndarray               # [nnz] int64
    prN: np.ndarray               # [nnz] int32
    diffusion: np.ndarray         # [S,T] float64
    h: float
    dt: float
    num_steps: int
    output_steps: np.ndarray      # [T_out] int32
    static_domain: bool = True
    rho0: float = 1.0
    c0: float = 10.0
    P0: float | None = None
    gravity: tuple = (0.0, 0.0, 0.0)
    v: np.ndarray | None = None   # [N,3] float64
    u0: np.ndarray | None = None  # [N,S] uint32 (voxel-major)
    name: str = "scenario"
    rxn_code: np.ndarray | None = None      # custom propensity programs (int32)
    rxn_code_off: np.ndarray | None = None  # [R+1] int64
    rxn_consts: np.ndarray | None = None    # float64
    data_fn: np.ndarray | None = None       # [num_data_fn, N] float64
    enable_pde: bool = False                # deterministic concentrations C
    ode_code: np.ndarray | None = None      # ODE propensity programs, one per reaction
    ode_code_off: np.ndarray | None = None
    ode_consts: np.ndarray | None = None
    bc_box: np.ndarray | None = None        # [nbc, 6] xmin xmax ymin ymax zmin zmax
    bc_type: np.ndarray | None = None       # [nbc] int32, 0 = any
    bc_target: np.ndarray | None = None     # [nbc] int32 SP_BC_*
    bc_value: np.ndarray | None = None      # [nbc, 3]

    def __post_init__(self):
        self.x = np.ascontiguousarray(self.x, dtype=np.float64).reshape(-1, 3)
        n = self.x.shape[0]
        self.type = np.ascontiguousarray(self.type, dtype=np.int32).reshape(n)
        self.mass = np.ascontiguousarray(np.broadcast_to(self.mass, (n,)), dtype=np.float64)
        self.rho = np.ascontiguousarray(np.broadcast_to(self.rho, (n,)), dtype=np.float64)
        self.nu = np.ascontiguousarray(np.broadcast_to(self.nu, (n,)), dtype=np.float64)
        self.fixed = np.ascontiguousarray(np.broadcast_to(self.fixed, (n,)), dtype=np.uint8)
        self.rxn_rate = np.ascontiguousarray(self.rxn_rate, dtype=np.float64).reshape(-1)
        r = self.rxn_rate.shape[0]
        self.rxn_kind = np.ascontiguousarray(self.rxn_kind, dtype=np.int32).reshape(r)
        self.rxn_reactants = np.ascontiguousarray(self.rxn_reactants, dtype=np.int32).reshape(r, 2)
        if self.rxn_allowed is not None:
            self.rxn_allowed = np.ascontiguousarray(self.rxn_allowed, dtype=np.uint8).reshape(
                r, self.num_types + 1)
        self.jcN = np.ascontiguousarray(self.jcN, dtype=np.int64)
        self.irN = np.ascontiguousarray(self.irN, dtype=np.int64)
        self.prN = np.ascontiguousarray(self.prN, dtype=np.int32)
        self.diffusion = np.ascontiguousarray(self.diffusion, dtype=np.float64).reshape(
            len(self.species), self.num_types)
        self.output_steps = np.ascontiguousarray(self.output_steps, dtype=np.int32)
        if self.P0 is None:
            self.P0 = self.rho0 * self.c0 ** 2   # Domain default (domain.py:92-95)
        if self.v is not None:
            self.v = np.ascontiguousarray(self.v, dtype=np.float64).reshape(n, 3)
        if self.u0 is not None:
            self.u0 = np.ascontiguousarray(self.u0, dtype=np.uint32).reshape(n, len(self.species))
        if self.rxn_code is not None:
            self.rxn_code = np.ascontiguousarray(self.rxn_code, dtype=np.int32)
            self.rxn_code_off = np.ascontiguousarray(self.rxn_code_off, dtype=np.int64)
            self.rxn_consts = np.ascontiguousarray(self.rxn_consts, dtype=np.float64)
            if self.rxn_consts.size == 0:
                self.rxn_consts = np.zeros(1)
        if self.data_fn is not None:
            self.data_fn = np.ascontiguousarray(self.data_fn, dtype=np.float64).reshape(-1, n)
        if self.ode_code is not None:
            self.ode_code = np.ascontiguousarray(self.ode_code, dtype=np.int32)
            self.ode_code_off = np.ascontiguousarray(self.ode_code_off, dtype=np.int64)
            self.ode_consts = np.ascontiguousarray(self.ode_consts, dtype=np.float64)
            if self.ode_consts.size == 0:
                self.ode_consts = np.zeros(1)
        if self.bc_target is not None:
            nb = len(self.bc_target)
            self.bc_target = np.ascontiguousarray(self.bc_target, dtype=np.int32)
            self.bc_type = np.ascontiguousarray(self.bc_type, dtype=np.int32).reshape(nb)
            self.bc_box = np.ascontiguousarray(self.bc_box, dtype=np.float64).reshape(nb, 6)
            self.bc_value = np.ascontiguousarray(self.bc_value, dtype=np.float64).reshape(nb, 3)

    @property
    def num_particles(self) -> int:
        return self.x.shape[0]

    @property
    def num_species(self) -> int:
        return len(self.species)

    @property
    def num_reactions(self) -> int:
        return self.rxn_rate.shape[0]

    @property
    def vol(self) -> np.ndarray:
        return self.mass / self.rho

    def output_times(self) -> np.ndarray:
        return self.output_steps.astype(np.float64) * self.dt

    def copy(self, **changes) -> "Scenario":
        d = {f.name: getattr(self, f.name) for f in dataclasses.fields(self)}
        d.update(changes)
        return Scenario(**d)


# ----------------------------------------------------------------------------
# reaction network helpers (mass action, reaction.py:260-313)
# ----------------------------------------------------------------------------

def mass_action(species: list, reactions: list, num_types: int, params: dict | None = None,
                data_names: list = (), programs: dict | None = None):
    """Encode ``[(rate, {reactant: stoich}, {product: stoich}, restrict_types|None)]``.

    Returns (rate, kind, reactants, allowed, jcN, irN, prN).  The stoichiometry
    CSC matches ``Model.__create_stoichiometric_matrix`` (model.py:252-268):
    per reaction column, rows in ascending species order.

    A rate given as a string is a custom propensity function: the reaction
    gets kind SP_RXN_CUSTOM and its program (propensity.compile_expression
    over ``params`` and ``data_names``).  Pass a dict as ``programs`` to
    receive ``code``, ``off`` and ``consts`` (see :func:`custom_fields`).
    """
    S, R = len(species), len(reactions)
    idx = {s: i for i, s in enumerate(species)}
    rate = np.zeros(R)
    kind = np.zeros(R, np.int32)
    reac = -np.ones((R, 2), np.int32)
    allowed = np.ones((R, num_types + 1), np.uint8)
    allowed[:, 0] = 0
    restricted = False
    dense = np.zeros((S, R), np.int64)
    progs, consts = [None] * R, []
    oprogs, oconsts = [None] * R, []
    for r, entry in enumerate(reactions):
        k, reactants, products, types = entry[:4]
        order = sum(reactants.values())
        if isinstance(k, str):
            kind[r] = SP_RXN_CUSTOM
            progs[r] = prop.compile_expression(k, species, params or {}, consts, data_names)
            ode = entry[4] if len(entry) > 4 and entry[4] else k
            oprogs[r] = prop.compile_expression(ode, species, params or {}, oconsts, data_names)
        elif order > 2:
            raise ValueError("mass-action reactions are at most second order")
        else:
            rate[r] = float(k)
            # the ODE form of a mass-action propensity: k times each reactant
            # (reaction.py:283-300), no volume factor
            oprogs[r] = prop.mass_action_ode(float(k), [(idx[sp], n) for sp, n in
                                                        reactants.items()], oconsts)
        if kind[r] == SP_RXN_CUSTOM:
            pass
        elif order == 0:
            kind[r] = SP_RXN_ZERO
        elif len(reactants) == 1 and order == 1:
            kind[r] = SP_RXN_FIRST
            reac[r, 0] = idx[next(iter(reactants))]
        elif len(reactants) == 1:
            kind[r] = SP_RXN_DIMER
            reac[r, 0] = idx[next(iter(reactants))]
        else:
            kind[r] = SP_RXN_SECOND
            a, b = list(reactants)
            reac[r] = (idx[a], idx[b])
        for s, n in reactants.items():
            dense[idx[s], r] -= n
        for s, n in products.items():
            dense[idx[s], r] += n
        if types is not None:
            restricted = True
            allowed[r, :] = 0
            for t in types:
                allowed[r, t] = 1
    jcN = [0]
    irN, prN = [], []
    for r in range(R):
        for s in range(S):
            if dense[s, r] != 0:
                irN.append(s)
                prN.append(int(dense[s, r]))
        jcN.append(len(irN))
    if programs is not None:
        programs.update(custom_fields(progs, consts))
        ocode, ooff = prop.pack(oprogs)
        programs.update({"ode_code": ocode, "ode_code_off": ooff,
                         "ode_consts": np.array(oconsts if oconsts else [0.0], np.float64)})
    return (rate, kind, reac, allowed if restricted else None,
            np.array(jcN, np.int64), np.array(irN, np.int64), np.array(prN, np.int32))


def custom_fields(progs: list, consts: list) -> dict:
    """Scenario fields for custom propensity programs (all None without any)."""
    if not any(p is not None for p in progs):
        return {"rxn_code": None, "rxn_code_off": None, "rxn_consts": None}
    code, off = prop.pack(progs)
    return {"rxn_code": code, "rxn_code_off": off,
            "rxn_consts": np.array(consts if consts else [0.0], np.float64)}


def find_h(x: np.ndarray) -> float:
    """2.2 x the largest nearest-neighbour distance (Domain.find_h, domain.py:751-769)."""
    from scipy.spatial import cKDTree
    d, _ = cKDTree(x).query(x, 2)
    return 2.2 * float(np.max(d[:, 1]))


def timespan(t_end: float, num_points: int, dt: float):
    """Uniform TimeSpan.linspace(t, num_points, timestep_size) (timespan.py:72-85)."""
    items = np.linspace(0, t_end, num_points)
    interval = items[1] - items[0]
    freq = interval / dt
    num_steps = math.ceil((num_points - 1) * freq)
    steps = np.arange(0, num_steps + dt, freq)
    steps = np.unique(np.round(steps).astype(int))
    return num_steps, steps.astype(np.int32)


def scatter(counts_by_species: dict, allowed_voxels: dict, nvox: int, species: list,
            seed: int) -> np.ndarray:
    """ScatterInitialCondition (initialcondition.py:178-197): one
    ``randint(0, nvox)`` per molecule from numpy's legacy global generator
    seeded once, shared by every trajectory (u0 is baked into the build)."""
    rs = np.random.RandomState(seed)
    u0 = np.zeros((nvox, len(species)), np.uint32)
    for s, count in counts_by_species.items():
        j = species.index(s)
        vox = allowed_voxels.get(s)
        for _ in range(count):
            if vox is None:
                u0[rs.randint(0, nvox), j] += 1
            else:
                u0[vox[rs.randint(0, len(vox))], j] += 1
    return u0


def lattice(axes: list) -> np.ndarray:
    """Cartesian product of 1-D coordinate arrays with x varying slowest, the
    nesting order of CartesianLattice.apply (lattice.py:210-229)."""
    grids = np.meshgrid(*axes, indexing="ij")
    pts = np.stack([g.reshape(-1) for g in grids], axis=1)
    if pts.shape[1] < 3:
        pts = np.concatenate([pts, np.zeros((pts.shape[0], 3 - pts.shape[1]))], axis=1)
    return pts


# ----------------------------------------------------------------------------
# workload builders
# ----------------------------------------------------------------------------

def config_birth_death_2d(n: int = 10, k_birth: float = 10.0, k_death: float = 0.1,
                          D: float = 0.1, count: int = 100, t_end: float = 10.0,
                          num_points: int = 11, dt: float = 1.0, seed: int = 1) -> Scenario:
    """Spatial birth-death on the unit square, n x n fixed particles on
    linspace(0,1,n)^2 (test/models/birth_death.py:19-50 with explicit points),
    vol = 1/n^2, mass 1, one type, D, birth k_b*vol, death k_d*x."""
    ax = np.linspace(0.0, 1.0, n)
    x = lattice([ax, ax])
    N = x.shape[0]
    vol = 1.0 / N
    species = ["Rabbits"]
    rate, kind, reac, allowed, jcN, irN, prN = mass_action(
        species, [(k_birth, {}, {"Rabbits": 1}, None), (k_death, {"Rabbits": 1}, {}, None)], 1)
    nt, steps = timespan(t_end, num_points, dt)
    u0 = scatter({"Rabbits": count}, {}, N, species, seed)
    return Scenario(dimension=2, x=x, type=np.ones(N), mass=1.0, rho=1.0 / vol, nu=1.0,
                    fixed=1, num_types=1, species=species, rxn_rate=rate, rxn_kind=kind,
                    rxn_reactants=reac, rxn_allowed=allowed, jcN=jcN, irN=irN, prN=prN,
                    diffusion=np.array([[D]]), h=find_h(x), dt=dt, num_steps=nt,
                    output_steps=steps, static_domain=True, u0=u0, name=f"birth_death_{n}x{n}")


def config_rdme_3d(n: int = 40, D=(1e-2, 1e-2, 1e-3), k_f: float = 1e-3, k_r: float = 0.1,
                   k_birth: float = 5.0, k_decay: float = 0.05, nA: int = 10000,
                   nB: int = 10000, t_end: float = 100.0, num_points: int = 101,
                   dt: float = 1.0, seed: int = 2, dims: int = 3) -> Scenario:
    """Static RDME: unit cube (or square, dims=2) with n^d fixed lattice
    particles (Domain.create_3D_domain, domain.py:574-645), type 1 = bulk,
    type 2 = 'left' (x < 0.1).  A+B->C (k_f*A*B/vol), C->A+B (k_r*C),
    0->A restricted to 'left' (k_birth*vol), C->0 (k_decay*C)."""
    ax = np.linspace(0.0, 1.0, n)
    x = lattice([ax] * dims)
    N = x.shape[0]
    vol = 1.0 / N
    typ = np.where(x[:, 0] < 0.1, 2, 1).astype(np.int32)
    species = ["A", "B", "C"]
    rate, kind, reac, allowed, jcN, irN, prN = mass_action(species, [
        (k_f, {"A": 1, "B": 1}, {"C": 1}, None),
        (k_r, {"C": 1}, {"A": 1, "B": 1}, None),
        (k_birth, {}, {"A": 1}, [2]),
        (k_decay, {"C": 1}, {}, None),
    ], 2)
    diff = np.array([[D[0], D[0]], [D[1], D[1]], [D[2], D[2]]], np.float64)
    nt, steps = timespan(t_end, num_points, dt)
    u0 = scatter({"A": nA, "B": nB}, {}, N, species, seed)
    return Scenario(dimension=dims, x=x, type=typ, mass=1.0, rho=1.0 / vol, nu=1.0, fixed=1,
                    num_types=2, species=species, rxn_rate=rate, rxn_kind=kind,
                    rxn_reactants=reac, rxn_allowed=allowed, jcN=jcN, irN=irN, prN=prN,
                    diffusion=diff, h=find_h(x), dt=dt, num_steps=nt, output_steps=steps,
                    static_domain=True, u0=u0, name=f"rdme_{dims}d_{n}")


def config_dam_break(spacing_div: int = 64, box=(1.0, 0.5, 0.5), fluid_frac_x: float = 0.75,
                     wall_layers: int = 3, rho0: float = 1.0, c0: float = 10.0,
                     nu: float = 1e-3, dt: float = 1e-4, num_steps: int = 10000,
                     h_factor: float = 1.5, species_D: float = 1e-3, decay: float = 0.01,
                     molecules: int = 50000, top_frac: float = 0.1, seed: int = 3,
                     num_outputs: int = 11, dims: int = 3) -> Scenario:
    """SDPD dam break in a walled box: fluid block at cell centres (i+1/2)s for
    x < fluid_frac_x*Lx, `wall_layers` layers of fixed wall particles around
    the box, m = rho0 s^3, gravity (0,0,-1), h = h_factor*s, non-static.
    One advected species (fluid-only diffusion, first-order decay) scattered
    over the fluid particles in the top `top_frac` of the fluid column.
    dims=2: the same in the xy-plane (box[0] x box[2], z = 0), m = rho0 s^2,
    gravity (0,-1,0)."""
    s = 1.0 / spacing_div
    if dims == 2:
        box = (box[0], box[2], s)
    nx, ny, nz = (int(round(L / s)) for L in box)
    L = wall_layers
    ix = np.arange(-L, nx + L)
    iy = np.arange(-L, ny + L)
    iz = np.arange(-L, nz + L) if dims == 3 else np.zeros(1)
    I = lattice([ix.astype(float), iy.astype(float), iz.astype(float)]).astype(np.int64)
    inside = ((I[:, 0] >= 0) & (I[:, 0] < nx) & (I[:, 1] >= 0) & (I[:, 1] < ny)
              & (I[:, 2] >= 0) & (I[:, 2] < nz))
    nfx = int(round(fluid_frac_x * nx))
    fluid = inside & (I[:, 0] < nfx)
    wall = ~inside
    keep = fluid | wall
    I = I[keep]
    fluid = fluid[keep]
    x = (I.astype(np.float64) + 0.5) * s
    if dims == 2:
        x[:, 2] = 0.0
    N = x.shape[0]
    typ = np.where(fluid, 1, 2).astype(np.int32)
    species = ["S"]
    rate, kind, reac, allowed, jcN, irN, prN = mass_action(
        species, [(decay, {"S": 1}, {}, None)], 2)
    diff = np.array([[species_D, 0.0]])
    # the top `top_frac` of the fluid column, at least one particle layer
    up = 2 if dims == 3 else 1          # the vertical axis
    layers = max(1, int(round(top_frac * (nz if dims == 3 else ny))))
    top = np.nonzero(fluid & (I[:, up] >= (nz if dims == 3 else ny) - layers))[0]
    u0 = scatter({"S": molecules}, {"S": top}, N, species, seed)
    steps = np.unique(np.round(np.linspace(0, num_steps, num_outputs)).astype(np.int32))
    gravity = (0.0, 0.0, -1.0) if dims == 3 else (0.0, -1.0, 0.0)
    return Scenario(dimension=dims, x=x, type=typ, mass=rho0 * s ** dims, rho=rho0, nu=nu,
                    fixed=(~fluid).astype(np.uint8), num_types=2, species=species,
                    rxn_rate=rate, rxn_kind=kind, rxn_reactants=reac, rxn_allowed=allowed,
                    jcN=jcN, irN=irN, prN=prN, diffusion=diff, h=h_factor * s, dt=dt,
                    num_steps=num_steps, output_steps=steps, static_domain=False, rho0=rho0,
                    c0=c0, gravity=gravity, u0=u0,
                    name=f"dam_break_{N}" if dims == 3 else f"dam_break_2d_{N}")


def config_uneven_ensemble(num_instances: int = 4096, vmin: int = 400, vmax: int = 40000,
                           seed: int = 4, num_intervals: int = 100, t_end: float = 10.0):
    """Batched uneven birth-death ensemble: instance i is 2-D when i is even and
    3-D when odd, with n^d lattice particles where n^d ~ logU[vmin, vmax];
    k_b, k_d, D each x 10^U(-1,1) around (10, 0.1, 0.1); initial count
    round(100 * total volume) = 100 scattered uniformly."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(num_instances):
        d = 2 if i % 2 == 0 else 3
        target = math.exp(rng.uniform(math.log(vmin), math.log(vmax)))
        n = max(2, int(round(target ** (1.0 / d))))
        kb, kd, D = (10.0 * 10 ** rng.uniform(-1, 1), 0.1 * 10 ** rng.uniform(-1, 1),
                     0.1 * 10 ** rng.uniform(-1, 1))
        useed = int(rng.integers(0, 2 ** 31 - 1))
        if d == 2:
            sc = config_birth_death_2d(n=n, k_birth=kb, k_death=kd, D=D, count=100,
                                       t_end=t_end, num_points=num_intervals + 1,
                                       dt=t_end / num_intervals, seed=useed)
        else:
            ax = np.linspace(0.0, 1.0, n)
            x = lattice([ax] * 3)
            N = x.shape[0]
            species = ["Rabbits"]
            rate, kind, reac, allowed, jcN, irN, prN = mass_action(
                species, [(kb, {}, {"Rabbits": 1}, None), (kd, {"Rabbits": 1}, {}, None)], 1)
            nt, steps = timespan(t_end, num_intervals + 1, t_end / num_intervals)
            u0 = scatter({"Rabbits": 100}, {}, N, species, useed)
            sc = Scenario(dimension=3, x=x, type=np.ones(N), mass=1.0, rho=float(N), nu=1.0,
                          fixed=1, num_types=1, species=species, rxn_rate=rate,
                          rxn_kind=kind, rxn_reactants=reac, rxn_allowed=allowed, jcN=jcN,
                          irN=irN, prN=prN, diffusion=np.array([[D]]), h=2.2 / (n - 1),
                          dt=t_end / num_intervals, num_steps=nt, output_steps=steps,
                          static_domain=True, u0=u0, name=f"bd3d_{n}")
        if d == 2:
            sc.h = 2.2 / (n - 1)
        out.append(sc)
    return out


# ----------------------------------------------------------------------------
# spatialpy.Model adapter
# ----------------------------------------------------------------------------

def from_model(model, h: float | None = None) -> Scenario:
    """Convert a ``spatialpy.Model`` to a :class:`Scenario`.

    Follows Solver.compile(): ``model.compile_prep()`` (model.py:982-1019),
    type index mapping (domain.py:137-146), diffusion matrix with
    ``restrict_to`` (solver.py:269-286), mass-action propensities
    (reaction.py:260-313; custom propensities raise NotImplementedError),
    ``h = find_h()`` unless given (solver.py:406-410), dimension from the
    vertex columns (solver.py:404-410).  Custom propensity functions become
    stack programs (propensity.py) over the model's parameters and data
    functions, the latter evaluated at the initial positions
    (solver.py:239-249)."""
    stoich, _dep = model.compile_prep()
    dom = model.domain
    tmap = dom.typeNdxMapping
    T = len(tmap) - 1
    species = list(model.listOfSpecies.keys())
    type_idx = np.array([tmap[t] for t in dom.type_id], np.int32)
    params = {n: p.value for n, p in model.listOfParameters.items()}
    data_names = list(getattr(model, "listOfDataFunctions", {}).keys())
    rxns = []
    for rname, r in model.listOfReactions.items():
        if not r.massaction:
            types = None
            if r.restrict_to:
                types = [tmap[t if str(t).startswith("type_") else f"type_{t}"]
                         for t in r.restrict_to]
            reactants = {s.name if hasattr(s, "name") else s: n for s, n in r.reactants.items()}
            products = {s.name if hasattr(s, "name") else s: n for s, n in r.products.items()}
            rxns.append((str(r.propensity_function), reactants, products, types,
                         str(r.ode_propensity_function or r.propensity_function)))
            continue
        k = r.marate
        if hasattr(k, "value"):
            k = k.value
        elif isinstance(k, str):
            k = float(eval(k, {"__builtins__": {}}, params))  # noqa: S307
        reactants = {s.name if hasattr(s, "name") else s: n for s, n in r.reactants.items()}
        products = {s.name if hasattr(s, "name") else s: n for s, n in r.products.items()}
        types = None
        if r.restrict_to:
            types = [tmap[t if str(t).startswith("type_") else f"type_{t}"] for t in r.restrict_to]
        rxns.append((float(k), reactants, products, types))
    programs = {}
    try:
        rate, kind, reac, allowed, jcN, irN, prN = mass_action(species, rxns, T, params,
                                                               data_names, programs)
    except prop.PropensityError as err:
        raise NotImplementedError(str(err)) from err
    # boundary conditions (boundarycondition.py:121-167)
    bcs = {}
    blist = list(getattr(model, "listOfBoundaryConditions", []))
    if blist:
        box, btype, btarget, bval = [], [], [], []
        for bc in blist:
            lim = [bc.xmin, bc.xmax, bc.ymin, bc.ymax, bc.zmin, bc.zmax]
            box.append([(-np.inf if q % 2 == 0 else np.inf) if v is None else float(v)
                        for q, v in enumerate(lim)])
            tid = bc.type_id
            btype.append(0 if tid is None else tmap[tid if str(tid).startswith("type_")
                                                    else f"type_{tid}"])
            tg = bc.target.name if hasattr(bc.target, "name") else bc.target
            if tg in species:
                btarget.append(3 + species.index(tg))
            else:
                btarget.append({"v": 0, "nu": 1, "rho": 2}[tg])
            val = bc.value
            bval.append(list(val) if isinstance(val, (list, tuple)) else [float(val), 0.0, 0.0])
        bcs = {"bc_box": box, "bc_type": btype, "bc_target": btarget, "bc_value": bval}
    data_fn = None
    if data_names:
        coords = np.asarray(dom.coordinates(), np.float64)
        data_fn = np.array([[float(f.map([c[0], c[1], c[2]])) for c in coords]
                            for f in model.listOfDataFunctions.values()])
    # the stoichiometry must agree with compile_prep's CSC
    if stoich is not None and min(stoich.shape) > 0:
        assert np.array_equal(np.asarray(stoich.indptr), jcN)
        assert np.array_equal(np.asarray(stoich.indices), irN)
    diff = np.zeros((len(species), T))
    for i, sp in enumerate(model.listOfSpecies.values()):
        for tname, t in tmap.items():
            if t == 0:
                continue
            restr = model.listOfDiffusionRestrictions.get(sp)
            if restr is None or tname in restr:
                diff[i, t - 1] = float(sp.diffusion_coefficient)
    verts = dom.vertices
    if not np.count_nonzero(verts[:, 1]):
        dim = 1
    elif not np.count_nonzero(verts[:, 2]):
        dim = 2
    else:
        dim = 3
    ts = model.tspan
    u0 = np.ascontiguousarray(model.u0.T.astype(np.uint32))
    return Scenario(dimension=dim, x=np.asarray(verts, np.float64), type=type_idx,
                    mass=dom.mass, rho=dom.rho, nu=dom.nu, fixed=dom.fixed.astype(np.uint8),
                    num_types=T, species=species, rxn_rate=rate, rxn_kind=kind,
                    rxn_reactants=reac, rxn_allowed=allowed, jcN=jcN, irN=irN, prN=prN,
                    diffusion=diff, h=float(h if h is not None else dom.find_h()),
                    dt=float(ts.timestep_size), num_steps=int(ts.num_timesteps),
                    output_steps=np.asarray(ts.output_steps, np.int32),
                    static_domain=bool(model.staticDomain), rho0=float(dom.rho0),
                    c0=float(dom.c0), P0=float(dom.P0),
                    gravity=tuple(dom.gravity) if dom.gravity is not None else (0.0, 0.0, 0.0),
                    u0=u0, name=model.name, data_fn=data_fn,
                    enable_pde=bool(getattr(model, "enable_pde", False)), **programs, **bcs)
