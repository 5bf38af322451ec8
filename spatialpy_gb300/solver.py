"""Drop-in ``spatialpy.Solver`` that runs on the GPU engine.

``GpuSolver`` keeps the reference plugin interface
(spatialpy/solvers/solver.py:46-607): ``GpuSolver(model, debug_level=0)``,
``.compile(debug=False, profile=False)`` and ``.run(number_of_trajectories=1,
seed=None, timeout=None, number_of_threads=None, debug=False, profile=False,
verbose=True)``.  It also keeps the behaviour the reference's tests pin:

* trajectory i uses seed + i (solver.py:558-559); ``seed=None`` draws one;
* the ensemble is the first ``Result`` with the others appended (:602-605);
* a ``timeout`` sets ``result.timeout = True`` (:583-587);
* engine failures raise ``SimulationError`` (:499-505, 595-597).

``compile()`` converts the model with ``scenario.from_model`` (which calls
``Model.compile_prep``) and uploads it to the device.  There is no code
generation, no C++ build and no subprocess.  When spatialpy is importable
the classes subclass ``spatialpy.Solver`` / ``spatialpy.Result``, so
``isinstance`` checks and ``Result.get_species`` work unchanged.

``Model.run`` hard-codes the stock solver (model.py:1021-1056); use
:func:`run` (``run(model, solver=GpuSolver, ...)``) to pick this one.
"""
from __future__ import annotations

import os
import tempfile

import numpy as np

from . import abi
from . import scenario as S
from .engine import Engine, EngineError

try:  # the reference package, when present
    from spatialpy.core.result import Result as _RefResult
    from spatialpy.core.spatialpyerror import SimulationError
    from spatialpy.solvers.solver import Solver as _RefSolver
except Exception:  # noqa: BLE001 - any import failure means "not available"
    _RefSolver = object
    _RefResult = object

    class SimulationError(Exception):
        """Raised when the engine cannot run a model (mirrors spatialpy's)."""


class GpuResult(_RefResult):
    """One trajectory held in memory; ``read_step`` returns what the
    reference reads from ``outputN.vtk`` (result.py:270-321)."""

    def __init__(self, model, scenario, counts, times, particles=None, chem=None):
        self.model = model
        self.tspan = None
        self.success = True
        self.stdout = None
        self.stderr = None
        self.timeout = False
        self.official_vtk = False
        self.result_dir = None
        self.listOfResultObjects = [self]
        self.scenario = scenario
        self.counts = counts                      # [T, N, S] int32
        self.times = np.asarray(times, np.float64)
        self.particles = particles                # optional (x [T,N,3], v [T,N,3], rho [T,N])
        self.chem = chem                          # optional [T,N,S] deterministic concentrations

    # -- ensemble container (result.py:161-171)
    def __len__(self):
        return len(self.listOfResultObjects)

    def __getitem__(self, index):
        return self.listOfResultObjects[index]

    def append(self, item):
        self.listOfResultObjects.append(item)

    def __eq__(self, other):
        if isinstance(other, GpuResult):
            return np.array_equal(self.counts, other.counts)
        return NotImplemented

    def __ne__(self, other):
        eq = self.__eq__(other)
        return eq if eq is NotImplemented else not eq

    def __getstate__(self):
        return {k: v for k, v in self.__dict__.items()}

    def __setstate__(self, state):
        self.__dict__ = state

    def __del__(self):
        pass

    def read_step(self, step_num, debug=False):
        sc = self.scenario
        n = sc.num_particles
        if self.particles is not None:
            x, v, rho = (a[step_num] for a in self.particles)
        else:
            x, v, rho = sc.x, np.zeros((n, 3)), sc.rho
        data = {"id": np.arange(n), "type": sc.type.copy(), "v": v, "rho": rho,
                "mass": sc.mass.copy(), "bvf_phi": np.zeros(n), "nu": sc.nu.copy()}
        for s, name in enumerate(sc.species):
            if self.chem is not None:
                data[f"C[{name}]"] = self.chem[step_num][:, s].copy()
            data[f"D[{name}]"] = self.counts[step_num][:, s].astype(np.float64)
        return x, data

    def get_timespan(self):
        if self.model is not None and hasattr(self.model, "tspan"):
            self.tspan = self.model.tspan
            return self.tspan
        return self.times

    def get_species(self, species, timepoints=None, concentration=False, deterministic=False,
                    debug=False):
        if _RefResult is not object and self.model is not None:
            return super().get_species(species, timepoints, concentration, deterministic, debug)
        name = species if isinstance(species, str) else species.name
        s = self.scenario.species.index(name)
        if deterministic:
            if self.chem is None:
                raise ValueError("deterministic concentrations need a model with enable_pde")
            out = self.chem[:, :, s].copy()
        else:
            out = self.counts[:, :, s].astype(np.float64)
        if concentration:
            out = out / self.scenario.vol
        if timepoints is not None:
            out = out[timepoints]
        return out

    def export_vtk(self, directory):
        """Write outputN.vtk files in the reference layout (see vtk.py)."""
        from .vtk import write_outputs
        sc = self.scenario
        if self.particles is not None:
            x, v, rho = self.particles
        else:
            x, v, rho = sc.x, None, sc.rho
        return write_outputs(directory, x, sc.type, sc.mass, rho, sc.nu, sc.species,
                             self.counts, v=v, chem=self.chem)


class GpuSolver(_RefSolver):
    """``spatialpy.Solver`` replacement running the GB300 engine.

    Extra keyword arguments: ``device``, ``selection`` ("exact" or
    "reference", see include/spgpu.h), ``sdpd_precision`` ("f32"/"f64"),
    ``nsm_variant``.
    """

    def __init__(self, model, debug_level=0, device=0, selection="exact", sdpd_precision="f32",
                 nsm_variant=0):
        if isinstance(model, S.Scenario):
            self.model = None
            self.scenario = model
        else:
            if _RefSolver is not object:
                super().__init__(model, debug_level=debug_level)
            self.model = model
            self.scenario = None
        self.debug_level = debug_level
        self.is_compiled = False
        self.h = None
        self.device = device
        self.selection = abi.SP_SELECT_REFERENCE if selection == "reference" else abi.SP_SELECT_EXACT
        self.sdpd_precision = sdpd_precision
        self.nsm_variant = nsm_variant
        self.engine = None

    def __del__(self):
        eng = getattr(self, "engine", None)
        if eng is not None:
            eng.close()

    def compile(self, debug=False, profile=False):
        if self.model is not None:
            try:
                self.scenario = S.from_model(self.model, h=self.h)
            except NotImplementedError as err:
                raise SimulationError(str(err)) from err
        try:
            self.engine = Engine(self.scenario, device=self.device,
                                 sdpd_precision=self.sdpd_precision,
                                 nsm_variant=self.nsm_variant)
        except EngineError as err:
            raise SimulationError(f"GPU engine set-up failed: {err}") from err
        self.is_compiled = True

    def run(self, number_of_trajectories=1, seed=None, timeout=None, number_of_threads=None,
            debug=False, profile=False, verbose=True):
        if not self.is_compiled:
            self.compile(debug=debug, profile=profile)
        sc = self.scenario
        if seed is None:
            seed = int(np.random.SeedSequence().entropy % (2 ** 62))
        seeds = np.uint64(seed) + np.arange(number_of_trajectories, dtype=np.uint64)
        times = sc.output_times()
        if not sc.static_domain:
            return self._run_flow(seeds, times, timeout)
        try:
            res = self.engine.run(seeds, selection=self.selection, want_counts=True,
                                  timeout=timeout, want_chem=bool(sc.enable_pde))
        except EngineError as err:
            raise SimulationError(f"Solver execution failed: {err}") from err
        if res["rc"] == abi.SP_E_TRAJECTORY:
            raise SimulationError(f"Solver execution failed: {res.get('error')}")
        chem = res["chem"][0] if sc.enable_pde else None
        first = None
        for j in range(number_of_trajectories):
            r = GpuResult(self.model, sc, res["counts"][j], times, chem=chem)
            r.timeout = res["rc"] == abi.SP_E_TIMEOUT
            if first is None:
                first = r
            else:
                first.append(r)
        return first

    def _run_flow(self, seeds, times, timeout):
        """Moving domain: the SDPD flow with particle state at every output;
        with stochastic species, every trajectory's NSM runs over that one
        flow (queues rebuilt each step, simulate_rdme.cpp:53-68)."""
        sc = self.scenario
        if sc.num_species > 0 and sc.u0 is not None:
            try:
                res = self.engine.run(seeds, selection=self.selection, want_counts=True,
                                      timeout=timeout, want_particles=True,
                                      want_chem=bool(sc.enable_pde))
            except EngineError as err:
                raise SimulationError(f"Solver execution failed: {err}") from err
            if res["rc"] not in (abi.SP_OK, abi.SP_E_TIMEOUT):
                raise SimulationError(f"Solver execution failed: {res.get('error')}")
            particles = res["particles"][0]
            chem = res["chem"][0] if sc.enable_pde else None
            first = None
            for j in range(len(seeds)):
                r = GpuResult(self.model, sc, res["counts"][j], times, particles=particles,
                              chem=chem)
                r.timeout = res["rc"] == abi.SP_E_TIMEOUT
                if first is None:
                    first = r
                else:
                    first.append(r)
            return first
        xs, vs, rs = [], [], []
        done = 0
        for step in sc.output_steps:
            if step > done:
                self.engine.sdpd_advance(int(step - done))
                done = int(step)
            x, v, rho = self.engine.particles(0)
            xs.append(x)
            vs.append(v)
            rs.append(rho)
        counts = np.zeros((len(times), sc.num_particles, sc.num_species), np.int32)
        first = None
        for _ in seeds:
            r = GpuResult(self.model, sc, counts, times,
                          particles=(np.array(xs), np.array(vs), np.array(rs)))
            if first is None:
                first = r
            else:
                first.append(r)
        return first


def run(model, solver=GpuSolver, number_of_trajectories=1, seed=None, timeout=None,
        number_of_threads=None, debug_level=0, debug=False, profile=False, **solver_kwargs):
    """``Model.run`` with a choice of solver class (the reference's
    ``Model.run`` always builds the stock ``Solver``, model.py:1021-1056)."""
    sol = solver(model, debug_level=debug_level, **solver_kwargs)
    return sol.run(number_of_trajectories=number_of_trajectories, seed=seed, timeout=timeout,
                   number_of_threads=number_of_threads, debug=debug, profile=profile)


def default_tmpdir():
    return os.environ.get("SPATIALPY_TMPDIR", tempfile.gettempdir())
