"""The Solver plugin boundary and the VTK output format.

CPU tests import the reference package (where its sources exist) to check the
model conversion of its own test models and that its VTKReader reads files
written here.  GPU tests run the reference's solver tests
(test/integration_tests/test_solver.py:127-200) against GpuSolver."""
import numpy as np
import pytest

from spatialpy_gb300 import abi
from spatialpy_gb300 import scenario as S
from spatialpy_gb300 import vtk

from .refmodels import spatialpy_or_skip


def test_from_model_birth_death():
    spatialpy = spatialpy_or_skip()
    from models.birth_death import create_birth_death
    model = create_birth_death()
    sc = S.from_model(model)
    assert sc.num_particles == 121                     # create_2D_domain overshoot (numx=10)
    assert sc.species == ["Rabbits"]
    assert np.isclose(sc.h, model.domain.find_h())
    assert list(sc.rxn_kind) == [abi.SP_RXN_ZERO, abi.SP_RXN_FIRST]
    assert list(sc.rxn_rate) == [10.0, 0.1]
    assert sc.u0.sum() == 100 and sc.dimension == 2 and sc.static_domain
    assert list(sc.output_steps) == list(range(11)) and sc.dt == 1.0
    assert np.allclose(sc.diffusion, 0.1)


def test_from_model_restrictions_and_dimer():
    spatialpy = spatialpy_or_skip()
    m = spatialpy.Model("restr")
    dom = spatialpy.Domain.create_2D_domain(xlim=(0, 1), ylim=(0, 1), numx=6, numy=6,
                                            type_id="bulk", fixed=True)
    m.add_domain(dom)
    A = spatialpy.Species(name="A", diffusion_coefficient=0.1, restrict_to="bulk")
    B = spatialpy.Species(name="B", diffusion_coefficient=0.2)
    m.add_species([A, B])
    m.add_parameter(spatialpy.Parameter(name="k", expression=0.5))
    m.add_reaction(spatialpy.Reaction(name="dim", reactants={"A": 2}, products={"B": 1},
                                      rate="k"))
    m.add_reaction(spatialpy.Reaction(name="bi", reactants={"A": 1, "B": 1}, products={},
                                      rate="k", restrict_to="bulk"))
    m.add_initial_condition(spatialpy.ScatterInitialCondition(species="A", count=30))
    m.timespan(spatialpy.TimeSpan.linspace(t=2, num_points=3, timestep_size=0.5))
    sc = S.from_model(m)
    assert list(sc.rxn_kind) == [abi.SP_RXN_DIMER, abi.SP_RXN_SECOND]
    assert sc.rxn_allowed is not None and sc.rxn_allowed[1].sum() == 1
    assert sc.num_steps == 4 and list(sc.output_steps) == [0, 2, 4]


def test_vtk_layout_read_by_reference_reader(tmp_path):
    spatialpy_or_skip()
    from spatialpy.core.vtkreader import VTKReader
    sc = S.config_birth_death_2d(n=5)
    counts = np.stack([sc.u0, sc.u0 + 1]).astype(np.int32)
    paths = vtk.write_outputs(str(tmp_path), sc.x, sc.type, sc.mass, sc.rho, sc.nu, sc.species,
                              counts)
    for k, p in enumerate(paths):
        r = VTKReader(filename=p)
        r.read_file()
        pts = r.get_points()
        arr = r.get_arrays()
        assert np.allclose(np.asarray(pts, float).reshape(-1, 3), sc.x)
        np.testing.assert_array_equal(np.asarray(arr["D[Rabbits]"], float), counts[k, :, 0])
        assert np.allclose(np.asarray(arr["rho"], float), sc.rho)
        ours = vtk.read_step(p)[1]
        np.testing.assert_array_equal(ours["D[Rabbits]"], counts[k, :, 0])


def test_vtk_round_trip(tmp_path):
    sc = S.config_rdme_3d(n=4, nA=20, nB=10)
    counts = np.random.default_rng(0).integers(0, 50, (3, sc.num_particles, 3)).astype(np.int32)
    paths = vtk.write_outputs(str(tmp_path), sc.x, sc.type, sc.mass, sc.rho, sc.nu, sc.species,
                              counts, bbox=(0, 1, 0, 1, 0, 1))
    for k, p in enumerate(paths):
        pts, arr = vtk.read_step(p)
        assert np.allclose(pts, sc.x, rtol=1e-9)
        for s, name in enumerate(sc.species):
            np.testing.assert_array_equal(arr[f"D[{name}]"], counts[k, :, s])
        assert open(p).read().count("FIELD FieldData") == 1


# ---------------------------------------------------------------------------
# GPU: the reference's solver tests against GpuSolver
# ---------------------------------------------------------------------------
MOLECULES = 1000


def _diffusion_debug():
    """create_diffusion_debug (test_solver.py:28-46): 50x50 2-D domain on
    [-1,1]^2, mass 1 and rho = mass / vol (Domain.add_point, domain.py:244-245),
    one species D=0.01, dt 0.1, 11 outputs over t in [0,10].  The reference
    places 100,000 molecules at the origin particle (about 2e8 diffusion
    events per trajectory); 1,000 keep this test to seconds and leave every
    check below meaningful."""
    ax = np.linspace(-1.0, 1.0, 50)
    x = S.lattice([ax, ax])
    n = x.shape[0]
    rate, kind, reac, allowed, jcN, irN, prN = S.mass_action(["A"], [], 1)
    u0 = np.zeros((n, 1), np.uint32)
    u0[np.argmin(np.linalg.norm(x, axis=1)), 0] = MOLECULES
    nt, steps = S.timespan(10.0, 11, 0.1)
    return S.Scenario(dimension=2, x=x, type=np.ones(n), mass=1.0, rho=n / 4.0, nu=1.0, fixed=1,
                      num_types=1, species=["A"], rxn_rate=rate, rxn_kind=kind,
                      rxn_reactants=reac.reshape(0, 2), rxn_allowed=allowed, jcN=jcN, irN=irN,
                      prN=prN, diffusion=np.array([[0.01]]), h=S.find_h(x), dt=0.1,
                      num_steps=nt, output_steps=steps, static_domain=True, rho0=1.0, c0=1.0,
                      P0=1.0, u0=u0, name="diffusion_debug")


@pytest.mark.gpu
def test_reference_solver_tests_on_gpu_solver():
    from spatialpy_gb300.solver import GpuSolver
    sc = _diffusion_debug()
    sol = GpuSolver(sc)
    r1 = sol.run(seed=1)
    np.testing.assert_array_equal(r1.read_step(0)[1]["D[A]"], sc.u0[:, 0])   # test_solver_io
    assert r1.get_species("A").shape == (11, sc.num_particles)
    assert r1.get_species("A")[-1].sum() == MOLECULES                         # conserved
    assert r1 == sol.run(seed=1)                                              # test_same_seed
    assert r1 != sol.run(seed=2)                                              # test_different_seeds
    ens = sol.run(number_of_trajectories=3, seed=7)                           # test_run_ensemble
    assert len(ens) == 3 and ens[0] != ens[1]
    assert ens[1] == sol.run(seed=8)                                          # trajectory i: seed + i
    spread = (r1.get_species("A")[-1] > 0).sum()
    assert spread > 100                                                       # it diffused


@pytest.mark.gpu
def test_gpu_solver_exports_reference_vtk(tmp_path):
    from spatialpy_gb300.solver import GpuSolver
    sc = S.config_birth_death_2d()
    r = GpuSolver(sc).run(seed=3)
    paths = r.export_vtk(str(tmp_path))
    assert len(paths) == 11
    for k, p in enumerate(paths):
        np.testing.assert_array_equal(vtk.read_step(p)[1]["D[Rabbits]"], r.counts[k][:, 0])


@pytest.mark.gpu
def test_real_model_through_gpu_solver_subclass():
    """The drop-in with a real spatialpy.Model: in a fresh interpreter whose
    path holds the reference package, GpuSolver subclasses spatialpy.Solver
    (Solver.__init__ enforces the subclass, solver.py:56-61) and runs the
    reference's own birth-death test model through run(model,
    solver=GpuSolver): Result instances, output 0 = u0, seed reproducibility,
    and the exact immigration-death mean at every output for 200
    trajectories (tests/gpu_model_dropin.py)."""
    import os
    import subprocess
    import sys
    from .refmodels import REF, STUBS
    if REF is None:
        pytest.skip("reference package not present")
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1",
               PYTHONPATH=os.pathsep.join([root, STUBS, REF, os.path.join(REF, "test")]))
    r = subprocess.run([sys.executable, os.path.join(here, "gpu_model_dropin.py")], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "drop-in ok" in r.stdout
