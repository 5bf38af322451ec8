"""Run by tests/test_solver_plugin.py in a fresh interpreter whose path holds
the reference spatialpy package: the reference's own birth-death test model
(test/models/birth_death.py) through GpuSolver, which then subclasses
spatialpy.Solver.  Exits non-zero on the first failed check."""
import numpy as np

import spatialpy
from models.birth_death import create_birth_death

from spatialpy_gb300.solver import GpuResult, GpuSolver, run


def main():
    model = create_birth_death()
    sol = GpuSolver(model)
    assert isinstance(sol, spatialpy.Solver), type(sol).__mro__
    n = 200
    res = run(model, solver=GpuSolver, number_of_trajectories=n, seed=11)
    assert isinstance(res, spatialpy.Result) and isinstance(res, GpuResult)
    assert len(res) == n
    u0 = res[0].read_step(0)[1]["D[Rabbits]"]
    assert u0.sum() == 100                                   # output 0 = u0 (test_solver.py:127)
    # the same compiled solver, same seed: the same trajectory (each compile
    # scatters the initial condition anew from numpy's global generator,
    # initialcondition.py:178-197, as the reference's does)
    a = sol.run(number_of_trajectories=2, seed=5)
    b = sol.run(number_of_trajectories=1, seed=5)
    assert a[0] == b[0] and a[0] != a[1]
    tot = np.array([r.get_species("Rabbits").sum(axis=1) for r in res])   # [n, 11]
    # exact selection: immigration-death from 100 molecules, birth 10 x total
    # volume 1.21 (121 particles of volume 0.01), death 0.1 per molecule
    t = np.linspace(0.0, 10.0, 11)
    q = np.exp(-0.1 * t)
    mean = 121.0 + (100.0 - 121.0) * q
    var = 100.0 * q * (1 - q) + 121.0 * (1 - q)
    se = np.sqrt(var / n)
    assert np.all(np.abs(tot.mean(0)[1:] - mean[1:]) <= 3.29 * se[1:]), (tot.mean(0), mean)
    print(f"drop-in ok: {n} trajectories, mean at t=10 {tot[:, -1].mean():.2f} "
          f"(exact {mean[-1]:.2f})")


if __name__ == "__main__":
    main()
