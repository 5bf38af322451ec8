"""GB300 (sm_103a) engine for SpatialPy's simulation hot path: the NSM exact
stochastic reaction-diffusion event loop and the SDPD particle step, behind
the ``spatialpy.Solver`` plugin interface, plus a learned surrogate for
parameter sweeps.

Modules:
  abi         ctypes bindings of include/spgpu.h (libspgpu.so)
  build       in-tree nvcc build of libspgpu.so from csrc/
  engine      ``Engine``: one sp_handle (model instances on the GPU, runs,
              moments, SDPD state, profiles)
  solver      ``GpuSolver`` (drop-in for ``spatialpy.Solver``) and
              ``GpuResult`` (the reference's ``Result`` read from memory)
  scenario    models and workloads as the flat arrays of ``sp_scenario``
  propensity  custom propensity expressions compiled to stack programs
  vtk         outputN.vtk files in the reference engine's layout
  philox      host Philox4x32-10 (trajectory keys, tests)
  fno         the surrogate network's C ABI (``FnoNet``)
  surrogate   surrogate sweeps with SSA fallback

There is no CPU fallback: without libspgpu.so or a CUDA device the engine
and the network raise.
"""
