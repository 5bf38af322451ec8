"""ctypes mirror of ``include/spgpu.h`` and loaders for ``libspgpu.so``.

The structures below must stay byte-for-byte identical to the C header; the
test suite checks the field offsets against the compiled library
(``sp_abi_version``) and the exported symbol list.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

SP_OK = 0
SP_E_INVALID = -1
SP_E_CUDA = -2
SP_E_NOMEM = -3
SP_E_UNSUPPORTED = -4
SP_E_TRAJECTORY = -5
SP_E_TIMEOUT = -6

SP_TRAJ_OK = 0
SP_TRAJ_NEG_COUNT = 1
SP_TRAJ_NAN_STATE = 2
SP_TRAJ_SELECT_OVERFLOW = 3
SP_TRAJ_BUDGET_EXHAUSTED = 4

SP_RXN_ZERO, SP_RXN_FIRST, SP_RXN_SECOND, SP_RXN_DIMER, SP_RXN_CUSTOM = 0, 1, 2, 3, 4
SP_BC_V, SP_BC_NU, SP_BC_RHO, SP_BC_C = 0, 1, 2, 3
SP_SELECT_EXACT, SP_SELECT_REFERENCE = 0, 1
SP_PREC_F32, SP_PREC_F64 = 0, 1

ABI_VERSION = 4

_p = C.POINTER


class SpScenario(C.Structure):
    _fields_ = [
        ("dimension", C.c_int32),
        ("num_particles", C.c_int32),
        ("x", _p(C.c_double)),
        ("v", _p(C.c_double)),
        ("type", _p(C.c_int32)),
        ("mass", _p(C.c_double)),
        ("rho", _p(C.c_double)),
        ("nu", _p(C.c_double)),
        ("fixed", _p(C.c_uint8)),
        ("num_types", C.c_int32),
        ("num_species", C.c_int32),
        ("num_reactions", C.c_int32),
        ("rxn_rate", _p(C.c_double)),
        ("rxn_kind", _p(C.c_int32)),
        ("rxn_reactants", _p(C.c_int32)),
        ("rxn_allowed", _p(C.c_uint8)),
        ("jcN", _p(C.c_int64)),
        ("irN", _p(C.c_int64)),
        ("prN", _p(C.c_int32)),
        ("diffusion", _p(C.c_double)),
        ("h", C.c_double),
        ("rho0", C.c_double),
        ("c0", C.c_double),
        ("P0", C.c_double),
        ("gravity", C.c_double * 3),
        ("dt", C.c_double),
        ("num_steps", C.c_int32),
        ("static_domain", C.c_int32),
        ("num_outputs", C.c_int32),
        ("output_steps", _p(C.c_int32)),
        ("rxn_code", _p(C.c_int32)),
        ("rxn_code_off", _p(C.c_int64)),
        ("rxn_consts", _p(C.c_double)),
        ("num_consts", C.c_int32),
        ("num_data_fn", C.c_int32),
        ("data_fn", _p(C.c_double)),
        ("enable_pde", C.c_int32),
        ("ode_code", _p(C.c_int32)),
        ("ode_code_off", _p(C.c_int64)),
        ("ode_consts", _p(C.c_double)),
        ("num_ode_consts", C.c_int32),
        ("num_bcs", C.c_int32),
        ("bc_box", _p(C.c_double)),
        ("bc_type", _p(C.c_int32)),
        ("bc_target", _p(C.c_int32)),
        ("bc_value", _p(C.c_double)),
    ]


class SpOptions(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("sdpd_precision", C.c_int32),
        ("nsm_variant", C.c_int32),
        ("sdpd_self_pair", C.c_int32),
        ("event_budget", C.c_int64),
    ]


class SpRunArgs(C.Structure):
    _fields_ = [
        ("num_trajectories", C.c_int32),
        ("selection", C.c_int32),
        ("instance", _p(C.c_int32)),
        ("seeds", _p(C.c_uint64)),
        ("u0", _p(_p(C.c_uint32))),
        ("buffers_on_device", C.c_int32),
        ("want_counts", C.c_int32),
        ("want_moments", C.c_int32),
        ("want_particles", C.c_int32),
        ("want_chem", C.c_int32),
        ("timeout_s", C.c_double),
    ]


class SpOutputs(C.Structure):
    _fields_ = [
        ("counts", _p(C.c_int32)),
        ("moments", _p(C.c_int64)),
        ("particle_x", _p(C.c_double)),
        ("particle_v", _p(C.c_double)),
        ("particle_rho", _p(C.c_double)),
        ("event_counts", _p(C.c_int64)),
        ("chem", _p(C.c_double)),
    ]


class SpProfile(C.Structure):
    _fields_ = [
        ("total_ms", C.c_double),
        ("kernel_ms", C.c_double),
        ("launches", C.c_int64),
        ("kernel", C.c_int64),
    ]


class SpTrajStatus(C.Structure):
    _fields_ = [
        ("code", C.c_int32),
        ("voxel", C.c_int32),
        ("time", C.c_double),
        ("events", C.c_int64),
        ("batches", C.c_int64),
        ("candidates", C.c_int64),
    ]


#: every entry point declared in include/spgpu.h
EXPORTED_SYMBOLS = (
    "sp_abi_version", "sp_create", "sp_run", "sp_run_start", "sp_run_continue",
    "sp_run_finish", "sp_status", "sp_last_error", "sp_destroy", "sp_get_neighbors",
    "sp_get_ddiag", "sp_get_particles", "sp_sdpd_advance", "sp_last_timing",
    "sp_last_profile", "sp_neighbors_noalloc",
    "sp_fno_create", "sp_fno_num_params", "sp_fno_set_params", "sp_fno_get_params",
    "sp_fno_get_grads", "sp_fno_forward", "sp_fno_backward", "sp_fno_adam",
    "sp_fno_train_step", "sp_fno_loss", "sp_fno_last_error", "sp_fno_destroy",
)


class SpFnoShape(C.Structure):
    """``sp_fno_shape`` of include/spgpu.h."""
    _fields_ = [(k, C.c_int32) for k in
                ("n", "width", "modes", "layers", "in_ch", "out_ch", "cond", "hidden",
                 "max_batch")]


def ptr(arr, ctype):
    """Pointer to a contiguous numpy array (or NULL for None)."""
    if arr is None:
        return C.cast(None, _p(ctype))
    if not arr.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return arr.ctypes.data_as(_p(ctype))


def scenario_struct(sc):
    """Build an ``SpScenario`` from a :class:`~spatialpy_gb300.scenario.Scenario`.

    The caller must keep ``sc`` alive while the struct is in use.
    """
    s = SpScenario()
    s.dimension = sc.dimension
    s.num_particles = sc.num_particles
    s.x = ptr(sc.x, C.c_double)
    s.v = ptr(sc.v, C.c_double)
    s.type = ptr(sc.type, C.c_int32)
    s.mass = ptr(sc.mass, C.c_double)
    s.rho = ptr(sc.rho, C.c_double)
    s.nu = ptr(sc.nu, C.c_double)
    s.fixed = ptr(sc.fixed, C.c_uint8)
    s.num_types = sc.num_types
    s.num_species = sc.num_species
    s.num_reactions = sc.num_reactions
    s.rxn_rate = ptr(sc.rxn_rate, C.c_double)
    s.rxn_kind = ptr(sc.rxn_kind, C.c_int32)
    s.rxn_reactants = ptr(sc.rxn_reactants, C.c_int32)
    s.rxn_allowed = ptr(sc.rxn_allowed, C.c_uint8)
    s.jcN = ptr(sc.jcN, C.c_int64)
    s.irN = ptr(sc.irN, C.c_int64)
    s.prN = ptr(sc.prN, C.c_int32)
    s.diffusion = ptr(sc.diffusion, C.c_double)
    s.h = sc.h
    s.rho0 = sc.rho0
    s.c0 = sc.c0
    s.P0 = sc.P0
    for d in range(3):
        s.gravity[d] = float(sc.gravity[d])
    s.dt = sc.dt
    s.num_steps = sc.num_steps
    s.static_domain = int(sc.static_domain)
    s.num_outputs = len(sc.output_steps)
    s.output_steps = ptr(sc.output_steps, C.c_int32)
    if sc.rxn_code is not None:
        s.rxn_code = ptr(sc.rxn_code, C.c_int32)
        s.rxn_code_off = ptr(sc.rxn_code_off, C.c_int64)
        s.rxn_consts = ptr(sc.rxn_consts, C.c_double)
        s.num_consts = len(sc.rxn_consts)
    if sc.data_fn is not None:
        s.num_data_fn = sc.data_fn.shape[0]
        s.data_fn = ptr(sc.data_fn, C.c_double)
    s.enable_pde = int(bool(sc.enable_pde))
    if sc.ode_code is not None:
        s.ode_code = ptr(sc.ode_code, C.c_int32)
        s.ode_code_off = ptr(sc.ode_code_off, C.c_int64)
        s.ode_consts = ptr(sc.ode_consts, C.c_double)
        s.num_ode_consts = len(sc.ode_consts)
    if sc.bc_target is not None and len(sc.bc_target):
        s.num_bcs = len(sc.bc_target)
        s.bc_box = ptr(sc.bc_box, C.c_double)
        s.bc_type = ptr(sc.bc_type, C.c_int32)
        s.bc_target = ptr(sc.bc_target, C.c_int32)
        s.bc_value = ptr(sc.bc_value, C.c_double)
    return s


_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libspgpu.so")

_lib = None


def load_library(path: str | None = None):
    """Load ``libspgpu.so`` (built in-tree by ``spatialpy_gb300.build``).

    Raises ``OSError`` when the library is missing: there is no CPU fallback.
    """
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(
            f"libspgpu.so not found at {p}; build it with "
            "`python -c 'import spatialpy_gb300.build as b; b.build()'`")
    lib = C.CDLL(p)
    lib.sp_abi_version.restype = C.c_int
    lib.sp_create.argtypes = [_p(SpScenario), C.c_int32, _p(SpOptions), _p(C.c_void_p)]
    lib.sp_create.restype = C.c_int
    lib.sp_run.argtypes = [C.c_void_p, _p(SpRunArgs), _p(SpOutputs)]
    lib.sp_run.restype = C.c_int
    lib.sp_run_start.argtypes = [C.c_void_p, _p(SpRunArgs), _p(SpOutputs)]
    lib.sp_run_start.restype = C.c_int
    lib.sp_run_continue.argtypes = [C.c_void_p, C.c_int32]
    lib.sp_run_continue.restype = C.c_int
    lib.sp_run_finish.argtypes = [C.c_void_p]
    lib.sp_run_finish.restype = C.c_int
    lib.sp_last_profile.argtypes = [C.c_void_p, _p(SpProfile)]
    lib.sp_last_profile.restype = C.c_int
    lib.sp_status.argtypes = [C.c_void_p, C.c_int32, _p(SpTrajStatus)]
    lib.sp_status.restype = C.c_int
    lib.sp_last_error.argtypes = [C.c_void_p]
    lib.sp_last_error.restype = C.c_char_p
    lib.sp_destroy.argtypes = [C.c_void_p]
    lib.sp_destroy.restype = None
    lib.sp_get_neighbors.argtypes = [C.c_void_p, C.c_int32, C.c_int32, _p(C.c_int32),
                                     _p(C.c_int32), _p(C.c_double), _p(C.c_double),
                                     _p(C.c_double)]
    lib.sp_get_neighbors.restype = C.c_int
    lib.sp_get_ddiag.argtypes = [C.c_void_p, C.c_int32, _p(C.c_double)]
    lib.sp_get_ddiag.restype = C.c_int
    lib.sp_get_particles.argtypes = [C.c_void_p, C.c_int32, _p(C.c_double), _p(C.c_double),
                                     _p(C.c_double)]
    lib.sp_get_particles.restype = C.c_int
    lib.sp_sdpd_advance.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    lib.sp_sdpd_advance.restype = C.c_int
    lib.sp_neighbors_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_double,
                                         C.c_void_p, C.c_void_p, _p(C.c_double),
                                         _p(C.c_double), C.c_int32, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_char_p, C.c_int32]
    lib.sp_neighbors_noalloc.restype = C.c_int
    lib.sp_last_timing.argtypes = [C.c_void_p, _p(C.c_double), _p(C.c_int64)]
    lib.sp_last_timing.restype = C.c_int
    vp, f32p, i32 = C.c_void_p, _p(C.c_float), C.c_int32
    lib.sp_fno_create.argtypes = [_p(SpFnoShape), _p(C.c_void_p)]
    lib.sp_fno_create.restype = C.c_int
    lib.sp_fno_num_params.argtypes = [vp]
    lib.sp_fno_num_params.restype = C.c_int64
    for name in ("sp_fno_set_params", "sp_fno_get_params", "sp_fno_get_grads"):
        getattr(lib, name).argtypes = [vp, f32p, C.c_int64]
        getattr(lib, name).restype = C.c_int
    lib.sp_fno_forward.argtypes = [vp, vp, i32, vp, i32, vp, vp]
    lib.sp_fno_forward.restype = C.c_int
    lib.sp_fno_backward.argtypes = [vp, vp, i32, vp]
    lib.sp_fno_backward.restype = C.c_int
    lib.sp_fno_adam.argtypes = [vp, C.c_float, C.c_float, C.c_float, C.c_float, vp]
    lib.sp_fno_adam.restype = C.c_int
    lib.sp_fno_train_step.argtypes = [vp, vp, i32, vp, vp, i32, _p(C.c_int32), i32, C.c_float,
                                      C.c_float, C.c_float, C.c_float, vp]
    lib.sp_fno_train_step.restype = C.c_int
    lib.sp_fno_loss.argtypes = [vp, f32p]
    lib.sp_fno_loss.restype = C.c_int
    lib.sp_fno_last_error.argtypes = [vp]
    lib.sp_fno_last_error.restype = C.c_char_p
    lib.sp_fno_destroy.argtypes = [vp]
    lib.sp_fno_destroy.restype = None
    if path is None:
        _lib = lib
    return lib


def as_np_ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)
