"""TEST INFRASTRUCTURE: ctypes front end of the CPU oracle.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package.  It wraps

* ``oracle/build/libsporacle.so`` — the project's C restatement of the
  SpatialPy hot path (``sp_oracle.c``, ``sdpd_oracle.c``), and
* ``oracle/_ref/libspref*.so`` — the unmodified reference engine linked with
  ``ref_driver.cpp`` (built by ``build_ref.sh`` where the reference sources
  are available).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from spatialpy_gb300.abi import SpScenario, scenario_struct

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "libsporacle.so")
REF_DIR = os.path.join(HERE, "_ref")

_p = C.POINTER
_lib = None


def build(quiet: bool = True) -> str:
    """Compile the C restatement (make in oracle/)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB


def reference_root() -> str | None:
    """Where the reference SpatialPy package lies: $SPATIALPY_REFERENCE, else
    its pip install in baseline/_ref (which carries the engine's C++ sources);
    None when neither holds a spatialpy/ directory."""
    for r in (os.environ.get("SPATIALPY_REFERENCE"),
              os.path.join(os.path.dirname(HERE), "baseline", "_ref")):
        if r and os.path.isdir(os.path.join(r, "spatialpy")):
            return r
    return None


def build_reference() -> bool:
    """Build oracle/_ref from the reference sources; False when they are absent."""
    root = reference_root()
    if root is None:
        return False
    script = os.path.join(HERE, "build_ref.sh")
    out = subprocess.run(["bash", script], capture_output=True, text=True,
                         env=dict(os.environ, SPATIALPY_REFERENCE=root))
    return out.returncode == 0


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.spo_philox4x32_10.argtypes = [_p(C.c_uint32), _p(C.c_uint32), _p(C.c_uint32)]
        L.spo_neglog.argtypes = [C.c_double]
        L.spo_neglog.restype = C.c_double
        L.spo_neighbors.argtypes = [C.c_int32, C.c_int32, _p(C.c_double), _p(C.c_double),
                                    C.c_double, _p(C.c_double), _p(C.c_double), C.c_int32,
                                    _p(C.c_int32), _p(C.c_int32), _p(C.c_double),
                                    _p(C.c_double), _p(C.c_double)]
        L.spo_diffusion_tables.argtypes = [_p(SpScenario), C.c_int32, _p(C.c_int32),
                                           _p(C.c_int32), _p(C.c_double), _p(C.c_float),
                                           _p(C.c_float)]
        L.spo_neglog_f.argtypes = [C.c_float]
        L.spo_neglog_f.restype = C.c_float
        L.spo_nsm_trajectory.argtypes = [_p(SpScenario), _p(C.c_uint32), C.c_uint64, C.c_int32,
                                         _p(C.c_int32), _p(C.c_int64)]
        L.spo_nsm_ensemble.argtypes = [_p(SpScenario), _p(C.c_uint32), _p(C.c_uint64),
                                       C.c_int32, C.c_int32, C.c_int32, _p(C.c_int32),
                                       _p(C.c_int64), _p(C.c_int32)]
        for fn in (L.spo_sdpd_f64, L.spo_sdpd_f32):
            fn.argtypes = [_p(SpScenario), C.c_int32, C.c_int32, C.c_int32, C.c_int32] + \
                [_p(C.c_double)] * 7 + [_p(C.c_int32), C.c_void_p, C.c_void_p, C.c_void_p]
        L.spo_coupled_ensemble.argtypes = [_p(SpScenario), _p(C.c_uint32), _p(C.c_uint64),
                                           C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                           C.c_int32, C.c_int32, _p(C.c_int32),
                                           _p(C.c_int64), _p(C.c_int32), _p(C.c_double),
                                           _p(C.c_double), _p(C.c_double)]
        L.spo_chem_static.argtypes = [_p(SpScenario), _p(C.c_uint32), C.c_int32,
                                      _p(C.c_double)]
        _lib = L
    return _lib


class SpoChem(C.Structure):
    _fields_ = [("C", _p(C.c_double)), ("Q", _p(C.c_double)), ("nu", _p(C.c_double))]


def _ptr(a, t):
    return a.ctypes.data_as(_p(t)) if a is not None else C.cast(None, _p(t))


def philox(ctr, key) -> np.ndarray:
    c = np.ascontiguousarray(ctr, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().spo_philox4x32_10(_ptr(c, C.c_uint32), _ptr(k, C.c_uint32), _ptr(o, C.c_uint32))
    return o


def neglog(u: float) -> float:
    return lib().spo_neglog(float(u))


def neglog_f(u: float) -> float:
    return lib().spo_neglog_f(float(u))


def neighbors(sc, kmax: int = 64, xq=None, xt=None):
    """(count, idx, dist, dWdr, Dij) with the reference predicate and order."""
    n = sc.num_particles
    xq = np.ascontiguousarray(sc.x if xq is None else xq, np.float64)
    xt = np.ascontiguousarray(sc.x if xt is None else xt, np.float64)
    cnt = np.zeros(n, np.int32)
    idx = np.full((n, kmax), -1, np.int32)
    dist = np.zeros((n, kmax))
    dw = np.zeros((n, kmax))
    dij = np.zeros((n, kmax))
    rc = lib().spo_neighbors(n, sc.dimension, _ptr(xq, C.c_double), _ptr(xt, C.c_double), sc.h,
                             _ptr(sc.mass, C.c_double), _ptr(sc.rho, C.c_double), kmax,
                             _ptr(cnt, C.c_int32), _ptr(idx, C.c_int32), _ptr(dist, C.c_double),
                             _ptr(dw, C.c_double), _ptr(dij, C.c_double))
    if rc != 0:
        raise ValueError("neighbour list overflow; raise kmax")
    return cnt, idx, dist, dw, dij


def diffusion_tables(sc, cnt, idx, dij):
    kmax = idx.shape[1]
    s = scenario_struct(sc)
    dd = np.zeros((sc.num_particles, sc.num_species), np.float32)
    cdf = np.zeros((sc.num_particles, sc.num_species, kmax), np.float32)
    lib().spo_diffusion_tables(C.byref(s), kmax, _ptr(cnt, C.c_int32), _ptr(idx, C.c_int32),
                               _ptr(np.ascontiguousarray(dij), C.c_double), _ptr(dd, C.c_float),
                               _ptr(cdf, C.c_float))
    return dd, cdf


def nsm_trajectory(sc, seed: int, selection: int = 0, u0=None):
    u0 = np.ascontiguousarray(sc.u0 if u0 is None else u0, np.uint32)
    s = scenario_struct(sc)
    out = np.zeros((len(sc.output_steps), sc.num_particles, sc.num_species), np.int32)
    ev = np.zeros(2, np.int64)
    st = lib().spo_nsm_trajectory(C.byref(s), _ptr(u0, C.c_uint32), seed, selection,
                                  _ptr(out, C.c_int32), _ptr(ev, C.c_int64))
    return out, ev, st


def nsm_ensemble(sc, seeds, selection: int = 0, threads: int = 0, want_counts: bool = True,
                 u0=None):
    """Returns (counts [ntraj,T,N,S] or None, events [ntraj,2], status [ntraj], threads)."""
    u0 = np.ascontiguousarray(sc.u0 if u0 is None else u0, np.uint32)
    seeds = np.ascontiguousarray(seeds, np.uint64)
    nt = len(seeds)
    s = scenario_struct(sc)
    out = (np.zeros((nt, len(sc.output_steps), sc.num_particles, sc.num_species), np.int32)
           if want_counts else None)
    ev = np.zeros((nt, 2), np.int64)
    st = np.zeros(nt, np.int32)
    used = lib().spo_nsm_ensemble(C.byref(s), _ptr(u0, C.c_uint32), _ptr(seeds, C.c_uint64), nt,
                                  selection, threads, _ptr(out, C.c_int32), _ptr(ev, C.c_int64),
                                  _ptr(st, C.c_int32))
    return out, ev, st, used


class SpoF32State(C.Structure):
    _fields_ = [("xh", _p(C.c_float)), ("xl", _p(C.c_float)), ("drho", _p(C.c_float)),
                ("valid", C.c_int32)]


class SdpdState:
    """Flow state between oracle calls.  x and rho are the double views; the
    FP32 flow keeps its stored state (positions as float hi + lo, densities
    as float deviations from rho0) in xh, xl, drho."""

    def __init__(self, sc):
        n = sc.num_particles
        self.xh = np.zeros((n, 3), np.float32)
        self.xl = np.zeros((n, 3), np.float32)
        self.drho = np.zeros(n, np.float32)
        self.f32_valid = 0
        self.x = sc.x.copy()
        self.v = np.zeros((n, 3)) if sc.v is None else sc.v.copy()
        self.vt = np.zeros((n, 3))
        self.rho = sc.rho.copy()
        self.F = np.zeros((n, 3))
        self.Fbp = np.zeros((n, 3))
        self.Frho = np.zeros(n)
        self.step = 0
        self.nbr_count = np.zeros(n, np.int32)
        self.nu = sc.nu.copy()      # boundary conditions may change it


def sdpd(sc, state: SdpdState, nsteps: int, precision: str = "f64", mode: int = 2,
         kmax: int = 64) -> SdpdState:
    """Advance the SDPD oracle in place.  mode bit 1 = Gauss-Seidel BVF reads,
    bit 2 = start-of-step neighbour points (both reference behaviours)."""
    s = scenario_struct(sc)
    fn = lib().spo_sdpd_f64 if precision == "f64" else lib().spo_sdpd_f32
    fs = SpoF32State(_ptr(state.xh, C.c_float), _ptr(state.xl, C.c_float),
                     _ptr(state.drho, C.c_float), state.f32_valid)
    rc = fn(C.byref(s), state.step, nsteps, mode, kmax, _ptr(state.x, C.c_double),
            _ptr(state.v, C.c_double), _ptr(state.vt, C.c_double), _ptr(state.rho, C.c_double),
            _ptr(state.F, C.c_double), _ptr(state.Fbp, C.c_double), _ptr(state.Frho, C.c_double),
            _ptr(state.nbr_count, C.c_int32), None,
            C.byref(SpoChem(None, None, _ptr(state.nu, C.c_double))), C.byref(fs))
    if rc != 0:
        raise RuntimeError(f"SDPD oracle failed (rc={rc})")
    state.f32_valid = fs.valid
    state.step += nsteps
    return state


def chem_static(sc, kmax: int = 64, u0=None):
    """Deterministic concentrations of a static domain (enable_pde) at every
    output: [T, N, S]."""
    u0 = np.ascontiguousarray(sc.u0 if u0 is None else u0, np.uint32)
    s = scenario_struct(sc)
    out = np.zeros((len(sc.output_steps), sc.num_particles, sc.num_species))
    rc = lib().spo_chem_static(C.byref(s), _ptr(u0, C.c_uint32), kmax, _ptr(out, C.c_double))
    if rc != 0:
        raise RuntimeError(f"chemistry oracle failed (rc={rc})")
    return out


def coupled_ensemble(sc, seeds, selection: int = 0, precision: str = "f32", mode: int = 6,
                     kmax: int = 48, u0=None, want_particles: bool = True, threads: int = 0,
                     want_counts: bool = True, want_chem: bool = False):
    """Moving domain with species: the SDPD flow plus, every step, new
    diffusion tables, volumes and event queues for each trajectory.
    Returns (counts [ntraj,T,N,S], events [ntraj,2], status [ntraj],
    positions [T,N,3] or None, rho [T,N] or None)."""
    u0 = np.ascontiguousarray(sc.u0 if u0 is None else u0, np.uint32)
    seeds = np.ascontiguousarray(seeds, np.uint64)
    nt, T, n = len(seeds), len(sc.output_steps), sc.num_particles
    s = scenario_struct(sc)
    out = np.zeros((nt, T, n, sc.num_species), np.int32) if want_counts else None
    ev = np.zeros((nt, 2), np.int64)
    st = np.zeros(nt, np.int32)
    px = np.zeros((T, n, 3)) if want_particles else None
    pr = np.zeros((T, n)) if want_particles else None
    ch = np.zeros((T, n, sc.num_species)) if want_chem else None
    rc = lib().spo_coupled_ensemble(C.byref(s), _ptr(u0, C.c_uint32), _ptr(seeds, C.c_uint64),
                                    nt, selection, 64 if precision == "f64" else 32, mode, kmax,
                                    threads, _ptr(out, C.c_int32), _ptr(ev, C.c_int64),
                                    _ptr(st, C.c_int32), _ptr(px, C.c_double),
                                    _ptr(pr, C.c_double), _ptr(ch, C.c_double))
    if rc != 0:
        raise RuntimeError(f"coupled oracle failed (rc={rc})")
    if want_chem:
        return out, ev, st, px, pr, ch
    return out, ev, st, px, pr


# ---------------------------------------------------------------------------
# the compiled reference engine (oracle/_ref)
# ---------------------------------------------------------------------------
_ref = {}


def reference_available(variant: str = "") -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libspref{variant}.so"))


def ref_lib(variant: str = ""):
    """variant: '' (stock -O2), '_exact' (rescaled selection), '_O0' (as shipped)."""
    if variant not in _ref:
        path = os.path.join(REF_DIR, f"libspref{variant}.so")
        if not os.path.exists(path):
            raise OSError(f"{path} missing: run oracle/build_ref.sh where the reference exists")
        L = C.CDLL(path)
        L.spref_neighbors.argtypes = [_p(SpScenario), C.c_int32, _p(C.c_int32), _p(C.c_int32),
                                      _p(C.c_double), _p(C.c_double), _p(C.c_double)]
        L.spref_nsm.argtypes = [_p(SpScenario), _p(C.c_uint32), C.c_uint64, _p(C.c_int32),
                                _p(C.c_int64)]
        L.spref_sdpd.argtypes = [_p(SpScenario), C.c_int32, _p(C.c_double), _p(C.c_double),
                                 _p(C.c_double)]
        L.spref_nsm_bench.argtypes = [_p(SpScenario), _p(C.c_uint32), C.c_uint64, C.c_int32,
                                      _p(C.c_int64), _p(C.c_double)]
        L.spref_chem.argtypes = [_p(SpScenario), _p(C.c_uint32), _p(C.c_double)]
        L.spref_coupled.argtypes = [_p(SpScenario), _p(C.c_uint32), C.c_uint64, _p(C.c_int32),
                                    _p(C.c_int64)]
        L.spref_moving_bench.argtypes = [_p(SpScenario), _p(C.c_uint32), C.c_uint64, C.c_int32,
                                         C.c_int32, _p(C.c_int64), _p(C.c_double)]
        L.spref_vtk_run.argtypes = [_p(SpScenario), _p(C.c_uint32), C.c_uint64,
                                    _p(C.c_char_p), C.c_char_p] + [_p(C.c_double)] * 5 + \
            [_p(C.c_int32), _p(C.c_double)]
        _ref[variant] = L
    return _ref[variant]


def ref_neighbors(sc, kmax: int = 64):
    n = sc.num_particles
    s = scenario_struct(sc)
    cnt = np.zeros(n, np.int32)
    idx = np.full((n, kmax), -1, np.int32)
    dist = np.zeros((n, kmax))
    dw = np.zeros((n, kmax))
    dij = np.zeros((n, kmax))
    rc = ref_lib().spref_neighbors(C.byref(s), kmax, _ptr(cnt, C.c_int32), _ptr(idx, C.c_int32),
                                   _ptr(dist, C.c_double), _ptr(dw, C.c_double),
                                   _ptr(dij, C.c_double))
    if rc != 0:
        raise ValueError(f"reference neighbour search failed ({rc})")
    return cnt, idx, dist, dw, dij


def ref_nsm(sc, seed: int, variant: str = "", u0=None):
    u0 = np.ascontiguousarray(sc.u0 if u0 is None else u0, np.uint32)
    s = scenario_struct(sc)
    out = np.zeros((len(sc.output_steps), sc.num_particles, sc.num_species), np.int32)
    ev = np.zeros(2, np.int64)
    rc = ref_lib(variant).spref_nsm(C.byref(s), _ptr(u0, C.c_uint32), seed, _ptr(out, C.c_int32),
                                    _ptr(ev, C.c_int64))
    if rc != 0:
        raise RuntimeError(f"reference NSM failed ({rc})")
    return out, ev


def _ref_bench_worker(args):
    sc, seeds, timed_from, variant = args
    L = ref_lib(variant)
    s = scenario_struct(sc)
    u0 = np.ascontiguousarray(sc.u0, np.uint32)
    events, seconds = 0, 0.0
    for seed in seeds:
        ev = np.zeros(2, np.int64)
        sec = C.c_double(0.0)
        rc = L.spref_nsm_bench(C.byref(s), _ptr(u0, C.c_uint32), int(seed), timed_from,
                               _ptr(ev, C.c_int64), C.byref(sec))
        if rc != 0:
            raise RuntimeError(f"reference NSM failed ({rc})")
        events += int(ev.sum())
        seconds += sec.value
    return events, seconds


def ref_nsm_bench(sc, seeds, timed_from: int, variant: str = "_exact", processes: int = 0):
    """All-core throughput of the compiled reference engine on a static
    domain.  The engine keeps global state (its mt19937_64 and the driver's
    tables), so trajectories run one at a time per process, spread over
    `processes` spawn-started processes (0 = every host core).  Each process
    times the event loop of steps [timed_from, nt) of its trajectories; the
    processes run side by side, so the all-core rate is the sum of their
    rates.  Returns (events/s, events timed, processes)."""
    import multiprocessing as mp
    seeds = np.asarray(seeds, np.uint64)
    processes = min(processes or os.cpu_count() or 1, len(seeds))
    chunks = [c for c in np.array_split(seeds, processes) if len(c)]
    with mp.get_context("spawn").Pool(len(chunks)) as pool:
        res = pool.map(_ref_bench_worker, [(sc, c, timed_from, variant) for c in chunks])
    rate = sum(ev / sec for ev, sec in res if sec > 0)
    return rate, sum(ev for ev, _ in res), len(chunks)


def ref_chem(sc, u0=None):
    """The reference's deterministic chemistry: concentrations [T, N, S] at
    the output steps."""
    u0 = np.ascontiguousarray(sc.u0 if u0 is None else u0, np.uint32)
    s = scenario_struct(sc)
    out = np.zeros((len(sc.output_steps), sc.num_particles, sc.num_species))
    rc = ref_lib().spref_chem(C.byref(s), _ptr(u0, C.c_uint32), _ptr(out, C.c_double))
    if rc != 0:
        raise RuntimeError(f"reference chemistry failed ({rc})")
    return out


def ref_coupled(sc, seed: int, variant: str = "", u0=None):
    """One moving-domain trajectory of the reference engine (flow + species):
    counts [T, N, S] at the output steps and (reactions, diffusions)."""
    u0 = np.ascontiguousarray(sc.u0 if u0 is None else u0, np.uint32)
    s = scenario_struct(sc)
    out = np.zeros((len(sc.output_steps), sc.num_particles, sc.num_species), np.int32)
    ev = np.zeros(2, np.int64)
    rc = ref_lib(variant).spref_coupled(C.byref(s), _ptr(u0, C.c_uint32), seed,
                                        _ptr(out, C.c_int32), _ptr(ev, C.c_int64))
    if rc != 0:
        raise RuntimeError(f"reference coupled run failed ({rc})")
    return out, ev


def _ref_moving_worker(args):
    sc, seeds, with_rdme, timed_from, variant = args
    L = ref_lib(variant)
    s = scenario_struct(sc)
    u0 = np.ascontiguousarray(sc.u0, np.uint32)
    out = []
    for seed in seeds:
        ev = np.zeros(2, np.int64)
        sec = C.c_double(0.0)
        rc = L.spref_moving_bench(C.byref(s), _ptr(u0, C.c_uint32), int(seed), int(with_rdme),
                                  timed_from, _ptr(ev, C.c_int64), C.byref(sec))
        if rc != 0:
            raise RuntimeError(f"reference moving-domain run failed ({rc})")
        out.append((int(ev.sum()), sec.value))
    return out


def ref_moving_bench(sc, seeds, with_rdme: bool, timed_from: int, variant: str = "_exact",
                     processes: int = 0):
    """The compiled engine on a moving domain, one run per seed, spread over
    `processes` spawn-started processes (0 = every host core); each run
    times its steps [timed_from, nt).  Returns [(events, seconds)] per run
    and the number of processes."""
    import multiprocessing as mp
    seeds = np.asarray(seeds, np.uint64)
    processes = min(processes or os.cpu_count() or 1, len(seeds))
    chunks = [c for c in np.array_split(seeds, processes) if len(c)]
    with mp.get_context("spawn").Pool(len(chunks)) as pool:
        res = pool.map(_ref_moving_worker,
                       [(sc, c, with_rdme, timed_from, variant) for c in chunks])
    return [x for part in res for x in part], len(chunks)


def ref_vtk_run(sc, seed: int, names, directory, variant: str = ""):
    """Runs the engine loop with the engine's own VTK writer into `directory`
    (outputN.vtk, N counting this process's files) and returns the state at
    each output: dict of x, v [T,N,3], rho, bvf_phi, nu [T,N], counts and
    chem [T,N,S]."""
    u0 = np.ascontiguousarray(sc.u0, np.uint32)
    s = scenario_struct(sc)
    T, n, S = len(sc.output_steps), sc.num_particles, sc.num_species
    r = {"x": np.zeros((T, n, 3)), "v": np.zeros((T, n, 3)), "rho": np.zeros((T, n)),
         "bvf_phi": np.zeros((T, n)), "nu": np.zeros((T, n)),
         "counts": np.zeros((T, n, S), np.int32), "chem": np.zeros((T, n, S))}
    cnames = (C.c_char_p * max(S, 1))(*[nm.encode() for nm in names])
    rc = ref_lib(variant).spref_vtk_run(
        C.byref(s), _ptr(u0, C.c_uint32), seed, cnames, os.fsencode(directory),
        *[_ptr(r[k], C.c_double) for k in ("x", "v", "rho", "bvf_phi", "nu")],
        _ptr(r["counts"], C.c_int32), _ptr(r["chem"], C.c_double))
    if rc != 0:
        raise RuntimeError(f"reference VTK run failed ({rc})")
    return r


def ref_sdpd(sc, nsteps: int):
    n = sc.num_particles
    s = scenario_struct(sc)
    x = np.zeros((n, 3))
    v = np.zeros((n, 3))
    rho = np.zeros(n)
    rc = ref_lib().spref_sdpd(C.byref(s), nsteps, _ptr(x, C.c_double), _ptr(v, C.c_double),
                              _ptr(rho, C.c_double))
    if rc != 0:
        raise RuntimeError(f"reference SDPD failed ({rc})")
    return x, v, rho
