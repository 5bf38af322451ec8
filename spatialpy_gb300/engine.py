"""Thin host layer over libspgpu's C ABI (include/spgpu.h).

:class:`Engine` owns one ``sp_handle`` (device copies of one or more model
instances) and runs ensembles through ``sp_run``.  Every call goes through
ctypes into the CUDA library; there is no host computation of the hot path
and no fallback: a missing library or device raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import SpOptions, SpOutputs, SpRunArgs, SpTrajStatus, ptr


KERNEL_NAMES = {1: "nsm_advance_generic", 2: "nsm_advance_small", 3: "nsm_advance_batch",
                4: "nsm_advance_batch+nsm_advance_small", 5: "nsm_advance_batchw2",
                6: "nsm_advance_batchw4"}


class EngineError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class Engine:
    """Device-resident model instances and their ensemble runs.

    Parameters
    ----------
    scenarios : Scenario or list of Scenario
        Model instances (a list runs heterogeneous batches in one launch).
    sdpd_precision : "f32" or "f64"
    sdpd_self_pair : "position" (default) or "step".  How a moved particle
        meets its own start-of-step point in the force pass: from the rounded
        positions, as the reference's FP64 engine (no pair when the step
        rounds away), or at the distance |dt vt| of the step.  FP32 always
        uses the step.
    nsm_variant : 0 chosen per run, 1 generic sequential warp, 2 speculative batch
        warp, 3 sequential register-resident warp, 4 / 5 speculative batches
        with 2 / 4 warps per trajectory
    """

    def __init__(self, scenarios, device: int = 0, sdpd_precision: str = "f32",
                 nsm_variant: int = 0, event_budget: int = 0, lib_path: str | None = None,
                 sdpd_self_pair: str = "position"):
        if sdpd_self_pair not in ("position", "step"):
            raise ValueError("sdpd_self_pair must be 'position' or 'step'")
        self.lib = abi.load_library(lib_path)
        if not isinstance(scenarios, (list, tuple)):
            scenarios = [scenarios]
        self.scenarios = list(scenarios)
        self._structs = (abi.SpScenario * len(scenarios))()
        for i, sc in enumerate(scenarios):
            self._structs[i] = abi.scenario_struct(sc)
        opt = SpOptions()
        opt.device = device
        opt.sdpd_precision = abi.SP_PREC_F64 if sdpd_precision == "f64" else abi.SP_PREC_F32
        opt.nsm_variant = nsm_variant
        opt.sdpd_self_pair = 1 if sdpd_self_pair == "step" else 0
        opt.event_budget = event_budget
        self._h = C.c_void_p()
        rc = self.lib.sp_create(self._structs, len(scenarios), C.byref(opt), C.byref(self._h))
        if rc != abi.SP_OK:
            msg = self.error()
            self.close()
            raise EngineError(rc, msg)

    # -- lifecycle ---------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.sp_destroy(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def error(self) -> str:
        m = self.lib.sp_last_error(self._h)
        return m.decode() if m else ""

    def _check(self, rc: int):
        if rc != abi.SP_OK:
            raise EngineError(rc, self.error())

    # -- runs ----------------------------------------------------------------
    def _prepare(self, seeds, instance, selection, want_counts, want_moments, u0, timeout,
                 want_particles=False, want_chem=False):
        seeds = np.ascontiguousarray(seeds, dtype=np.uint64).reshape(-1)
        nt = seeds.shape[0]
        inst = None
        if instance is not None:
            inst = np.ascontiguousarray(instance, dtype=np.int32).reshape(nt)
        u0s = []
        for i, sc in enumerate(self.scenarios):
            a = sc.u0 if u0 is None else (u0[i] if isinstance(u0, (list, tuple)) else u0)
            u0s.append(None if a is None else np.ascontiguousarray(a, dtype=np.uint32))
        u0p = (C.POINTER(C.c_uint32) * len(u0s))()
        for i, a in enumerate(u0s):
            u0p[i] = ptr(a, C.c_uint32)
        args = SpRunArgs()
        args.num_trajectories = nt
        args.selection = selection
        args.instance = ptr(inst, C.c_int32)
        args.seeds = ptr(seeds, C.c_uint64)
        args.u0 = u0p
        args.buffers_on_device = 0
        args.want_counts = int(want_counts)
        args.want_moments = int(want_moments)
        args.timeout_s = float(timeout or 0.0)
        T = [len(sc.output_steps) for sc in self.scenarios]
        idx = np.zeros(nt, np.int64) if inst is None else inst.astype(np.int64)
        sizes = [T[i] * self.scenarios[i].num_particles * self.scenarios[i].num_species
                 for i in idx]
        counts = np.zeros(int(sum(sizes)) if want_counts else 0, np.int32)
        msizes = [T[i] * sc.num_particles * sc.num_species for i, sc in enumerate(self.scenarios)]
        moments = np.zeros(2 * int(sum(msizes)) if want_moments else 0, np.int64)
        events = np.zeros((nt, 2), np.int64)
        out = SpOutputs()
        out.counts = ptr(counts if want_counts else None, C.c_int32)
        out.moments = ptr(moments if want_moments else None, C.c_int64)
        out.event_counts = ptr(events, C.c_int64)
        # moving domains: flow state at every output, instance-major
        psizes = [T[i] * sc.num_particles for i, sc in enumerate(self.scenarios)]
        np_tot = int(sum(psizes)) if want_particles else 0
        px = np.zeros(3 * np_tot)
        pv = np.zeros(3 * np_tot)
        prho = np.zeros(np_tot)
        args.want_particles = int(want_particles)
        csizes = [T[i] * sc.num_particles * sc.num_species for i, sc in enumerate(self.scenarios)]
        chem = np.zeros(int(sum(csizes)) if want_chem else 0)
        args.want_chem = int(want_chem)
        if want_chem:
            out.chem = ptr(chem, C.c_double)
        if want_particles:
            out.particle_x = ptr(px, C.c_double)
            out.particle_v = ptr(pv, C.c_double)
            out.particle_rho = ptr(prho, C.c_double)
        # keep every buffer the C side points at alive for the run
        self._run = dict(seeds=seeds, inst=inst, u0s=u0s, u0p=u0p, args=args, out=out, T=T,
                         idx=idx, sizes=sizes, counts=counts, msizes=msizes, moments=moments,
                         events=events, want_counts=want_counts, want_moments=want_moments,
                         want_particles=want_particles, psizes=psizes, px=px, pv=pv, prho=prho,
                         want_chem=want_chem, csizes=csizes, chem=chem)
        return self._run

    def _collect(self, rc):
        r = self._run
        nt = r["seeds"].shape[0]
        status = np.array([self.status(j)["code"] for j in range(nt)], np.int32)
        if rc not in (abi.SP_OK, abi.SP_E_TRAJECTORY, abi.SP_E_TIMEOUT):
            raise EngineError(rc, self.error())
        res = {"events": r["events"], "status": status, "rc": rc}
        if rc != abi.SP_OK:
            res["error"] = self.error()
        T = r["T"]
        if r["want_counts"]:
            parts, o = [], 0
            for j, i in enumerate(r["idx"]):
                sc = self.scenarios[i]
                n = r["sizes"][j]
                parts.append(r["counts"][o:o + n].reshape(T[i], sc.num_particles, sc.num_species))
                o += n
            res["counts"] = parts
        if r["want_moments"]:
            parts, o = [], 0
            for i, sc in enumerate(self.scenarios):
                n = r["msizes"][i]
                parts.append(r["moments"][2 * o:2 * (o + n)].reshape(
                    T[i], sc.num_particles, sc.num_species, 2))
                o += n
            res["moments"] = parts
        if r["want_particles"]:
            xs, vs, rs, o = [], [], [], 0
            for i, sc in enumerate(self.scenarios):
                n = r["psizes"][i]
                xs.append(r["px"][3 * o:3 * (o + n)].reshape(T[i], sc.num_particles, 3))
                vs.append(r["pv"][3 * o:3 * (o + n)].reshape(T[i], sc.num_particles, 3))
                rs.append(r["prho"][o:o + n].reshape(T[i], sc.num_particles))
                o += n
            res["particles"] = list(zip(xs, vs, rs))
        if r["want_chem"]:
            parts, o = [], 0
            for i, sc in enumerate(self.scenarios):
                n = r["csizes"][i]
                parts.append(r["chem"][o:o + n].reshape(T[i], sc.num_particles, sc.num_species))
                o += n
            res["chem"] = parts
        return res

    def run(self, seeds, instance=None, selection: int = abi.SP_SELECT_EXACT,
            want_counts: bool = True, want_moments: bool = False, u0=None,
            timeout: float | None = None, want_particles: bool = False,
            want_chem: bool = False):
        """Run one trajectory per seed over the whole time span.

        Returns a dict with ``counts`` (list per trajectory of [T,N,S] int32
        arrays) when ``want_counts``, ``moments`` (list per instance of
        [T,N,S,2] int64 sums of x and x^2) when ``want_moments``, ``events``
        ([ntraj,2] reaction/diffusion counts) and ``status`` codes.  On a
        moving domain every trajectory shares the flow; ``want_particles``
        adds ``particles`` (per instance: positions [T,N,3], velocities
        [T,N,3], densities [T,N] at the outputs); ``want_chem`` adds
        ``chem`` (per instance with enable_pde: concentrations [T,N,S]).
        """
        r = self._prepare(seeds, instance, selection, want_counts, want_moments, u0, timeout,
                          want_particles, want_chem)
        rc = self.lib.sp_run(self._h, C.byref(r["args"]), C.byref(r["out"]))
        return self._collect(rc)

    def start(self, seeds, instance=None, selection: int = abi.SP_SELECT_EXACT,
              want_counts: bool = False, want_moments: bool = False, u0=None,
              timeout: float | None = None):
        """Begin a run (queues built, outputs at step 0 written); see advance/finish."""
        r = self._prepare(seeds, instance, selection, want_counts, want_moments, u0, timeout)
        self._check(self.lib.sp_run_start(self._h, C.byref(r["args"]), C.byref(r["out"])))

    def advance(self, num_outputs: int = 1) -> int:
        """Advance the run through the next ``num_outputs`` outputs."""
        rc = self.lib.sp_run_continue(self._h, int(num_outputs))
        if rc not in (abi.SP_OK,):
            raise EngineError(rc, self.error())
        return rc

    def finish(self):
        rc = self.lib.sp_run_finish(self._h)
        return self._collect(rc)

    def profile(self) -> dict:
        p = abi.SpProfile()
        self._check(self.lib.sp_last_profile(self._h, C.byref(p)))
        return {"total_ms": p.total_ms, "kernel_ms": p.kernel_ms, "launches": p.launches,
                "kernel": KERNEL_NAMES.get(p.kernel, "none")}

    def status(self, j: int) -> dict:
        st = SpTrajStatus()
        self._check(self.lib.sp_status(self._h, j, C.byref(st)))
        return {"code": st.code, "voxel": st.voxel, "time": st.time, "events": st.events,
                "batches": st.batches, "candidates": st.candidates}

    def last_timing(self):
        ms = C.c_double()
        n = C.c_int64()
        self._check(self.lib.sp_last_timing(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    # -- inspection ------------------------------------------------------------
    def neighbors(self, inst: int = 0, kmax: int = 64):
        sc = self.scenarios[inst]
        n = sc.num_particles
        cnt = np.zeros(n, np.int32)
        idx = np.full((n, kmax), -1, np.int32)
        dist = np.zeros((n, kmax))
        dw = np.zeros((n, kmax))
        dij = np.zeros((n, kmax))
        self._check(self.lib.sp_get_neighbors(self._h, inst, kmax, ptr(cnt, C.c_int32),
                                              ptr(idx, C.c_int32), ptr(dist, C.c_double),
                                              ptr(dw, C.c_double), ptr(dij, C.c_double)))
        return cnt, idx, dist, dw, dij

    def ddiag(self, inst: int = 0):
        sc = self.scenarios[inst]
        out = np.zeros((sc.num_particles, sc.num_species))
        self._check(self.lib.sp_get_ddiag(self._h, inst, ptr(out, C.c_double)))
        return out

    def particles(self, inst: int = 0):
        n = self.scenarios[inst].num_particles
        x = np.zeros((n, 3))
        v = np.zeros((n, 3))
        rho = np.zeros(n)
        self._check(self.lib.sp_get_particles(self._h, inst, ptr(x, C.c_double),
                                              ptr(v, C.c_double), ptr(rho, C.c_double)))
        return x, v, rho

    def sdpd_advance(self, nsteps: int, inst: int = 0):
        self._check(self.lib.sp_sdpd_advance(self._h, inst, nsteps))
