"""The device path behind the reference's solver API: a handle on the CUDA
library with the methods of ``PhysicsModule`` / ``LocalTimeStepping``
(src/physics/traits.rs:61-165, src/physics/builder.rs:420-783) and the
``CaseDevice::run_2d`` entry of a case run (src/case/run.rs:179-212).

Every call goes through the C ABI (include/dgswe.h); a failure raises
:class:`DeviceError` with the library's message, as the reference's device
returns ``Err(String)``. There is no CPU fallback: without the built CUDA
library, or without a GPU, construction fails."""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi
from .physics import SWEDeviceForm2D

_dp = C.POINTER(C.c_double)


class DeviceError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64).reshape(-1)


@dataclass
class DeviceRun:
    """DeviceRun (src/case/run.rs:273-289)."""

    span: tuple[float, float]
    cfl: float = 0.5
    interval: float | None = None
    dt_max: float | None = None
    dt_min: float | None = None
    max_steps: int | None = None
    scheme: int = abi.SSP_RK3
    stop: C.c_int32 | None = None  # set .value = 1 to stop at the next step
    # local time stepping's levels below the coarsest (Multirate on the
    # stepper), 0 for global steps
    levels: int = 0


@dataclass
class DeviceRunReport:
    """DeviceRunReport (src/case/run.rs:292-300) with its SimulationResult."""

    success: bool
    final_time: float
    n_steps: int
    dt_min: float
    dt_max: float
    wall_time: float
    negative_depth_clips: int
    message: str
    device: str
    # MultirateStats of a run with local time stepping (SimulationResult::
    # local_time_stepping, src/simulation/runner.rs:89-90)
    local_time_stepping: abi.MultirateStats | None = None


class SWEPhysics2D:
    """The device's SWE physics on one mesh: a dgswe handle.

    ``library`` is any :class:`abi.Library` exporting the ABI (default: the
    in-tree CUDA library)."""

    def __init__(self, form: SWEDeviceForm2D, device: int = 0, library: abi.Library | None = None):
        self.lib = library or abi.cuda_library()
        self.form = form
        c_form, self._keep = form.to_c()
        handle = C.c_void_p()
        status = self.lib.create(C.byref(c_form), device, C.byref(handle))
        if status != abi.OK:
            message = self.lib.error_text(handle, status)
            if handle:
                self.lib.destroy(handle)
            raise DeviceError(status, f"create: {message}")
        self.handle = handle
        self.n_values = int(self.lib.n_values(handle))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()

    def _check(self, status: int, what: str):
        if status != abi.OK:
            raise DeviceError(status, f"{what}: {self.lib.error_text(self.handle, status)}")

    # -- state ---------------------------------------------------------------
    def upload(self, h, hu, hv, buffer: int = abi.STATE):
        h, hu, hv = _f64(h), _f64(hu), _f64(hv)
        self._check(self.lib.upload(self.handle, buffer, _ptr(h), _ptr(hu), _ptr(hv),
                                    self.n_values), "upload")

    def download(self, buffer: int = abi.STATE):
        out = [np.empty(self.n_values) for _ in range(3)]
        self._check(self.lib.download(self.handle, buffer, *map(_ptr, out), self.n_values),
                    "download")
        return tuple(out)

    # -- PhysicsModule ---------------------------------------------------------
    def compute_rhs_into(self, time: float, input: int = abi.STATE):
        """The RHS of buffer ``input`` at ``time`` (compute_rhs_into)."""
        out = [np.empty(self.n_values) for _ in range(3)]
        self._check(self.lib.compute_rhs(self.handle, input, time, *map(_ptr, out),
                                         self.n_values), "compute_rhs")
        return tuple(out)

    def compute_rhs_mass_fluxes_into(self, time: float, input: int = abi.STATE):
        """The RHS of buffer ``input`` at ``time`` with its mass fluxes
        (compute_rhs_swe_2d_mass_fluxes_into, src/solver/rhs/swe_2d.rs:
        1042-1075): F*_h of every element face node, ``[K][4][N+1]``, and
        the mass flux through every subcell interface, ``[K][2(N+1)N]``, NaN
        in the elements without subcells."""
        n1 = self.form.order + 1
        k = self.form.mesh.n_elements
        out = [np.empty(self.n_values) for _ in range(3)]
        face = np.empty(k * 4 * n1)
        sub = np.empty(k * 2 * n1 * (n1 - 1))
        self._check(self.lib.compute_rhs_mass_fluxes(
            self.handle, input, time, *map(_ptr, out), self.n_values, _ptr(face), face.size,
            _ptr(sub), sub.size), "compute_rhs_mass_fluxes")
        return tuple(out), face.reshape(k, 4, n1), sub.reshape(k, -1)

    def autotune(self, repeats: int = 5, face_threads: int = -1, stage_shape: int = -1) -> dict:
        """dgswe_autotune: time the kernels' launch shapes on this mesh and
        state and keep the fastest (or set them, where given)."""
        t = abi.Tuning()
        self._check(self.lib.autotune(self.handle, repeats, face_threads, stage_shape,
                                      C.byref(t)), "autotune")
        return {"face_threads": t.face_threads, "stage_threads": t.stage_threads,
                "face_ms": list(t.face_ms), "stage_ms": list(t.stage_ms)}

    def element_dt(self, cfl: float, scheme: int = abi.SSP_RK3) -> np.ndarray:
        """LocalTimeStepping::element_dt: every element's stable step."""
        out = np.empty(self.form.mesh.n_elements)
        dt_min = C.c_double()
        self._check(self.lib.element_dt(self.handle, cfl, scheme, _ptr(out), C.byref(dt_min)),
                    "element_dt")
        return out

    def compute_dt_ssp(self, cfl: float, scheme: int = abi.SSP_RK3) -> float:
        """PhysicsModule::compute_dt_ssp of a wet/dry run: the smallest
        positivity-bounded element step."""
        dt_min = C.c_double()
        self._check(self.lib.element_dt(self.handle, cfl, scheme, None, C.byref(dt_min)),
                    "element_dt")
        return dt_min.value

    # -- LocalTimeStepping -------------------------------------------------------
    def stage_where(self, *, base: int, input: int, out: int, time: float, a: float, b: float,
                    c: float, acc: int | None = None, w: float = 1.0, keep: float = 0.0):
        """One stage pass over every element: out = a·base + b·input +
        c·F(input), damped, then summed into ``acc`` (w·out + keep·acc) or
        post-processed."""
        plan = abi.StagePlan(base, input, out, acc if acc is not None else 0, time, a, b, c,
                             1 if acc is not None else 0, w, keep)
        self._check(self.lib.stage(self.handle, C.byref(plan)), "stage")

    def finish_where(self, acc: int):
        """state ← acc, post-processed."""
        self._check(self.lib.finish(self.handle, acc), "finish")

    def implicit_damping(self, stage: int, from_: int, dt: float):
        """PhysicsModule::implicit_damping: buffer ``stage`` damped over ``dt``
        (bottom friction, thin-layer relaxation), the rates frozen at buffer
        ``from_``."""
        self._check(self.lib.implicit_damping(self.handle, stage, from_, dt), "implicit_damping")

    def post_process(self, buffer: int = abi.STATE):
        """PhysicsModule::post_process: the wet/dry correction of ``buffer``
        in place."""
        self._check(self.lib.post_process(self.handle, buffer), "post_process")

    # -- LocalTimeStepping passes (a host-planned multirate coarse step) ----------
    def begin_coarse_step(self, levels, rates):
        """LocalTimeStepping::begin_coarse_step: the coarse step's levels
        [n_elements] and stage rates [n_stages][n_elements]."""
        lv = np.ascontiguousarray(levels, dtype=np.uint8)
        rt = np.ascontiguousarray(rates, dtype=np.uint8)
        if lv.shape != (self.form.mesh.n_elements,) or rt.shape[1:] != lv.shape:
            raise ValueError("one level per element and one rate per stage and element")
        u8 = C.POINTER(C.c_uint8)
        self._check(self.lib.begin_coarse_step(self.handle, rt.shape[0], lv.ctypes.data_as(u8),
                                               rt.ctypes.data_as(u8)), "begin_coarse_step")

    def multirate_stage(self, plan: abi.MultirateStage):
        """LocalTimeStepping::stage_where: the stage pass over the elements
        whose rate of ``plan.stage`` is at least ``plan.depth``."""
        self._check(self.lib.stage_where(self.handle, C.byref(plan)), "stage_where")

    def multirate_finish(self, acc: int, depth: int):
        """LocalTimeStepping::finish_where: state ← acc on the elements whose
        level is at least ``depth``."""
        self._check(self.lib.finish_where(self.handle, acc, depth), "finish_where")

    def depth_flags(self, d0: float, d1: float, d2: float, buffer: int = abi.STATE) -> np.ndarray:
        """Per element, bit i set when every node of ``buffer`` is deeper
        than d_i (the line-local and coarse-step-bound tests)."""
        out = np.zeros(self.form.mesh.n_elements, dtype=np.uint8)
        self._check(self.lib.depth_flags(self.handle, buffer, d0, d1, d2,
                                         out.ctypes.data_as(C.POINTER(C.c_uint8))), "depth_flags")
        return out

    def step(self, t: float, dt: float, scheme: int = abi.SSP_RK3):
        """One fused one-level SSP step of the state."""
        self._check(self.lib.step(self.handle, scheme, t, dt), "step")

    def step_host(self, t: float, cfl: float, h, hu, hv, scheme: int = abi.SSP_RK3,
                  dt_max: float = 0.0) -> float:
        """One step of a host state (contiguous float64 arrays of n_values,
        updated in place): upload, the CFL step on the device, the step, the
        result copied back while the last stage runs. Returns the step."""
        for a in (h, hu, hv):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != self.n_values:
                raise ValueError("step_host takes contiguous float64 arrays of n_values")
        dt = C.c_double()
        self._check(self.lib.step_host(self.handle, scheme, t, cfl, dt_max, _ptr(h), _ptr(hu),
                                       _ptr(hv), self.n_values, C.byref(dt)), "step_host")
        return dt.value

    def negative_depth_clips(self) -> int:
        return int(self.lib.negative_depth_clips(self.handle))

    # -- Simulation --------------------------------------------------------------
    def run_with_callback(self, run: DeviceRun, callback=None) -> DeviceRunReport:
        """Simulation::run_with_callback on the state; ``callback(t, h, hu,
        hv)`` gets copies of the state on the host."""
        cfg = abi.RunConfig()
        cfg.scheme = run.scheme
        cfg.cfl = run.cfl
        cfg.t_start, cfg.t_end = run.span
        cfg.interval = run.interval or 0.0
        cfg.dt_max = run.dt_max or 0.0
        cfg.dt_min = run.dt_min or 0.0
        cfg.max_steps = run.max_steps or 0
        cfg.stop = C.pointer(run.stop) if run.stop is not None else None
        cfg.levels = run.levels

        def trampoline(_user, t, h, hu, hv, count):
            if callback is not None:
                callback(t, *(np.ctypeslib.as_array(p, shape=(count,)).copy() for p in (h, hu, hv)))

        cb = abi.CALLBACK(trampoline)
        report = abi.Report()
        status = self.lib.run(self.handle, C.byref(cfg), cb, None, C.byref(report))
        result = DeviceRunReport(
            success=bool(report.success), final_time=report.final_time,
            n_steps=int(report.n_steps), dt_min=report.dt_min_used, dt_max=report.dt_max_used,
            wall_time=report.wall_time, negative_depth_clips=int(report.negative_depth_clips),
            message=report.message.decode(), device=report.device.decode())
        if status not in (abi.OK, abi.ERR_NONFINITE, abi.ERR_DT_MIN, abi.ERR_MAX_STEPS,
                          abi.ERR_STOPPED):
            self._check(status, "run")
        result.status = status
        if run.levels > 0:
            stats = abi.MultirateStats()
            self._check(self.lib.multirate_stats_get(self.handle, C.byref(stats)), "stats")
            result.local_time_stepping = stats
        return result


class Cuda:
    """CaseDevice for CUDA (src/case/run.rs:179-212; the reference's
    gpu/src/case.rs:36-70): step ``form`` on device ``ordinal`` from ``q``
    over the run's span, calling ``callback(q, t)`` with the state on the
    host at the start, every interval and the end; ``q`` is left with the
    state at the end. A run that stops early (a non-finite state, a step
    below dt_min, the step limit, the stop flag) returns its report with
    ``success`` false and the reason, as the reference's SimulationResult
    does; a device failure raises :class:`DeviceError`, the reference's
    ``Err(String)``."""

    def run_2d(self, ordinal: int, form: SWEDeviceForm2D, q, run: DeviceRun,
               callback=None) -> DeviceRunReport:
        dev = SWEPhysics2D(form, ordinal)
        try:
            dev.upload(*q)
            report = dev.run_with_callback(
                run, (lambda t, h, hu, hv: callback((h, hu, hv), t)) if callback else None)
            h, hu, hv = dev.download()
            for dst, src in zip(q, (h, hu, hv)):
                dst[...] = src.reshape(dst.shape)
            return report
        finally:
            dev.close()
