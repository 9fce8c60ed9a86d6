"""The multirate level planner through the C ABI (``dgswe_planner_*`` in
include/dgswe.h; host only, no device): MultirateStepper's level assignment
(src/time/multirate.rs:527-752, 993-1157) on a form's mesh. A run with
local time stepping (``DeviceRun(levels=…)``) plans with the same code.

``HostStepper`` takes multirate coarse steps with the planning on the host
and every pass through the LocalTimeStepping entry points
(``dgswe_begin_coarse_step``, ``dgswe_stage_where``, ``dgswe_finish_where``,
``dgswe_depth_flags``): the way the reference's own MultirateStepper drives
its device backend (src/time/multirate.rs:1160-1331, gpu/src/swe2d.rs:4403-4660),
and the sequence a binding that keeps that stepper follows."""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi
from .device import DeviceError
from .physics import SWEDeviceForm2D

_dp = C.POINTER(C.c_double)
_u8 = C.POINTER(C.c_uint8)


@dataclass
class Plan:
    dt: float              # the coarse step, fitted to the landing
    stable_step: float     # the step the elements (and the cap) allow
    finest: int
    evaluations: int       # element RHS evaluations per coarse step
    level_evaluations: int
    inverse_dt_sum: float
    levels: np.ndarray     # [n_elements]
    rates: np.ndarray      # [n_stages][n_elements]
    order: np.ndarray      # [n_stages + 1][n_elements]: each key's elements, largest first

    def at_or_above(self, key: int, d: int) -> list[int]:
        """The elements whose key (a stage's rate, or the level for
        key = n_stages) is at least d, in index order."""
        values = self.levels if key == self.rates.shape[0] else self.rates[key]
        return sorted(int(k) for k in self.order[key][: int((values >= d).sum())])


class Planner:
    def __init__(self, form: SWEDeviceForm2D, max_levels: int, scheme: int = abi.SSP_RK3,
                 library: abi.Library | None = None):
        self.lib = library or abi.cuda_library()
        c_form, self._keep = form.to_c()
        handle = C.c_void_p()
        status = self.lib.planner_create(C.byref(c_form), max_levels, scheme, C.byref(handle))
        if status != abi.OK:
            raise DeviceError(status, "planner_create")
        self.handle = handle
        self.n = form.mesh.n_elements
        self.n_stages = 4 if scheme == abi.SSP_RK43 else 3

    def assign(self, element_dt, line_local=None, dt_cap: float | None = None,
               landing: float | None = None) -> Plan:
        dts = np.ascontiguousarray(element_dt, dtype=np.float64).reshape(-1)
        if dts.size != self.n:
            raise ValueError("one time step per element")
        flags = None
        if line_local is not None:
            flags = np.ascontiguousarray(np.asarray(line_local, dtype=bool), dtype=np.uint8)
        levels = np.zeros(self.n, dtype=np.uint8)
        rates = np.zeros((self.n_stages, self.n), dtype=np.uint8)
        order = np.zeros((self.n_stages + 1, self.n), dtype=np.int32)
        r = abi.PlanResult()
        status = self.lib.planner_assign(
            self.handle, dts.ctypes.data_as(_dp),
            flags.ctypes.data_as(_u8) if flags is not None else None,
            dt_cap or 0.0, landing or 0.0, C.byref(r), levels.ctypes.data_as(_u8),
            rates.ctypes.data_as(_u8), order.ctypes.data_as(C.POINTER(C.c_int32)))
        if status != abi.OK:
            raise DeviceError(status, "planner_assign")
        return Plan(r.dt, r.stable_step, r.finest, r.evaluations, r.level_evaluations,
                    r.inverse_dt_sum, levels, rates, order)

    def spread(self, levels, limit: bool = False, line_local=None):
        """The jump limit (if ``limit``) and every stage's rates of given
        levels: (levels, rates [n_stages][n_elements])."""
        lv = np.ascontiguousarray(levels, dtype=np.uint8).copy()
        flags = None
        if line_local is not None:
            flags = np.ascontiguousarray(np.asarray(line_local, dtype=bool), dtype=np.uint8)
        rates = np.zeros((self.n_stages, self.n), dtype=np.uint8)
        status = self.lib.planner_spread(
            self.handle, lv.ctypes.data_as(_u8), 1 if limit else 0,
            flags.ctypes.data_as(_u8) if flags is not None else None, rates.ctypes.data_as(_u8))
        if status != abi.OK:
            raise DeviceError(status, "planner_spread")
        return lv, rates

    def close(self):
        if getattr(self, "handle", None):
            self.lib.planner_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


LINE_LOCAL_HEADROOM = 1.0         # src/physics/builder.rs:148
SUBCELL_CAP_DEPTH_FACTOR = 100.0  # src/solver/rhs/swe_2d.rs:2185
LANDING_SLACK = 1e-9              # src/time/multirate.rs:589

# Shu–Osher weights per stage (start, input, beta, c): SspScheme::stages
SHU_OSHER = {
    abi.SSP_RK3: ((1.0, 0.0, 1.0, 0.0), (0.75, 0.25, 0.25, 1.0),
                  (1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0, 0.5)),
    abi.SSP_RK43: ((1.0, 0.0, 0.5, 0.0), (0.0, 1.0, 0.5, 0.5),
                   (2.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0, 1.0), (0.0, 1.0, 0.5, 0.5)),
}


def substep_depth(p: int, finest: int) -> int:
    """The depth of finest substep p of 2^finest: the coarsest level whose
    substep starts there (MultirateStepper::schedule)."""
    if p == 0 or p == 1 << finest:
        return 0
    return finest - ((p & -p).bit_length() - 1)


class HostStepper:
    """MultirateStepper::step on a device handle, planned on the host.

    Buffers: the state (0), the stage values 1..n-1, the last stage n and
    the substep sums n+1, as in a device-driven run."""

    def __init__(self, dev, max_levels: int, scheme: int = abi.SSP_RK3):
        self.dev = dev
        self.scheme = scheme
        self.stages = SHU_OSHER[scheme]
        self.planner = Planner(dev.form, max_levels, scheme)
        c_form, _keep = dev.form.to_c()
        lines = bool(c_form.has_line_local) and dev.form.order >= 1
        depth = c_form.line_local_depth
        self.d0 = (np.inf if not lines else
                   (-np.inf if depth == -np.inf else depth + LINE_LOCAL_HEADROOM))
        self.lines = lines
        h_dry = c_form.positivity_h_dry
        self.bounded = h_dry > 0.0
        self.d1 = SUBCELL_CAP_DEPTH_FACTOR * h_dry if self.bounded else np.inf
        self.d2 = h_dry if self.bounded else np.inf
        self.plans = 0

    def start(self):
        """The stage values, the last stage's and the sums start as the
        state (src/time/multirate.rs:1287-1293)."""
        q = self.dev.download()
        for b in range(1, len(self.stages) + 2):
            self.dev.upload(*q, buffer=b)

    def coarse_step_bound(self, element_dt, flags) -> float:
        """SWEPhysics2D::coarse_step_bound (src/physics/builder.rs:610-632)."""
        if not self.bounded:
            return np.inf
        finite = np.isfinite(element_dt)
        for bit in (2, 4):
            sel = finite & ((flags & bit) != 0)
            longest = float(element_dt[sel].max()) if sel.any() else 0.0
            if longest > 0.0:
                return longest
        return np.inf

    def step(self, t: float, target: float, cfl: float, dt_max: float | None = None):
        """One coarse step from t toward target: (the new time, the plan)."""
        dev = self.dev
        dts = dev.element_dt(cfl, self.scheme)
        flags = dev.depth_flags(self.d0, self.d1, self.d2)
        bound = self.coarse_step_bound(dts, flags)
        cap = min(dt_max, bound) if dt_max else bound
        if not np.isfinite(cap):
            cap = 0.0
        plan = self.planner.assign(dts, (flags & 1) != 0 if self.lines else None, cap,
                                   target - t)
        dt = plan.stable_step
        if dt_max:
            dt = min(dt, dt_max)
        dt = min(dt, plan.dt)
        landed = t + dt * (1.0 + LANDING_SLACK) >= target
        if landed:
            dt = target - t
        dev.begin_coarse_step(plan.levels, plan.rates)
        n, L = len(self.stages), plan.finest
        for p in range(1 << L):
            d = substep_depth(p, L)
            for s, (start, inp, beta, c) in enumerate(self.stages):
                last = s + 1 == n
                dev.multirate_stage(abi.MultirateStage(
                    t, dt, L, p, d, s, int(last), start, inp, beta, c,
                    abi.STATE, abi.STATE if s == 0 else s, s + 1 if not last else n,
                    n + 1 if last else 0))
            dev.multirate_finish(n + 1, substep_depth(p + 1, L))
        self.plans += 1
        return (target if landed else t + dt), plan

    def close(self):
        self.planner.close()
