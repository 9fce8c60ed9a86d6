"""The multirate level planner through the C ABI (``dgswe_planner_*`` in
include/dgswe.h; host only, no device): MultirateStepper's level assignment
(src/time/multirate.rs:527-752, 993-1157) on a form's mesh. A run with
local time stepping (``DeviceRun(levels=…)``) plans with the same code."""

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
