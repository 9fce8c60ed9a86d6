"""Ensembles of independent runs advanced together on one device.

No counterpart in the reference, which runs one case per
``CaseDevice::run_2d`` call (src/case/run.rs:179-212): a member is what one
such call runs. Members may differ in mesh, order, bathymetry, Manning
coefficient and boundary data; every other physics option is shared. Each
member takes its own time step, and a member's result equals a run of that
member alone, bit for bit. All calls go through the C ABI
(``dgswe_ensemble_*`` in include/dgswe.h); there is no CPU fallback."""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .device import DeviceError, DeviceRunReport, _f64, _ptr
from .physics import SWEDeviceForm2D


class Ensemble:
    """A dgswe_ensemble handle over ``forms`` (one per member)."""

    def __init__(self, forms: list[SWEDeviceForm2D], device: int = 0,
                 library: abi.Library | None = None):
        self.lib = library or abi.cuda_library()
        if not forms:
            raise ValueError("an ensemble needs at least one member")
        self.forms = list(forms)
        self._keep = []
        array = (abi.Form * len(forms))()
        for i, form in enumerate(forms):
            c_form, keep = form.to_c()
            array[i] = c_form
            self._keep.append(keep)
        self._array = array
        handle = C.c_void_p()
        status = self.lib.ensemble_create(array, len(forms), device, C.byref(handle))
        if status != abi.OK:
            message = self._error(handle, status)
            if handle:
                self.lib.ensemble_destroy(handle)
            raise DeviceError(status, message)
        self.handle = handle

    def _error(self, handle, status: int) -> str:
        raw = self.lib.ensemble_last_error(handle) if handle else None
        return (raw.decode() if raw else "") or f"status {status}"

    def _check(self, status: int):
        if status != abi.OK:
            raise DeviceError(status, self._error(self.handle, status))

    @property
    def n_members(self) -> int:
        return self.lib.ensemble_n_members(self.handle)

    def n_values(self, member: int) -> int:
        return self.lib.ensemble_n_values(self.handle, member)

    def upload(self, member: int, h, hu, hv):
        arrays = [_f64(x) for x in (h, hu, hv)]
        self._check(self.lib.ensemble_upload(self.handle, member, *map(_ptr, arrays),
                                             arrays[0].size))

    def download(self, member: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        n = self.n_values(member)
        out = [np.empty(n) for _ in range(3)]
        self._check(self.lib.ensemble_download(self.handle, member, *map(_ptr, out), n))
        return out[0], out[1], out[2]

    def run(self, steps: int, cfl: float, scheme: int = abi.SSP_RK3, t_start: float = 0.0,
            dt_max: float | None = None, dt_min: float | None = None,
            raise_on_failure: bool = True) -> tuple[list[DeviceRunReport], abi.Profile]:
        """``steps`` SSP steps of every member from ``t_start``: the members'
        reports and the device time of the steps."""
        cfg = abi.RunConfig()
        cfg.scheme = scheme
        cfg.cfl = cfl
        cfg.t_start = t_start
        cfg.t_end = 0.0
        cfg.interval = 0.0
        cfg.dt_max = dt_max or 0.0
        cfg.dt_min = dt_min or 0.0
        cfg.max_steps = 0
        reports = (abi.Report * len(self.forms))()
        profile = abi.Profile()
        status = self.lib.ensemble_run(self.handle, C.byref(cfg), steps, reports, C.byref(profile))
        if status != abi.OK and raise_on_failure:
            raise DeviceError(status, self._error(self.handle, status))
        out = [DeviceRunReport(success=bool(r.success), final_time=r.final_time,
                               n_steps=r.n_steps, dt_min=r.dt_min_used, dt_max=r.dt_max_used,
                               wall_time=r.wall_time, negative_depth_clips=r.negative_depth_clips,
                               message=r.message.decode(), device=r.device.decode())
               for r in reports]
        return out, profile

    def close(self):
        if getattr(self, "handle", None):
            self.lib.ensemble_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
