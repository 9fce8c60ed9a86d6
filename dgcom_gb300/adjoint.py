"""The discrete adjoint of a WetDry SSP-RK3 run through the C ABI
(``dgswe_adjoint_*`` in include/dgswe.h). No counterpart in the reference,
which has no adjoint.

The functional is a station misfit, J = Σ over the steps and the stations
of (η − η_obs)², η = h + B at the station. ``forward`` runs the steps and
returns J; ``reverse`` returns ∂J/∂ of the initial state, the bed per node,
Manning's n per node (and per element) and each boundary's tide
constituents. The derivatives are those of the steps the forward took (its
time steps and branches fixed); ``forward(..., dts=…)`` replays given time
steps, as a finite-difference check of the gradient needs."""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi
from .device import DeviceError, _f64, _ptr
from .physics import SWEDeviceForm2D

_dp = C.POINTER(C.c_double)


@dataclass
class Gradient:
    h0: np.ndarray
    hu0: np.ndarray
    hv0: np.ndarray
    bed: np.ndarray        # ∂J/∂B per node
    manning: np.ndarray    # ∂J/∂n per node
    tide: np.ndarray       # [n_boundaries][MAX_CONSTITUENTS][amplitude, phase]

    def manning_per_element(self, nn: int) -> np.ndarray:
        """∂J/∂n_e for n constant on each element (nn nodes each)."""
        return self.manning.reshape(-1, nn).sum(axis=1)


class Adjoint:
    def __init__(self, form: SWEDeviceForm2D, n_steps: int, stations, cfl: float = 0.5,
                 t_start: float = 0.0, memory_budget: float = 0.0, device: int = 0,
                 library: abi.Library | None = None):
        self.lib = library or abi.cuda_library()
        self.form = form
        self.n_steps = int(n_steps)
        self.stations = np.ascontiguousarray(np.asarray(stations, dtype=np.float64).reshape(-1, 2))
        c_form, self._keep = form.to_c()
        cfg = abi.AdjointConfig()
        cfg.scheme = abi.SSP_RK3
        cfg.cfl = cfl
        cfg.t_start = t_start
        cfg.n_steps = self.n_steps
        cfg.n_stations = self.stations.shape[0]
        cfg.stations = self.stations.ctypes.data_as(_dp) if self.stations.size else None
        cfg.memory_budget = memory_budget
        handle = C.c_void_p()
        status = self.lib.adjoint_create(C.byref(c_form), device, C.byref(cfg), C.byref(handle))
        if status != abi.OK:
            raw = self.lib.adjoint_last_error(handle) if handle else None
            message = (raw.decode() if raw else "") or f"status {status}"
            if handle:
                self.lib.adjoint_destroy(handle)
            raise DeviceError(status, message)
        self.handle = handle
        self.n_values = self.lib.adjoint_n_values(handle)

    def _check(self, status: int):
        if status != abi.OK:
            raw = self.lib.adjoint_last_error(self.handle)
            raise DeviceError(status, (raw.decode() if raw else "") or f"status {status}")

    def station_weights(self) -> tuple[np.ndarray, np.ndarray]:
        """Each station's element and its interpolation weights [n][nn]."""
        n = self.stations.shape[0]
        nn = self.n_values // self.form.mesh.n_elements
        elem = np.zeros(n, dtype=np.int64)
        w = np.zeros((n, nn))
        self._check(self.lib.adjoint_stations(self.handle, elem.ctypes.data_as(C.POINTER(C.c_int64)),
                                              w.ctypes.data_as(_dp)))
        return elem, w

    def forward(self, state, dts=None, eta_obs=None) -> tuple[float, np.ndarray, np.ndarray]:
        """J, η at the stations after each step [N][n_stations], and the time
        steps taken (``dts`` replayed when given)."""
        h, hu, hv = (_f64(x) for x in state)
        n_st = self.stations.shape[0]
        eta = np.zeros((self.n_steps, n_st))
        dts_out = np.zeros(self.n_steps)
        J = C.c_double(0.0)
        d = _f64(dts) if dts is not None else None
        obs = _f64(eta_obs) if eta_obs is not None else None
        self._check(self.lib.adjoint_forward(
            self.handle, _ptr(h), _ptr(hu), _ptr(hv), _ptr(d) if d is not None else None,
            _ptr(obs) if obs is not None else None, eta.ctypes.data_as(_dp),
            dts_out.ctypes.data_as(_dp), C.byref(J)))
        return J.value, eta, dts_out

    def reverse(self) -> Gradient:
        n = self.n_values
        out = [np.zeros(n) for _ in range(5)]
        nb = max(1, len(self.form.boundaries or {}))
        tide = np.zeros((nb, abi.MAX_CONSTITUENTS, 2))
        self._check(self.lib.adjoint_reverse(self.handle, *(_ptr(x) for x in out),
                                             tide.ctypes.data_as(_dp)))
        return Gradient(*out, tide)

    def stats(self) -> abi.AdjointStats:
        s = abi.AdjointStats()
        self._check(self.lib.adjoint_get_stats(self.handle, C.byref(s)))
        return s

    def close(self):
        if getattr(self, "handle", None):
            self.lib.adjoint_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
