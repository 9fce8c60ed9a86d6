"""The discrete adjoint of a WetDry SSP-RK3 run through the C ABI
(``dgswe_adjoint_*`` in include/dgswe.h). No counterpart in the reference,
which has no adjoint.

The functional is a station misfit, J = Σ over the steps and the stations
of (η − η_obs)², η = h + B at the station. ``forward`` runs the steps and
returns J; ``reverse`` returns ∂J/∂ of the initial state, the bed per node,
Manning's n per node (and per element) and each boundary's tide
constituents. The derivatives are those of the steps the forward took (its
time steps and branches fixed); ``forward(..., dts=…)`` replays given time
steps, as a finite-difference check of the gradient needs. ``Adjoint.ensemble``
runs the adjoint of many members (one order) in one batched sweep."""

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
                 library: abi.Library | None = None, *, checkpoint_every: int = 0,
                 _members=None, _station_member=None):
        self.lib = library or abi.cuda_library()
        self.forms = list(_members) if _members is not None else [form]
        self.form = self.forms[0]
        self.n_members = len(self.forms)
        self.n_steps = int(n_steps)
        self.stations = np.ascontiguousarray(np.asarray(stations, dtype=np.float64).reshape(-1, 2))
        n_st = self.stations.shape[0]
        member = np.zeros(n_st, dtype=np.int32) if _station_member is None else \
            np.ascontiguousarray(np.asarray(_station_member, dtype=np.int32).reshape(-1))
        if member.shape[0] != n_st:
            raise ValueError("one member per station")
        self.station_member = member
        cfg = abi.AdjointConfig()
        cfg.scheme = abi.SSP_RK3
        cfg.cfl = cfl
        cfg.t_start = t_start
        cfg.n_steps = self.n_steps
        cfg.n_stations = n_st
        cfg.stations = self.stations.ctypes.data_as(_dp) if self.stations.size else None
        cfg.memory_budget = memory_budget
        cfg.station_member = member.ctypes.data_as(C.POINTER(C.c_int32)) if n_st else None
        cfg.checkpoint_every = int(checkpoint_every)
        handle = C.c_void_p()
        if _members is None:
            c_form, self._keep = form.to_c()
            status = self.lib.adjoint_create(C.byref(c_form), device, C.byref(cfg),
                                             C.byref(handle))
        else:
            array = (abi.Form * self.n_members)()
            self._keep = []
            for i, f in enumerate(self.forms):
                array[i], keep = f.to_c()
                self._keep.append(keep)
            self._keep.append(array)
            status = self.lib.adjoint_create_ensemble(array, self.n_members, device, C.byref(cfg),
                                                      C.byref(handle))
        if status != abi.OK:
            raw = self.lib.adjoint_last_error(handle) if handle else None
            message = (raw.decode() if raw else "") or f"status {status}"
            if handle:
                self.lib.adjoint_destroy(handle)
            raise DeviceError(status, message)
        self.handle = handle
        self.n_values = self.lib.adjoint_n_values(handle)
        self.offsets = [self.lib.adjoint_member_offset(handle, m) for m in range(self.n_members)]
        self.n_conditions = [len(f.boundaries or {}) for f in self.forms]

    @classmethod
    def ensemble(cls, forms, n_steps: int, stations, station_member, cfl: float = 0.5,
                 t_start: float = 0.0, memory_budget: float = 0.0, device: int = 0,
                 library: abi.Library | None = None, checkpoint_every: int = 0) -> "Adjoint":
        """One batched adjoint over ensemble members of one order: each member
        its own time steps and stations (``station_member``); arrays are the
        members' concatenated (``member_slice``)."""
        if not forms:
            raise ValueError("an ensemble needs at least one member")
        return cls(forms[0], n_steps, stations, cfl, t_start, memory_budget, device, library,
                   checkpoint_every=checkpoint_every, _members=forms,
                   _station_member=station_member)

    def member_slice(self, member: int) -> slice:
        """Member ``member``'s values in the concatenated per-node arrays."""
        end = self.offsets[member + 1] if member + 1 < self.n_members else self.n_values
        return slice(self.offsets[member], end)

    def member_tide(self, tide: np.ndarray, member: int) -> np.ndarray:
        """Member ``member``'s rows of the concatenated tide gradient."""
        c0 = sum(self.n_conditions[:member])
        return tide[c0:c0 + self.n_conditions[member]]

    def member_J(self) -> np.ndarray:
        """Each member's part of J from the last forward sweep."""
        out = np.zeros(self.n_members)
        self._check(self.lib.adjoint_member_misfit(self.handle, out.ctypes.data_as(_dp)))
        return out

    def _check(self, status: int):
        if status != abi.OK:
            raw = self.lib.adjoint_last_error(self.handle)
            raise DeviceError(status, (raw.decode() if raw else "") or f"status {status}")

    def station_weights(self) -> tuple[np.ndarray, np.ndarray]:
        """Each station's element and its interpolation weights [n][nn]."""
        n = self.stations.shape[0]
        nn = self.n_values // sum(f.mesh.n_elements for f in self.forms)
        elem = np.zeros(n, dtype=np.int64)
        w = np.zeros((n, nn))
        self._check(self.lib.adjoint_stations(self.handle, elem.ctypes.data_as(C.POINTER(C.c_int64)),
                                              w.ctypes.data_as(_dp)))
        return elem, w

    def forward(self, state, dts=None, eta_obs=None) -> tuple[float, np.ndarray, np.ndarray]:
        """J, η at the stations after each step [N][n_stations], and the time
        steps taken (``dts`` replayed when given), [N] for one mesh and
        [N][n_members] for an ensemble."""
        h, hu, hv = (_f64(x) for x in state)
        n_st = self.stations.shape[0]
        eta = np.zeros((self.n_steps, n_st))
        dts_out = np.zeros((self.n_steps, self.n_members)) if self.n_members > 1 \
            else np.zeros(self.n_steps)
        J = C.c_double(0.0)
        d = _f64(dts) if dts is not None else None
        obs = _f64(eta_obs) if eta_obs is not None else None
        self._check(self.lib.adjoint_forward(
            self.handle, _ptr(h), _ptr(hu), _ptr(hv), _ptr(d) if d is not None else None,
            _ptr(obs) if obs is not None else None, eta.ctypes.data_as(_dp),
            dts_out.ctypes.data_as(_dp), C.byref(J)))
        return J.value, eta, dts_out

    def reverse(self, bed: bool = True) -> Gradient:
        """The gradients of the last forward sweep; ``bed=False`` skips the
        bed's (its field is then zero), which the sweep then does not form."""
        n = self.n_values
        out = [np.zeros(n) for _ in range(5)]
        nb = max(1, sum(self.n_conditions))
        tide = np.zeros((nb, abi.MAX_CONSTITUENTS, 2))
        ptrs = [_ptr(x) for x in out]
        if not bed:
            ptrs[3] = None
        self._check(self.lib.adjoint_reverse(self.handle, *ptrs, tide.ctypes.data_as(_dp)))
        return Gradient(*out, tide)

    def set_parameters(self, manning=None, tide=None):
        """New Manning's n per node [n_values] and tide (amplitude, phase)
        [n_conditions][MAX_CONSTITUENTS][2] for the next forward sweep, in
        the gradients' layout (None: unchanged)."""
        m = _f64(manning) if manning is not None else None
        t = _f64(tide) if tide is not None else None
        if m is not None and m.size != self.n_values:
            raise ValueError("Manning's n needs one value per node")
        if t is not None and t.size != sum(self.n_conditions) * abi.MAX_CONSTITUENTS * 2:
            raise ValueError("tide needs [n_conditions][MAX_CONSTITUENTS][2] values")
        self._check(self.lib.adjoint_set_parameters(
            self.handle, _ptr(m) if m is not None else None, _ptr(t) if t is not None else None))

    def tide_parameters(self) -> np.ndarray:
        """The forms' tide (amplitude, phase) [n_conditions][MAX_CONSTITUENTS][2]."""
        out = np.zeros((max(1, sum(self.n_conditions)), abi.MAX_CONSTITUENTS, 2))
        row = 0
        for f in self.forms:
            for _, bc in sorted((f.boundaries or {}).items()):  # the C form's order
                for i, c in enumerate(getattr(bc, "constituents", None) or []):
                    out[row, i] = (c.amplitude, c.phase)
                row += 1
        return out

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
