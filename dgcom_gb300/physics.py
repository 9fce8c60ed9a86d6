"""The 2D physics as the device runs it: ``SWEDeviceForm2D``
(src/physics/device.rs:27-62) as plain host data, turned into the C ABI's
``dgswe_form`` by :meth:`SWEDeviceForm2D.to_c`.

Defaults follow the reference's case runner (src/case/run.rs:642-787): g =
9.81, h_min = 1e-6, the `WetDry` split form with subcells below 1 mm, the
wet/dry correction with h_dry = 1 mm, a 1 s thin-layer time and a 20 m/s
velocity cap, its positivity-bounded step, and walls (Reflective2D,
h_min 1e-6) on untagged faces."""

from __future__ import annotations

import math

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .mesh import TAG_WALL, QuadMesh, node_positions


@dataclass
class WallBoundary:
    """Reflective2D (src/boundary/boundary_2d.rs:249-300)."""

    h_min: float = 1e-6


@dataclass
class TidalBoundary:
    """CharacteristicOBC with a uniform HarmonicTide
    (src/boundary/characteristic.rs:360-437, src/boundary/harmonic_tide.rs)."""

    constituents: list = field(default_factory=list)  # abi.TideConstituent
    mean_elevation: float = 0.0
    ramp_duration: float | None = 3600.0
    incoming_wave: bool = False
    # InverseBarometer (src/boundary/characteristic.rs:273-340): the external
    # η raised by this factor times the form's atmosphere's level; None: not
    raise_factor: float | None = None


@dataclass
class NodeTidesBoundary:
    """CharacteristicOBC with BoundaryTides: an atlas's harmonic constants
    per forced boundary node (src/boundary/tidal_atlas.rs:855-1070, the
    device form DeviceExternal2D::Tides). ``coefficients`` [n_slots][n][6]
    are C, S of η, u and v per constituent at the epoch's nodal terms;
    ``omega`` ω′ and ``f_rate`` ḟ/f₀ per constituent; ``slot_of_node`` the
    slot of each flat mesh node (0xFFFFFFFF: none; None: by nearest
    position)."""

    omega: np.ndarray
    f_rate: np.ndarray
    positions: np.ndarray            # [n_slots][2]
    coefficients: np.ndarray         # [n_slots][n][6]
    mean: np.ndarray | None = None
    source_depth: np.ndarray | None = None
    slot_of_node: np.ndarray | None = None
    velocity: bool = False
    use_mean: bool = False
    max_transport_ratio: float | None = None
    ramp_duration: float | None = None
    incoming_wave: bool = False
    raise_factor: float | None = None


@dataclass
class ParentBoundary:
    """CharacteristicOBC driven by a parent model's state per boundary node
    (OceanModelState, src/boundary/ocean_nesting.rs; the device form
    DeviceExternal2D::Parent). ``values`` [n_slots][n_times][3] are ζ, u, v
    (stored as float32, as the reference stores them) at the snapshot
    ``times`` (simulation seconds); ``cubic`` Lagrange through up to four
    snapshots, else linear."""

    positions: np.ndarray            # [n_slots][2]
    times: np.ndarray                # [n_times]
    values: np.ndarray               # [n_slots][n_times][3]
    parent_depth: np.ndarray | None = None
    on_boundary: np.ndarray | None = None
    slot_of_node: np.ndarray | None = None
    cubic: bool = True
    velocity: bool = True
    reference_level: float = 0.0
    max_transport_ratio: float | None = None
    ramp_duration: float | None = None
    incoming_wave: bool = False
    raise_factor: float | None = None


@dataclass
class RelaxationBand:
    """NestingRelaxation2D (src/boundary/ocean_nesting.rs:900-1065; the
    device source DeviceSource2D::NestingRelaxation): relax the band's nodes
    towards ``parent`` (its slot_of_node covers them) at rate ``weight[slot]
    · rate``."""

    parent: "ParentBoundary"
    weight: np.ndarray             # [n_slots]
    rate: float                    # 1/τ (1/s)
    wet_depth: float = 0.05
    momentum_only: bool = False


@dataclass
class GriddedAtmosphere:
    """GriddedAtmosphere2D (src/source/swe_2d/gridded_atmosphere.rs) as a
    device holds it: a weather model's snapshots regridded onto the mesh
    nodes (``values`` [n_times][n_values][5] f32: u, v, ∂p/∂x, ∂p/∂y,
    p − p_ref, the wind in the mesh axes, unramped) at the Unix ``times``,
    with ``epoch_unix`` the Unix time of simulation time 0 (ModelClock).
    With ``source`` it is the device source DeviceSource2D::Atmosphere (the
    wind stress where ``wind``, the pressure gradient where ``pressure``);
    boundaries with a ``raise_factor`` read its inverse-barometer level,
    which is the pressure's when ``pressure`` and the weather has a pressure
    field (``has_pressure``; GriddedAtmosphere2D::has_level), else 0. The
    defaults are the reference's: Large & Pond drag, ρ_air 1.225 kg/m³,
    ρ 1025 kg/m³, nodes shallower than 1 cm not forced, no ramp."""

    times: np.ndarray
    values: np.ndarray
    epoch_unix: float = 0.0
    source: bool = True
    wind: bool = True
    pressure: bool = True
    has_pressure: bool = True
    drag: int = abi.DRAG_LARGE_POND
    drag_cd: float = 0.0
    rho_air: float = 1.225
    rho_water: float = 1025.0
    h_min: float = 0.01
    ramp_duration: float | None = None

    def model_times(self) -> np.ndarray:
        """The snapshots' simulation times."""
        return np.asarray(self.times, dtype=np.float64) - self.epoch_unix


@dataclass
class SWEDeviceForm2D:
    mesh: QuadMesh
    order: int
    bathymetry: np.ndarray | None = None  # (n_elements, (N+1)²)
    g: float = 9.81
    h_min: float = 1e-6
    formulation: int = abi.WET_DRY
    subcell_depth: float = 1e-3
    subcell_h_dry: float = 1e-3
    wet_dry: bool = True
    h_dry: float = 1e-3
    relaxation_time: float = 1.0
    max_velocity: float = 20.0
    positivity_h_dry: float | None = 1e-3
    manning_n: float | np.ndarray | None = None  # uniform n, or n per node
    friction_g: float | None = None
    manning_h_min: float = 1e-6
    coriolis_f0: float | None = None
    coriolis_beta: float = 0.0
    coriolis_y0: float = 0.0
    boundaries: dict = field(default_factory=lambda: {TAG_WALL: WallBoundary()})
    numerics: int = abi.NUMERICS_FAST
    # Local time stepping: the depth below which a node takes its element out
    # of the line-local form (SWEDeviceForm2D::line_local_depth,
    # src/physics/device.rs:62-66); None: no element is line-local; "auto":
    # SWEPhysics2D::line_local_depth's value for this form
    # (src/physics/builder.rs:296-322), the WetDry subcells' depth and the
    # wet/dry correction's h_dry, whichever is deeper
    line_local_depth: float | None | str = "auto"
    relaxation: RelaxationBand | None = None
    atmosphere: GriddedAtmosphere | None = None

    def local_depth(self) -> float | None:
        """The line-local depth the C form carries (None: none)."""
        if self.line_local_depth != "auto":
            return self.line_local_depth
        if self.formulation != abi.WET_DRY or self.order < 1:
            return None
        return max(self.subcell_depth, self.h_dry if self.wet_dry else -math.inf)

    @property
    def n_nodes(self) -> int:
        return (self.order + 1) ** 2

    @property
    def n_values(self) -> int:
        return self.mesh.n_elements * self.n_nodes

    def positions(self):
        return node_positions(self.mesh, self.order)

    def to_c(self) -> tuple[abi.Form, list]:
        """The C form and the objects that must outlive it."""
        keep: list = []

        def arr(a, dtype):
            a = np.ascontiguousarray(a, dtype=dtype)
            keep.append(a)
            return a

        def parent_series(bc) -> abi.ParentSeries:
            ps = abi.ParentSeries()
            pos = arr(np.asarray(bc.positions).reshape(-1, 2), np.float64)
            ps.n_slots = pos.shape[0]
            ps.positions = pos.ctypes.data_as(C.POINTER(C.c_double))
            tt = arr(bc.times, np.float64)
            ps.n_times = tt.size
            ps.times = tt.ctypes.data_as(C.POINTER(C.c_double))
            vals = arr(np.asarray(bc.values).reshape(-1), np.float32)
            if vals.size != pos.shape[0] * tt.size * 3:
                raise ValueError("values need [n_slots][n_times][3] entries")
            ps.values = vals.ctypes.data_as(C.POINTER(C.c_float))
            if bc.parent_depth is not None:
                ps.parent_depth = arr(bc.parent_depth, np.float64).ctypes.data_as(
                    C.POINTER(C.c_double))
            if bc.on_boundary is not None:
                ps.on_boundary = arr(np.asarray(bc.on_boundary, dtype=bool),
                                     np.uint8).ctypes.data_as(C.POINTER(C.c_uint8))
            if bc.slot_of_node is not None:
                sl = arr(np.asarray(bc.slot_of_node).reshape(-1), np.uint32)
                if sl.size != self.n_values:
                    raise ValueError("slot_of_node needs one slot per mesh node")
                ps.slot_of_node = sl.ctypes.data_as(C.POINTER(C.c_uint32))
            ps.cubic = 1 if bc.cubic else 0
            ps.velocity = 1 if bc.velocity else 0
            ps.reference_level = bc.reference_level
            ps.max_transport_ratio = bc.max_transport_ratio or 0.0
            ps.ramp_duration = bc.ramp_duration or 0.0
            keep.append(ps)
            return ps

        f = abi.Form()
        f.abi_version = abi.ABI_VERSION
        f.order = self.order
        v = arr(self.mesh.vertices, np.float64)
        f.n_vertices = v.shape[0]
        f.vertices = v.ctypes.data_as(C.POINTER(C.c_double))
        e = arr(self.mesh.elements, np.int64)
        f.n_elements = e.shape[0]
        f.elements = e.ctypes.data_as(C.POINTER(C.c_int64))
        p = arr(self.mesh.periodic.reshape(-1, 4), np.int64)
        f.n_periodic = p.shape[0]
        f.periodic = p.ctypes.data_as(C.POINTER(C.c_int64)) if p.size else None
        if self.mesh.face_tags is not None:
            t = arr(self.mesh.face_tags, np.int32)
            f.face_tags = t.ctypes.data_as(C.POINTER(C.c_int32))
        if self.bathymetry is not None:
            b = arr(self.bathymetry.reshape(-1), np.float64)
            if b.size != self.n_values:
                raise ValueError("bathymetry needs one value per node")
            f.bathymetry = b.ctypes.data_as(C.POINTER(C.c_double))
        f.g = self.g
        f.h_min = self.h_min
        f.formulation = self.formulation
        f.subcell_depth = self.subcell_depth
        f.subcell_h_dry = self.subcell_h_dry
        f.has_wet_dry = 1 if self.wet_dry else 0
        f.wet_dry_h_dry = self.h_dry
        f.wet_dry_relaxation_time = self.relaxation_time
        f.wet_dry_max_velocity = self.max_velocity
        f.positivity_h_dry = self.positivity_h_dry or 0.0
        if self.manning_n is None:
            f.friction = abi.FRICTION_NONE
        elif np.ndim(self.manning_n) == 0:
            f.friction = abi.FRICTION_MANNING
            f.manning_n = float(self.manning_n)
        else:
            f.friction = abi.FRICTION_MANNING_NODES
            n = arr(np.asarray(self.manning_n).reshape(-1), np.float64)
            if n.size != self.n_values:
                raise ValueError("per-node Manning needs one value per node")
            f.manning_n_nodes = n.ctypes.data_as(C.POINTER(C.c_double))
        f.friction_g = self.g if self.friction_g is None else self.friction_g
        f.manning_h_min = self.manning_h_min
        f.has_coriolis = 0 if self.coriolis_f0 is None else 1
        f.coriolis_f0 = self.coriolis_f0 or 0.0
        f.coriolis_beta = self.coriolis_beta
        f.coriolis_y0 = self.coriolis_y0
        bcs = (abi.Boundary * max(1, len(self.boundaries)))()
        for i, (tag, bc) in enumerate(sorted(self.boundaries.items())):
            bcs[i].tag = tag
            if isinstance(bc, WallBoundary):
                bcs[i].kind = abi.BC_WALL
                bcs[i].wall_h_min = bc.h_min
            elif isinstance(bc, ParentBoundary):
                bcs[i].kind = abi.BC_PARENT
                bcs[i].elevation_only = abi.INCOMING_WAVE if bc.incoming_wave else abi.AT_REST
                bcs[i].parent = C.pointer(parent_series(bc))
            elif isinstance(bc, NodeTidesBoundary):
                bcs[i].kind = abi.BC_NODE_TIDES
                bcs[i].elevation_only = abi.INCOMING_WAVE if bc.incoming_wave else abi.AT_REST
                nt = abi.NodeTides()
                nt.n_constituents = len(bc.omega)
                nt.omega = arr(bc.omega, np.float64).ctypes.data_as(C.POINTER(C.c_double))
                nt.f_rate = arr(bc.f_rate, np.float64).ctypes.data_as(C.POINTER(C.c_double))
                pos = arr(np.asarray(bc.positions).reshape(-1, 2), np.float64)
                nt.n_slots = pos.shape[0]
                nt.positions = pos.ctypes.data_as(C.POINTER(C.c_double))
                coef = arr(np.asarray(bc.coefficients).reshape(-1), np.float64)
                if coef.size != pos.shape[0] * len(bc.omega) * 6:
                    raise ValueError("coefficients need [n_slots][n_constituents][6] values")
                nt.coefficients = coef.ctypes.data_as(C.POINTER(C.c_double))
                if bc.mean is not None:
                    nt.mean = arr(bc.mean, np.float64).ctypes.data_as(C.POINTER(C.c_double))
                if bc.source_depth is not None:
                    nt.source_depth = arr(bc.source_depth, np.float64).ctypes.data_as(
                        C.POINTER(C.c_double))
                if bc.slot_of_node is not None:
                    sl = arr(np.asarray(bc.slot_of_node).reshape(-1), np.uint32)
                    if sl.size != self.n_values:
                        raise ValueError("slot_of_node needs one slot per mesh node")
                    nt.slot_of_node = sl.ctypes.data_as(C.POINTER(C.c_uint32))
                nt.velocity = 1 if bc.velocity else 0
                nt.use_mean = 1 if bc.use_mean else 0
                nt.max_transport_ratio = bc.max_transport_ratio or 0.0
                nt.ramp_duration = bc.ramp_duration or 0.0
                keep.append(nt)
                bcs[i].node_tides = C.pointer(nt)
            else:
                bcs[i].kind = abi.BC_CHARACTERISTIC
                bcs[i].elevation_only = abi.INCOMING_WAVE if bc.incoming_wave else abi.AT_REST
                cons = (abi.TideConstituent * max(1, len(bc.constituents)))(*bc.constituents)
                keep.append(cons)
                bcs[i].n_constituents = len(bc.constituents)
                bcs[i].constituents = cons
                bcs[i].mean_elevation = bc.mean_elevation
                bcs[i].ramp_duration = bc.ramp_duration or 0.0
            factor = getattr(bc, "raise_factor", None)
            if factor is not None:
                bcs[i].raise_ = 1
                bcs[i].raise_factor = float(factor)
        keep.append(bcs)
        f.n_boundaries = len(self.boundaries)
        f.boundaries = bcs
        f.numerics = self.numerics
        depth = self.local_depth()
        f.has_line_local = 0 if depth is None else 1
        f.line_local_depth = 0.0 if depth is None else float(depth)
        if self.relaxation is not None:
            r = abi.Relaxation()
            r.parent = C.pointer(parent_series(self.relaxation.parent))
            w = arr(self.relaxation.weight, np.float64)
            r.weight = w.ctypes.data_as(C.POINTER(C.c_double))
            r.rate = self.relaxation.rate
            r.wet_depth = self.relaxation.wet_depth
            r.momentum_only = 1 if self.relaxation.momentum_only else 0
            keep.append(r)
            f.relaxation = C.pointer(r)
        if self.atmosphere is not None:
            at = self.atmosphere
            a = abi.Atmosphere()
            tt = arr(at.times, np.float64)
            vals = arr(np.asarray(at.values).reshape(-1), np.float32)
            if vals.size != tt.size * self.n_values * 5:
                raise ValueError("the atmosphere needs [n_times][n_values][5] values")
            a.n_times = tt.size
            a.times = tt.ctypes.data_as(C.POINTER(C.c_double))
            a.epoch_unix = float(at.epoch_unix)
            a.values = vals.ctypes.data_as(C.POINTER(C.c_float))
            a.source = 1 if at.source else 0
            a.wind = 1 if at.wind else 0
            a.pressure = 1 if at.pressure else 0
            a.level = 1 if (at.pressure and at.has_pressure) else 0
            a.drag = int(at.drag)
            a.drag_cd = float(at.drag_cd)
            a.rho_air = float(at.rho_air)
            a.rho_water = float(at.rho_water)
            a.h_min = float(at.h_min)
            a.ramp_duration = at.ramp_duration or 0.0
            keep.append(a)
            f.atmosphere = C.pointer(a)
        return f, keep


def at_rest(form: SWEDeviceForm2D, eta: float = 0.0):
    """Still water at level ``eta``: h = max(0, η − B), no momentum
    (src/case/run.rs:1157-1170)."""
    b = np.zeros(form.n_values) if form.bathymetry is None else form.bathymetry.reshape(-1)
    h = np.maximum(eta - b, 0.0)
    return h, np.zeros_like(h), np.zeros_like(h)
