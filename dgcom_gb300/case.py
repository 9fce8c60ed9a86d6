"""Case files: the reference's TOML case schema (src/case/schema.rs) for what
the device path runs, turned into a form, a state and a run on the GPU.

A case file names the mesh (a rectangle, or a Gmsh file through
``dgcom_gb300.gmsh``), the bed, the physics, the open boundaries, the time
stepping and the stations; ``run_case`` steps it on a GB300 through the
C ABI (``Cuda.run_2d``) and writes the stations' records as the reference's
run does (``stations.csv``: station, time_s, eta_m, u_m_s, v_m_s, depth_m).

Read strictly, like the reference's ``deny_unknown_fields``: an unknown key
is an error. Keys and sections the reference has but the device path does
not run are refused by name, saying why: a placed mesh (``geographic``,
``origin``, stations by ``lon``/``lat``, ``beta_plane``) and a raster bed,
tidal atlases and parent models read from files, the weather, 3D, waves,
farms, rivers, restarts, viscosity, drag-coefficient friction, and gauge
scoring. The sections it takes mean what they mean in the reference, with
its defaults: ``[run]`` (``start`` gives Greenwich phase lags and nodal
corrections), ``[mesh]`` (``order`` 1–4, ``rectangle`` or ``gmsh``,
``drop_land``), ``[bathymetry]`` (``depth_m`` or ``ramp``), ``[physics]``,
``[initial]``, ``[[boundary]]`` (``still`` or ``tide``, ``velocity``),
``[numerics]`` (``integrator``, ``cfl``, ``dt_max_s``,
``local_time_stepping_levels``), ``[compute]`` and ``[output]``
(``interval_minutes``, ``station_interval_minutes``, stations)."""

from __future__ import annotations

import csv
import math
import tomllib
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import abi, gmsh, tides
from .astronomy import ModelClock, canonical_name
from .cases import coriolis_parameter, ramp_depth
from .mesh import (TAG_OPEN, TAG_RIVER, TAG_TIDAL, TAG_WALL, QuadMesh, gll_nodes,
                   node_positions, uniform_rectangle)
from .physics import SWEDeviceForm2D, TidalBoundary, WallBoundary

SIDE_TAGS = {"wall": TAG_WALL, "open": TAG_OPEN, "tidal": TAG_TIDAL, "river": TAG_RIVER}
ORDERS = range(1, 5)
LINEAR_CFL_SAFETY = 0.9
# linear_cfl_swe_2d (src/solver/rhs/swe_2d.rs:1263-1300): orders 1–4
LINEAR_CFL = {abi.SSP_RK3: (1.6, 1.04, 0.73, 0.56), abi.SSP_RK43: (2.2, 1.51, 1.15, 0.93)}
MAX_LEVELS = abi.MAX_LEVELS

_NOT_ON_DEVICE = {
    "atmosphere": "a weather model's wind and pressure",
    "three_d": "3D runs",
    "waves": "spectral waves",
    "farm": "net cages",
    "rivers": "rivers",
    "restart": "restart files",
}


class CaseError(ValueError):
    """A case file that is malformed, invalid, or asks for what the device
    path does not run."""


def _refuse(what: str, why: str):
    raise CaseError(f"{what}: {why} is not on the device path of this library")


def _keys(section: dict, name: str, allowed: set[str], refused: dict[str, str] | None = None):
    for key in section:
        if refused and key in refused:
            _refuse(f"{name}.{key}", refused[key])
        if key not in allowed:
            raise CaseError(f"unknown key {name}.{key}")


def _number(v, what: str, positive=False, nonneg=False) -> float:
    if isinstance(v, bool) or not isinstance(v, (int, float)):
        raise CaseError(f"{what} must be a number, not {v!r}")
    v = float(v)
    if not math.isfinite(v) or (positive and v <= 0.0) or (nonneg and v < 0.0):
        raise CaseError(f"{what} must be {'positive' if positive else 'non-negative' if nonneg else 'finite'}, not {v}")
    return v


def _int(v, what: str, lo: int | None = None) -> int:
    if isinstance(v, bool) or not isinstance(v, int) or (lo is not None and v < lo):
        raise CaseError(f"{what} must be an integer{f' of at least {lo}' if lo is not None else ''}, not {v!r}")
    return v


def _pair(v, what: str) -> tuple[float, float]:
    if not isinstance(v, list) or len(v) != 2:
        raise CaseError(f"{what} must be a pair [a, b], not {v!r}")
    return _number(v[0], what), _number(v[1], what)


@dataclass
class Station:
    name: str
    x: float
    y: float
    open_water_depth: float = 3.0
    max_offset: float = 3000.0


@dataclass
class Case:
    """A validated case file: every value resolved to its default."""
    path: Path
    name: str
    duration_s: float
    start: str | None
    order: int
    rectangle: dict | None
    gmsh_path: Path | None
    drop_land: bool
    depth: float | None
    ramp: dict | None
    gravity: float
    coriolis_f: float | None
    manning: float | None
    wetting_drying: bool
    eta0: float
    boundaries: dict  # face tag → TidalBoundary
    scheme: int
    cfl: float
    dt_max: float | None
    levels: int
    ordinal: int
    output_dir: Path
    interval_s: float
    station_interval_s: float
    stations: list = field(default_factory=list)


def load_case(path) -> Case:
    """Read and validate a case file (relative paths are the file's)."""
    path = Path(path)
    try:
        doc = tomllib.loads(path.read_text())
    except tomllib.TOMLDecodeError as e:
        raise CaseError(f"{path}: {e}") from None
    return parse_case(doc, path)


def parse_case(doc: dict, path: Path) -> Case:
    top = {"run", "mesh", "bathymetry", "physics", "initial", "boundary", "numerics", "compute",
           "output"}
    _keys(doc, "case", top, _NOT_ON_DEVICE)
    for required in ("run", "mesh", "bathymetry"):
        if required not in doc:
            raise CaseError(f"missing section [{required}]")
    base = path.parent

    run = doc["run"]
    _keys(run, "run", {"name", "start", "duration_hours"})
    if "duration_hours" not in run:
        raise CaseError("run.duration_hours is required")
    name = str(run.get("name", "case"))
    duration = _number(run["duration_hours"], "run.duration_hours", positive=True) * 3600.0
    start = run.get("start")
    clock = ModelClock(start) if start is not None else None

    mesh = doc["mesh"]
    _keys(mesh, "mesh", {"order", "rectangle", "gmsh", "drop_land"},
          {"geographic": "a mesh placed on the Earth", "origin": "a mesh placed on the Earth"})
    order = _int(mesh.get("order", 2), "mesh.order")
    if order not in ORDERS:
        raise CaseError(f"mesh.order must be {ORDERS.start}–{ORDERS.stop - 1} on the device, not {order}")
    rect, gpath = mesh.get("rectangle"), mesh.get("gmsh")
    if (rect is None) == (gpath is None):
        raise CaseError("[mesh] needs exactly one of `rectangle` and `gmsh`")
    if rect is not None:
        _keys(rect, "mesh.rectangle", {"x_m", "y_m", "nx", "ny", "south", "east", "north", "west"})
        for k in ("x_m", "y_m", "nx", "ny"):
            if k not in rect:
                raise CaseError(f"mesh.rectangle.{k} is required")
        x0, x1 = _pair(rect["x_m"], "mesh.rectangle.x_m")
        y0, y1 = _pair(rect["y_m"], "mesh.rectangle.y_m")
        if not (x1 > x0 and y1 > y0):
            raise CaseError("mesh.rectangle needs x_m[0] < x_m[1] and y_m[0] < y_m[1]")
        sides = []
        for side in ("south", "east", "north", "west"):
            tag = rect.get(side, "wall")
            if tag not in SIDE_TAGS:
                raise CaseError(f"mesh.rectangle.{side} must be one of {sorted(SIDE_TAGS)}, not {tag!r}")
            sides.append(SIDE_TAGS[tag])
        rect = {"x": (x0, x1), "y": (y0, y1), "nx": _int(rect["nx"], "mesh.rectangle.nx", 1),
                "ny": _int(rect["ny"], "mesh.rectangle.ny", 1), "sides": tuple(sides)}
    else:
        gpath = (base / str(gpath)).resolve()
    drop_land = bool(mesh.get("drop_land", True))

    bath = doc["bathymetry"]
    _keys(bath, "bathymetry", {"depth_m", "ramp", "rx0_min_depth_m", "wall_low_water_m"},
          {"raster": "a raster bed", "smooth_rx0": "bed smoothing",
           "lower_wall_land": "lowering wall land", "slopes_3d": "the 3D bed"})
    depth, ramp = bath.get("depth_m"), bath.get("ramp")
    if (depth is None) == (ramp is None):
        raise CaseError("[bathymetry] needs exactly one of `depth_m` and `ramp`")
    if depth is not None:
        depth = _number(depth, "bathymetry.depth_m")
    else:
        _keys(ramp, "bathymetry.ramp", {"from_m", "to_m", "depth_m"})
        ramp = {k: _pair(ramp.get(k), f"bathymetry.ramp.{k}") for k in ("from_m", "to_m", "depth_m")}
        if ramp["from_m"] == ramp["to_m"]:
            raise CaseError("bathymetry.ramp needs from_m ≠ to_m")

    phys = doc.get("physics", {})
    _keys(phys, "physics", {"gravity", "coriolis", "friction", "viscosity_m2_s", "smagorinsky",
                            "wetting_drying"})
    gravity = _number(phys.get("gravity", 9.81), "physics.gravity", positive=True)
    for k in ("viscosity_m2_s", "smagorinsky"):
        if _number(phys.get(k, 0.0), f"physics.{k}", nonneg=True) > 0.0:
            _refuse(f"physics.{k}", "horizontal viscosity")
    coriolis_f = None
    cor = phys.get("coriolis")
    if cor == "beta_plane":
        _refuse("physics.coriolis", "the beta plane (a mesh placed on the Earth)")
    elif isinstance(cor, dict) and len(cor) == 1 and "f_plane" in cor:
        coriolis_f = _number(cor["f_plane"], "physics.coriolis.f_plane")
    elif isinstance(cor, dict) and len(cor) == 1 and "latitude" in cor:
        coriolis_f = coriolis_parameter(_number(cor["latitude"], "physics.coriolis.latitude"))
    elif cor is not None:
        raise CaseError(f"physics.coriolis must be {{ f_plane = f }}, {{ latitude = φ }} or \"beta_plane\", not {cor!r}")
    manning = None
    fr = phys.get("friction")
    if isinstance(fr, dict) and len(fr) == 1 and "manning" in fr:
        manning = _number(fr["manning"], "physics.friction.manning", nonneg=True)
    elif isinstance(fr, dict) and len(fr) == 1 and "drag_coefficient" in fr:
        _refuse("physics.friction.drag_coefficient", "quadratic drag with a constant coefficient")
    elif fr is not None:
        raise CaseError(f"physics.friction must be {{ manning = n }} or {{ drag_coefficient = c }}, not {fr!r}")
    wetting_drying = bool(phys.get("wetting_drying", True))

    init = doc.get("initial", {})
    _keys(init, "initial", {"eta_m"})
    eta0 = _number(init.get("eta_m", 0.0), "initial.eta_m")

    boundaries = {}
    for i, b in enumerate(doc.get("boundary", [])):
        where = f"boundary[{i}]"
        _keys(b, where, {"tag", "still", "tide", "velocity", "inverse_barometer"},
              {"atlas": "a tidal atlas read from a file",
               "nesting": "a parent ocean model read from files"})
        tag = b.get("tag")
        if tag not in ("open", "tidal", "river"):
            raise CaseError(f"{where}.tag must be \"open\", \"tidal\" or \"river\", not {tag!r}")
        if SIDE_TAGS[tag] in boundaries:
            raise CaseError(f"two [[boundary]] entries for tag {tag!r}")
        velocity = b.get("velocity", "at_rest")
        if velocity not in ("at_rest", "incoming_wave"):
            raise CaseError(f"{where}.velocity must be \"at_rest\" or \"incoming_wave\"")
        if b.get("inverse_barometer") is not None:
            _number(b["inverse_barometer"], f"{where}.inverse_barometer")  # no weather here
        still, tide = b.get("still"), b.get("tide")
        if (still is None) == (tide is None):
            raise CaseError(f"{where} needs exactly one of `still` and `tide`")
        if still is not None:
            _keys(still, f"{where}.still", {"eta_m"})
            bc = TidalBoundary([], _number(still.get("eta_m", 0.0), f"{where}.still.eta_m"), None,
                               velocity == "incoming_wave")
        else:
            _keys(tide, f"{where}.tide", {"constituents", "mean_m", "ramp_hours"})
            cons = []
            for j, c in enumerate(tide.get("constituents", [])):
                _keys(c, f"{where}.tide.constituents[{j}]", {"name", "amplitude_m", "phase_deg"})
                cname = canonical_name(str(c.get("name", "")))
                if cname is None:
                    raise CaseError(f"{where}.tide: unknown constituent {c.get('name')!r}")
                amp = _number(c.get("amplitude_m"), f"{where}.tide {cname} amplitude_m", nonneg=True)
                cons.append(tides.constituent(cname, amp,
                                              _number(c.get("phase_deg", 0.0), f"{cname} phase_deg"),
                                              clock))
            if not cons:
                raise CaseError(f"{where}.tide needs at least one constituent")
            if len(cons) > abi.MAX_CONSTITUENTS:
                raise CaseError(f"{where}.tide: at most {abi.MAX_CONSTITUENTS} constituents")
            ramp_h = _number(tide.get("ramp_hours", 1.0), f"{where}.tide.ramp_hours", nonneg=True)
            bc = TidalBoundary(cons, _number(tide.get("mean_m", 0.0), f"{where}.tide.mean_m"),
                               3600.0 * ramp_h, velocity == "incoming_wave")
        boundaries[SIDE_TAGS[tag]] = bc

    num = doc.get("numerics", {})
    _keys(num, "numerics", {"integrator", "cfl", "dt_max_s", "local_time_stepping_levels"})
    integrator = num.get("integrator", "ssp_rk43")
    if integrator not in ("ssp_rk43", "ssp_rk3"):
        raise CaseError(f"numerics.integrator must be \"ssp_rk43\" or \"ssp_rk3\", not {integrator!r}")
    scheme = abi.SSP_RK43 if integrator == "ssp_rk43" else abi.SSP_RK3
    cfl = (_number(num["cfl"], "numerics.cfl", positive=True) if "cfl" in num
           else LINEAR_CFL_SAFETY * LINEAR_CFL[scheme][order - 1])
    dt_max = (_number(num["dt_max_s"], "numerics.dt_max_s", positive=True)
              if "dt_max_s" in num else None)
    levels = _int(num.get("local_time_stepping_levels", 0), "numerics.local_time_stepping_levels", 0)
    if levels > MAX_LEVELS:
        raise CaseError(f"numerics.local_time_stepping_levels: at most {MAX_LEVELS} on the device")

    comp = doc.get("compute", {})
    _keys(comp, "compute", {"device"})
    dev = comp.get("device", "cpu")
    if dev in ("cpu", "cuda"):
        ordinal = 0  # this library steps every case on a GPU
    elif isinstance(dev, str) and dev.startswith("cuda:") and dev[5:].isdigit():
        ordinal = int(dev[5:])
    else:
        raise CaseError(f"compute.device must be \"cpu\", \"cuda\" or \"cuda:N\", not {dev!r}")

    out = doc.get("output", {})
    _keys(out, "output", {"directory", "interval_minutes", "station_interval_minutes",
                          "spinup_hours", "snapshot", "vtk", "netcdf", "station"})
    for k in ("vtk", "netcdf"):
        if out.get(k):
            _refuse(f"output.{k}", f"{k} output")
    interval = 60.0 * _number(out.get("interval_minutes", 60.0), "output.interval_minutes",
                              positive=True)
    st_interval = 60.0 * _number(out.get("station_interval_minutes", interval / 60.0),
                                 "output.station_interval_minutes", positive=True)
    big, small = max(interval, st_interval), min(interval, st_interval)
    if abs(big / small - round(big / small)) > 1e-9:
        raise CaseError("one of output.interval_minutes and station_interval_minutes must be a "
                        "whole multiple of the other")
    stations = []
    for j, s in enumerate(out.get("station", [])):
        where = f"output.station[{j}]"
        _keys(s, where, {"name", "x_m", "y_m", "open_water_depth_m", "max_offset_m"},
              {"lon": "a station placed on the Earth", "lat": "a station placed on the Earth",
               "gauge": "scoring against a tide gauge"})
        if "name" not in s or "x_m" not in s or "y_m" not in s:
            raise CaseError(f"{where} needs name, x_m and y_m")
        stations.append(Station(str(s["name"]), _number(s["x_m"], f"{where}.x_m"),
                                _number(s["y_m"], f"{where}.y_m"),
                                _number(s.get("open_water_depth_m", 3.0),
                                        f"{where}.open_water_depth_m", nonneg=True),
                                _number(s.get("max_offset_m", 3000.0), f"{where}.max_offset_m",
                                        nonneg=True)))
    out_dir = base / str(out.get("directory", f"output/{name}"))
    return Case(path, name, duration, start, order, rect, gpath, drop_land, depth, ramp, gravity,
                coriolis_f, manning, wetting_drying, eta0, boundaries, scheme, cfl, dt_max, levels,
                ordinal, out_dir, interval, st_interval, stations)


# ---------------------------------------------------------------------------
# The domain
# ---------------------------------------------------------------------------

def retain_elements(mesh: QuadMesh, keep: np.ndarray) -> QuadMesh:
    """The kept elements, in order, their vertices renumbered by first use;
    faces to dropped elements become walls (Mesh2D::retain_elements)."""
    K = mesh.n_elements
    a = mesh.elements.reshape(-1)
    b = mesh.elements[:, [1, 2, 3, 0]].reshape(-1)
    key = np.minimum(a, b) * mesh.vertices.shape[0] + np.maximum(a, b)
    kept_face = np.repeat(keep, 4)
    _, inv = np.unique(key, return_inverse=True)
    kept_count = np.bincount(inv, weights=kept_face.astype(float))
    all_count = np.bincount(inv)
    tags = (mesh.face_tags.reshape(-1).copy() if mesh.face_tags is not None
            else np.zeros(4 * K, np.int32))
    lost = (all_count[inv] == 2) & (kept_count[inv] == 1)  # its neighbour was dropped
    tags[lost] = TAG_WALL
    idx = np.nonzero(keep)[0]
    new_of_old = np.full(K, -1, np.int64)
    new_of_old[idx] = np.arange(idx.size)
    periodic = mesh.periodic
    if periodic.size:
        both = keep[periodic[:, 0]] & keep[periodic[:, 2]]
        for k0, f0, k1, f1 in periodic[~both]:
            if keep[k0]:
                tags[4 * k0 + f0] = TAG_WALL
            if keep[k1]:
                tags[4 * k1 + f1] = TAG_WALL
        periodic = periodic[both].copy()
        periodic[:, 0] = new_of_old[periodic[:, 0]]
        periodic[:, 2] = new_of_old[periodic[:, 2]]
    elements = mesh.elements[idx]
    used, first = np.unique(elements.reshape(-1), return_index=True)
    by_use = used[np.argsort(first, kind="stable")]
    new_vertex = np.full(mesh.vertices.shape[0], -1, np.int64)
    new_vertex[by_use] = np.arange(by_use.size)
    return QuadMesh(mesh.vertices[by_use], new_vertex[elements], periodic,
                    tags.reshape(K, 4)[idx].astype(np.int32))


def _bed(case: Case, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    if case.depth is not None:
        return np.full_like(x, -case.depth)
    r = case.ramp
    return -ramp_depth(x, y, r["from_m"], r["to_m"], r["depth_m"])


def build_form(case: Case) -> tuple[SWEDeviceForm2D, tuple]:
    """The device form and the initial state (still water at initial.eta_m)."""
    if case.rectangle is not None:
        r = case.rectangle
        mesh = uniform_rectangle(*r["x"], *r["y"], r["nx"], r["ny"], sides=r["sides"])
    else:
        mesh = gmsh.read_gmsh_mesh(case.gmsh_path)
    x, y = node_positions(mesh, case.order)
    bed = _bed(case, x, y)
    if case.drop_land:
        keep = (bed < 0.0).any(axis=1)
        if not keep.any():
            raise CaseError("no element has a node below mean sea level: the domain is all land")
        mesh = retain_elements(mesh, keep)
        bed = bed[keep]
    form = SWEDeviceForm2D(mesh=mesh, order=case.order, g=case.gravity)
    form.bathymetry = bed
    if case.manning is not None:
        form.manning_n = case.manning
    if case.coriolis_f is not None:
        form.coriolis_f0 = case.coriolis_f
    if not case.wetting_drying:
        form.wet_dry = False
        form.positivity_h_dry = None
    tags = set(np.unique(mesh.face_tags).tolist()) if mesh.face_tags is not None else {TAG_WALL}
    boundaries = {TAG_WALL: WallBoundary()}
    for tag in sorted(tags):
        if tag in case.boundaries:
            boundaries[tag] = case.boundaries[tag]
        elif tag in (TAG_OPEN, TAG_TIDAL, TAG_RIVER) and _tag_on_boundary(mesh, tag):
            name = [k for k, v in SIDE_TAGS.items() if v == tag][0]
            raise CaseError(f"the mesh has {name!r} faces and no [[boundary]] for them")
        else:
            boundaries[tag] = WallBoundary()  # custom groups and walls
    form.boundaries = boundaries
    h = np.maximum(case.eta0 - bed, 0.0).reshape(-1)
    return form, (h, np.zeros_like(h), np.zeros_like(h))


def _tag_on_boundary(mesh: QuadMesh, tag: int) -> bool:
    rows = gmsh.boundary_edges(mesh)
    return bool((rows[:, 4] == tag).any())


# ---------------------------------------------------------------------------
# Stations
# ---------------------------------------------------------------------------

def _inverse_bilinear(c: np.ndarray, x: float, y: float) -> tuple[float, float]:
    """(r, s) of (x, y) in the bilinear map of corners c (4, 2), by Newton."""
    r = s = 0.0
    for _ in range(50):
        n = np.array([(1 - r) * (1 - s), (1 + r) * (1 - s), (1 + r) * (1 + s), (1 - r) * (1 + s)]) / 4
        dr = np.array([-(1 - s), (1 - s), (1 + s), -(1 + s)]) / 4
        ds = np.array([-(1 - r), -(1 + r), (1 + r), (1 - r)]) / 4
        px, py = n @ c[:, 0] - x, n @ c[:, 1] - y
        j = np.array([[dr @ c[:, 0], ds @ c[:, 0]], [dr @ c[:, 1], ds @ c[:, 1]]])
        step = np.linalg.solve(j, [px, py])
        r, s = r - step[0], s - step[1]
        if abs(step[0]) + abs(step[1]) < 1e-14:
            break
    return r, s


def _segment_point(p, a, b):
    d = b - a
    t = float(np.clip(np.dot(p - a, d) / max(np.dot(d, d), 1e-300), 0.0, 1.0))
    return a + t * d


class Probe:
    """A point of one element and its GLL interpolation weights."""

    def __init__(self, mesh: QuadMesh, order: int, element: int, x: float, y: float):
        self.element = element
        self.x, self.y = x, y
        r, s = _inverse_bilinear(mesh.corners()[element], x, y)
        g = gll_nodes(order)

        def lagrange(t):
            out = np.ones(order + 1)
            for i in range(order + 1):
                for m in range(order + 1):
                    if m != i:
                        out[i] *= (t - g[m]) / (g[i] - g[m])
            return out

        self.weights = np.outer(lagrange(s), lagrange(r)).reshape(-1)  # node j·n1 + a

    def value(self, field: np.ndarray) -> float:
        return float(self.weights @ field[self.element])


def locate(mesh: QuadMesh, x: float, y: float) -> int | None:
    """The element containing (x, y), or None."""
    c = mesh.corners()
    inside = np.ones(mesh.n_elements, bool)
    for i in range(4):
        a, b = c[:, i], c[:, (i + 1) % 4]
        cross = (b[:, 0] - a[:, 0]) * (y - a[:, 1]) - (b[:, 1] - a[:, 1]) * (x - a[:, 0])
        scale = np.hypot(b[:, 0] - a[:, 0], b[:, 1] - a[:, 1])
        inside &= cross >= -1e-9 * scale * scale
    hits = np.nonzero(inside)[0]
    return int(hits[0]) if hits.size else None


def station_probe(mesh: QuadMesh, order: int, bed: np.ndarray, st: Station) -> Probe:
    """Probe2D::in_open_water: at the station if its element is at least
    open_water_depth deep at every node, else at the nearest point of such
    an element within max_offset; 0 samples where it is. The current is
    sampled at the same point."""
    k = locate(mesh, st.x, st.y)
    if st.open_water_depth <= 0.0 or (k is not None and
                                      (-bed[k] >= st.open_water_depth).all()):
        if k is None:
            raise CaseError(f"station {st.name!r} at ({st.x:.1f}, {st.y:.1f}) m is outside the mesh")
        return Probe(mesh, order, k, st.x, st.y)
    deep = np.nonzero((-bed >= st.open_water_depth).all(axis=1))[0]
    c = mesh.corners()
    p = np.array([st.x, st.y])
    best = (np.inf, None, None)
    for e in deep:
        for i in range(4):
            q = _segment_point(p, c[e, i], c[e, (i + 1) % 4])
            d = float(np.hypot(*(q - p)))
            if d < best[0]:
                best = (d, e, q)
    if best[1] is None or best[0] > st.max_offset:
        raise CaseError(f"station {st.name!r} at ({st.x:.1f}, {st.y:.1f}) m has no element at least "
                        f"{st.open_water_depth} m deep within {st.max_offset} m")
    return Probe(mesh, order, int(best[1]), float(best[2][0]), float(best[2][1]))


# ---------------------------------------------------------------------------
# Running a case
# ---------------------------------------------------------------------------

@dataclass
class CaseRun:
    case: Case
    report: object
    records: list       # (station, time_s, eta_m, u_m_s, v_m_s, depth_m)
    state: tuple


def run_case(path, ordinal: int | None = None, max_steps: int | None = None,
             write: bool = True) -> CaseRun:
    """Run a case file on the GPU: the stations sampled every station
    interval from the start, and ``stations.csv`` in the output directory."""
    from .device import Cuda, DeviceRun

    case = load_case(path)
    form, q = build_form(case)
    n1 = case.order + 1
    bed = form.bathymetry.reshape(form.mesh.n_elements, n1 * n1)
    probes = [station_probe(form.mesh, case.order, bed, s) for s in case.stations]
    records = []

    def sample(fields, t):
        h, hu, hv = fields
        K = form.mesh.n_elements
        hh, uu, vv = (a.reshape(K, n1 * n1) for a in (h, hu, hv))
        for st, pr in zip(case.stations, probes):
            depth = pr.value(hh)
            eta = depth + pr.value(bed)
            u = pr.value(uu) / depth if depth > 1e-6 else 0.0
            v = pr.value(vv) / depth if depth > 1e-6 else 0.0
            records.append((st.name, t, eta, u, v, depth))

    state = [np.array(a) for a in q]
    run = DeviceRun(span=(0.0, case.duration_s), cfl=case.cfl, interval=case.station_interval_s,
                    dt_max=case.dt_max, max_steps=max_steps, scheme=case.scheme,
                    levels=case.levels)
    report = Cuda().run_2d(case.ordinal if ordinal is None else ordinal, form, state, run, sample)
    if write:
        case.output_dir.mkdir(parents=True, exist_ok=True)
        with open(case.output_dir / "stations.csv", "w", newline="") as f:
            w = csv.writer(f)
            w.writerow(["station", "time_s", "eta_m", "u_m_s", "v_m_s", "depth_m"])
            for row in records:
                w.writerow([row[0]] + [repr(float(v)) for v in row[1:]])
    return CaseRun(case, report, records, tuple(state))
