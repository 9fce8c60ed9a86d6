"""The workloads of the device path, built on the host with fixed seeds:

- :func:`tidal_channel`: the idealised tidal channel (50 km × 5 km,
  200 × 20 quads, N = 2) whose bed ramps from 20 m deep at the open western
  end to 1 m above datum at the head, so a tidal flat floods and drains,
  under an M2 tide of 1 m, Manning n = 0.025 and f = 1.26e-4 s⁻¹;
- :func:`coastal_box`: a synthetic coastal quad mesh of ≈ 1.0 M elements
  (200 km × 150 km, element sizes 100–250 m, jittered, in Hilbert order),
  N = 3, over a seeded Gaussian random bed of 2–300 m with 30 Gaussian
  islands above the datum, under a 4-constituent tide (M2, S2, N2, K1) with
  seeded phases, Manning n = 0.02 and Coriolis at 63° N;
- :func:`adjoint_channel` and :func:`adjoint_ensemble_members`: the
  station-misfit adjoint workloads (one channel; a batched ensemble of
  coastal boxes under eight constituents);
- :func:`split_form_setup`: the meshes, beds and states of the reference's
  split-form unit tests (src/solver/rhs/swe_2d_split_form.rs:1144-1232).

No public dataset is involved: every input is generated here."""

from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass

import numpy as np

from . import abi, tides
from .mesh import (TAG_OPEN, TAG_WALL, QuadMesh, graded_jittered_box, in_hilbert_order,
                   node_positions, uniform_periodic, uniform_rectangle, move_vertices)
from .physics import SWEDeviceForm2D, TidalBoundary, WallBoundary, at_rest

EARTH_ROTATION_RATE = 7.292_115e-5  # rad/s (src/source/swe_2d/coriolis.rs:24-25)


def coriolis_parameter(latitude_deg: float) -> float:
    """f = 2Ω sin φ (src/source/swe_2d/coriolis.rs:28-31)."""
    return 2.0 * EARTH_ROTATION_RATE * math.sin(math.radians(latitude_deg))


def ramp_depth(x, y, from_m, to_m, depth_m):
    """[bathymetry.ramp]: depth linear along from → to, constant across
    (src/case/schema.rs:658-663)."""
    x0, y0 = from_m
    dx, dy = to_m[0] - x0, to_m[1] - y0
    s = np.clip(((x - x0) * dx + (y - y0) * dy) / (dx * dx + dy * dy), 0.0, 1.0)
    return depth_m[0] + s * (depth_m[1] - depth_m[0])


@dataclass
class Case:
    form: SWEDeviceForm2D
    state: tuple  # (h, hu, hv)
    cfl: float
    scheme: int
    t_end: float
    stations: np.ndarray | None = None  # (n, 2) positions


def tidal_channel(nx: int = 200, ny: int = 20, order: int = 2,
                  numerics: int = abi.NUMERICS_FAST) -> Case:
    lx, ly = 50_000.0, 5_000.0
    mesh = uniform_rectangle(0.0, lx, 0.0, ly, nx, ny,
                             sides=(TAG_WALL, TAG_WALL, TAG_WALL, TAG_OPEN))
    form = SWEDeviceForm2D(mesh=mesh, order=order, numerics=numerics)
    x, y = node_positions(mesh, order)
    depth = ramp_depth(x, y, (0.0, 0.5 * ly), (lx, 0.5 * ly), (20.0, -1.0))
    form.bathymetry = -depth
    form.manning_n = 0.025
    form.coriolis_f0 = 1.26e-4
    form.boundaries = {
        TAG_WALL: WallBoundary(),
        TAG_OPEN: TidalBoundary([tides.constituent("M2", 1.0, 0.0)], ramp_duration=3600.0),
    }
    stations = np.stack([np.arange(0.0, lx + 1.0, 5_000.0), np.full(11, 0.5 * ly)], axis=1)
    return Case(form, at_rest(form), 0.5, abi.SSP_RK3, 25.0 * 3600.0, stations)


def gaussian_random_field(nx: int, ny: int, spacing: float, corr: float,
                          rng: np.random.Generator) -> np.ndarray:
    """Unit-variance Gaussian random field on an (ny, nx) grid of the given
    spacing with a Gaussian correlation of length ``corr``, by spectral
    synthesis (white noise filtered in Fourier space)."""
    noise = rng.standard_normal((ny, nx))
    kx = np.fft.fftfreq(nx, d=spacing) * 2.0 * np.pi
    ky = np.fft.fftfreq(ny, d=spacing) * 2.0 * np.pi
    k2 = kx[None, :] ** 2 + ky[:, None] ** 2
    field = np.real(np.fft.ifft2(np.fft.fft2(noise) * np.exp(-0.25 * k2 * corr * corr)))
    field -= field.mean()
    return field / field.std()


def _bilinear_grid(field: np.ndarray, spacing: float, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    ny, nx = field.shape
    fx = np.clip(x / spacing, 0.0, nx - 1.000001)
    fy = np.clip(y / spacing, 0.0, ny - 1.000001)
    i = fx.astype(np.int64)
    j = fy.astype(np.int64)
    tx, ty = fx - i, fy - j
    return ((1 - tx) * (1 - ty) * field[j, i] + tx * (1 - ty) * field[j, i + 1]
            + (1 - tx) * ty * field[j + 1, i] + tx * ty * field[j + 1, i + 1])


def coastal_bed(x: np.ndarray, y: np.ndarray, lx: float, ly: float, seed: int,
                n_islands: int = 30, island_radius: tuple[float, float] = (1000.0, 5000.0)
                ) -> np.ndarray:
    """Bed elevation B at (x, y): a seeded Gaussian random field (5 km
    correlation, on a 1 km grid, bilinear to the points) mapped to depths of
    2–300 m, with ``n_islands`` Gaussian islands (radius 1–5 km) whose crests
    reach 2–20 m above the datum, away from the open western side."""
    from scipy.special import ndtr

    rng = np.random.default_rng(seed)
    spacing = 1000.0
    gx, gy = int(lx / spacing) + 2, int(ly / spacing) + 2
    z = gaussian_random_field(gx, gy, spacing, 5000.0, rng)
    depth_grid = 2.0 + 298.0 * ndtr(z)
    depth = _bilinear_grid(depth_grid, spacing, x, y)
    bed = -depth
    cx = rng.uniform(0.15 * lx, 0.95 * lx, n_islands)
    cy = rng.uniform(0.05 * ly, 0.95 * ly, n_islands)
    radius = rng.uniform(island_radius[0], island_radius[1], n_islands)
    crest = rng.uniform(2.0, 20.0, n_islands)
    centre_depth = _bilinear_grid(depth_grid, spacing, cx, cy)
    # an island adds nothing representable beyond 6.5 radii (e^-42.25 · 320 m
    # < 1e-16 m), so each one visits only the points of the 2 km buckets
    # within that reach
    shape = np.shape(bed)
    bed = np.array(bed, dtype=np.float64).reshape(-1)
    px, py = np.asarray(x, np.float64).reshape(-1), np.asarray(y, np.float64).reshape(-1)
    cell = 2000.0
    ncx = int(lx / cell) + 2
    ncy = int(ly / cell) + 2
    bx = np.clip((px / cell).astype(np.int64), 0, ncx - 1)
    by = np.clip((py / cell).astype(np.int64), 0, ncy - 1)
    order = np.argsort(by * ncx + bx, kind="stable")
    start = np.searchsorted((by * ncx + bx)[order], np.arange(ncx * ncy + 1))
    for i in range(n_islands):
        reach = 6.5 * radius[i]
        i0 = max(0, int((cx[i] - reach) / cell))
        i1 = min(ncx - 1, int((cx[i] + reach) / cell))
        j0 = max(0, int((cy[i] - reach) / cell))
        j1 = min(ncy - 1, int((cy[i] + reach) / cell))
        if i0 > i1 or j0 > j1:
            continue
        idx = np.concatenate([order[start[j * ncx + i0]:start[j * ncx + i1 + 1]]
                              for j in range(j0, j1 + 1)])
        r2 = (px[idx] - cx[i]) ** 2 + (py[idx] - cy[i]) ** 2
        bed[idx] = bed[idx] + (centre_depth[i] + crest[i]) * np.exp(-r2 / radius[i] ** 2)
    return bed.reshape(shape)


COASTAL_TIDE = (("M2", 1.0), ("S2", 0.35), ("N2", 0.2), ("K1", 0.1))

# √area of the quads of an unrefined quadtree leaf is its side / (2√3); the
# three levels of the coastal paving hold quads of 400, 200 and 100 m at the
# default mean size (√(200 km · 150 km / 1 M) = 173.2 m)
PAVING_MEAN = 173.2
PAVING_COARSEST = 400.0


def _paving_count(level: np.ndarray, max_level: int) -> int:
    """Quads of :func:`mesh.quadtree_paving` on a balanced level field, without
    building it: three per triangle, four triangles per leaf plus one per
    leaf edge with a finer neighbour."""
    leaves = float((0.25 ** (max_level - level)).sum())
    splits = 0.0
    for a, b in ((level[:, :-1], level[:, 1:]), (level[:-1, :], level[1:, :])):
        coarse = np.minimum(a, b)
        splits += float((0.5 ** (max_level - coarse))[a != b].sum())
    return int(round(3.0 * (4.0 * leaves + splits)))


def coastal_paving(n_elements: int, seed: int, lx: float, ly: float, n_islands: int = 30,
                   island_radius: tuple[float, float] = (1000.0, 5000.0)):
    """A depth-graded unstructured quad paving of lx × ly with about
    ``n_elements`` quads: a three-level quadtree (quads of 400, 200 and
    100 m × mean/173.2 m, mean = √(lx·ly/n_elements)) whose leaves are
    finest over shallow water and land and coarsest over deep water — the
    level of a cell follows u^γ (u = (depth − 2 m)/298 m clipped to [0, 1],
    levels at u^γ < ¼ and < ¾), with γ found by bisection so that the count
    comes closest to ``n_elements``. Walls on the south, east and north
    sides, open to the west."""
    from .mesh import quadtree_levels, quadtree_paving

    max_level = 2
    scale = math.sqrt(lx * ly / n_elements) / PAVING_MEAN
    root = PAVING_COARSEST * 2.0 * math.sqrt(3.0) * scale
    nx, ny = (max(1, int(round(lx / root))) << max_level, max(1, int(round(ly / root))) << max_level)
    xc = (np.arange(nx) + 0.5) * (lx / nx)
    yc = (np.arange(ny) + 0.5) * (ly / ny)
    gx, gy = np.meshgrid(xc, yc)
    depth = -coastal_bed(gx, gy, lx, ly, seed, n_islands, island_radius)
    u = np.clip((depth - 2.0) / 298.0, 0.0, 1.0)

    def desired(log_gamma):
        w = u ** math.exp(log_gamma)
        return np.where(w < 0.25, 2, np.where(w < 0.75, 1, 0))

    lo, hi = -8.0, 8.0  # the count grows with γ
    for _ in range(40):
        mid = 0.5 * (lo + hi)
        if _paving_count(quadtree_levels(desired(mid), max_level), max_level) < n_elements:
            lo = mid
        else:
            hi = mid
    best = min((lo, hi), key=lambda g: abs(
        _paving_count(quadtree_levels(desired(g), max_level), max_level) - n_elements))
    return quadtree_paving(lx, ly, desired(best), max_level,
                           sides=(TAG_WALL, TAG_WALL, TAG_WALL, TAG_OPEN), jitter=0.1,
                           seed=seed, smoothing=1)


def coastal_box(n_elements: int = 1_000_000, order: int = 3, seed: int = 2026,
                numerics: int = abi.NUMERICS_FAST, lx: float = 200_000.0,
                ly: float = 150_000.0, n_islands: int = 30,
                island_radius: tuple[float, float] = (1000.0, 5000.0),
                tide: tuple = COASTAL_TIDE, manning_n: float = 0.02) -> Case:
    """The 1 M-quad coastal box: an unstructured quad paving of lx × ly
    (:func:`coastal_paving`, element size 100–400 m at the default size),
    Hilbert-ordered, with the seeded coastal bed, walls on three sides and a
    tide on the open western side, Manning's n and Coriolis at 63° N, from
    rest."""
    mesh = coastal_paving(n_elements, seed, lx, ly, n_islands, island_radius)
    mesh, _ = in_hilbert_order(mesh)
    form = SWEDeviceForm2D(mesh=mesh, order=order, numerics=numerics)
    x, y = node_positions(mesh, order)
    form.bathymetry = coastal_bed(x, y, lx, ly, seed, n_islands, island_radius)
    form.manning_n = manning_n
    form.coriolis_f0 = coriolis_parameter(63.0)
    rng = np.random.default_rng(seed + 1)
    phases = rng.uniform(0.0, 360.0, len(tide))
    cons = [tides.constituent(name, amp, ph) for (name, amp), ph in zip(tide, phases)]
    form.boundaries = {TAG_WALL: WallBoundary(), TAG_OPEN: TidalBoundary(cons, ramp_duration=3600.0)}
    return Case(form, at_rest(form), 0.5, abi.SSP_RK3, 2000.0)


def _member_box(n_elements: int) -> tuple:
    """lx, ly, island count and radius range of an ensemble member's box."""
    mean = 173.0
    area = n_elements * mean * mean
    lx = math.sqrt(area * 4.0 / 3.0)
    ly = 0.75 * lx
    n_islands = max(1, int(round(30.0 * area / (200_000.0 * 150_000.0))))
    radius = (min(1000.0, 0.05 * ly), min(5000.0, 0.1 * ly))
    return lx, ly, n_islands, radius


def ensemble_member(n_elements: int, order: int, seed: int, manning_n: float,
                    m2_amplitude: float, numerics: int = abi.NUMERICS_FAST) -> Case:
    """One member of a batched ensemble: the coastal-box generator scaled to
    ``n_elements`` quads of the same element sizes (mean 173 m, 4:3 box),
    with islands in proportion to the area (at least one, radii at most a
    tenth of the box) and an M2 tide of ``m2_amplitude``."""
    lx, ly, n_islands, radius = _member_box(n_elements)
    return coastal_box(n_elements, order, seed, numerics, lx, ly, n_islands, radius,
                       (("M2", m2_amplitude),), manning_n)


def ensemble_members(n_members: int = 256, seed: int = 2027,
                     k_range: tuple[int, int] = (5_000, 200_000), orders: tuple = (2, 3),
                     numerics: int = abi.NUMERICS_FAST) -> list[Case]:
    """The batched-ensemble workload: element counts log-uniform over
    ``k_range``, orders drawn from ``orders``, Manning n ~ U(0.015, 0.035)
    and M2 amplitude ~ U(0.5, 1.5) m per member, every draw seeded."""
    rng = np.random.default_rng(seed)
    k = np.exp(rng.uniform(math.log(k_range[0]), math.log(k_range[1]), n_members))
    order = rng.choice(np.asarray(orders), n_members)
    manning = rng.uniform(0.015, 0.035, n_members)
    amp = rng.uniform(0.5, 1.5, n_members)
    return [ensemble_member(int(round(k[i])), int(order[i]), seed * 1000 + i, float(manning[i]),
                            float(amp[i]), numerics) for i in range(n_members)]


def adjoint_channel(nx: int = 1000, ny: int = 100, order: int = 3, n_stations: int = 50,
                    seed: int = 2028, numerics: int = abi.NUMERICS_FAST):
    """The adjoint workload: the tidal channel refined to nx × ny quads
    (1000 × 100 at 50 m by default), Manning's n per element, seeded
    stations, and the friction field of the observations,
    n_obs = 0.02·(1 + 0.2·GRF) with a seeded Gaussian random field (2 km
    correlation) at the element centres. Returns the case (n = 0.02 per
    element), the stations [n][2] and n_obs per element."""
    case = tidal_channel(nx=nx, ny=ny, order=order, numerics=numerics)
    mesh = case.form.mesh
    rng = np.random.default_rng(seed)
    lx, ly = 50_000.0, 5_000.0
    stations = np.column_stack([rng.uniform(0.02 * lx, 0.98 * lx, n_stations),
                                rng.uniform(0.05 * ly, 0.95 * ly, n_stations)])
    centres = mesh.vertices[mesh.elements].mean(axis=1)
    spacing = 250.0
    grid = gaussian_random_field(int(lx / spacing) + 2, int(ly / spacing) + 2, spacing, 2_000.0, rng)
    z = _bilinear_grid(grid, spacing, centres[:, 0], centres[:, 1])
    nn = (order + 1) ** 2
    n_obs = 0.02 * (1.0 + 0.2 * z)
    case.form.manning_n = np.repeat(np.full(mesh.n_elements, 0.02), nn)
    return case, stations, n_obs


# the eight constituents of the batched adjoint, with typical amplitude ratios
ADJOINT_TIDE = (("M2", 1.0), ("S2", 0.35), ("N2", 0.2), ("K2", 0.1), ("K1", 0.1),
                ("O1", 0.08), ("P1", 0.03), ("Q1", 0.02))


@dataclass
class AdjointMember:
    """One member of the batched adjoint: its case (Manning's n per node),
    its stations [n][2], and the forcing of its observations (Manning's n
    per node and the tide's (amplitude, phase) [MAX_CONSTITUENTS][2], in
    the adjoint's parameter layout)."""
    case: Case
    stations: np.ndarray
    manning_obs: np.ndarray
    tide_obs: np.ndarray


def adjoint_ensemble_members(n_members: int = 64, seed: int = 2029,
                             k_range: tuple[int, int] = (10_000, 150_000), order: int = 3,
                             n_stations: int = 30,
                             numerics: int = abi.NUMERICS_FAST) -> list[AdjointMember]:
    """The batched-adjoint workload: ``n_members`` coastal boxes of
    log-uniform element counts over ``k_range`` (the ensemble generator's
    meshes and beds), order ``order``, each under the eight constituents of
    ``ADJOINT_TIDE`` scaled by U(0.5, 1.5) with seeded phases, with Manning's
    n per element n₀·(1 + 0.2·GRF), n₀ ~ U(0.015, 0.035) (5 km correlation),
    and ``n_stations`` stations at least 5 m deep (a sixth of them within
    3 km of the open side, which the tide reaches first). The observations' forcing
    perturbs each element's n by a factor 1 + 0.1·GRF and each constituent's
    amplitude by 5 % and phase by 3° (normal draws); a forward run under it
    gives the observed η."""
    rng = np.random.default_rng(seed)
    k = np.exp(rng.uniform(math.log(k_range[0]), math.log(k_range[1]), n_members))
    scale = rng.uniform(0.5, 1.5, n_members)
    n0 = rng.uniform(0.015, 0.035, n_members)
    out = []
    for m in range(n_members):
        mseed = seed * 1000 + m
        tide = tuple((name, amp * float(scale[m])) for name, amp in ADJOINT_TIDE)
        case = ensemble_member(int(round(k[m])), order, mseed, float(n0[m]), 1.0, numerics)
        mesh = case.form.mesh
        bc = case.form.boundaries[TAG_OPEN]
        mr = np.random.default_rng(mseed + 7)
        phases = mr.uniform(0.0, 360.0, len(tide))
        bc.constituents = [tides.constituent(name, amp, ph) for (name, amp), ph in zip(tide, phases)]
        # Manning's n per element, as a per-node field
        lx, ly, n_islands, radius = _member_box(int(round(k[m])))
        centres = mesh.vertices[mesh.elements].mean(axis=1)
        spacing = 1000.0
        nn = (order + 1) ** 2

        def field():
            g = gaussian_random_field(int(lx / spacing) + 2, int(ly / spacing) + 2, spacing,
                                      5_000.0, mr)
            return _bilinear_grid(g, spacing, centres[:, 0], centres[:, 1])

        n_elem = np.maximum(n0[m] * (1.0 + 0.2 * field()), 0.005)
        n_obs = np.maximum(n_elem * (1.0 + 0.1 * field()), 0.005)
        case.form.manning_n = np.repeat(n_elem, nn)
        # stations in water at least 5 m deep (the member's bed at the point),
        # a sixth of them within 3 km of the open (western) side
        def deep(n, x_hi):
            got = np.zeros((0, 2))
            while got.shape[0] < n:
                cand = np.column_stack([mr.uniform(0.02 * lx, x_hi, 4 * n),
                                        mr.uniform(0.02 * ly, 0.98 * ly, 4 * n)])
                bed = coastal_bed(cand[:, 0], cand[:, 1], lx, ly, mseed, n_islands, radius)
                got = np.vstack([got, cand[bed < -5.0]])
            return got[:n]

        n_near = n_stations // 6
        st = np.vstack([deep(n_near, min(3_000.0, 0.98 * lx)),
                        deep(n_stations - n_near, 0.98 * lx)])
        tide_obs = np.zeros((abi.MAX_CONSTITUENTS, 2))
        for i, c in enumerate(bc.constituents):
            tide_obs[i] = (c.amplitude * (1.0 + 0.05 * mr.standard_normal()),
                           c.phase + math.radians(3.0) * mr.standard_normal())
        out.append(AdjointMember(case, st[:n_stations], np.repeat(n_obs, nn), tide_obs))
    return out


def face_node_lists(n1: int) -> list[list[int]]:
    """The volume nodes of faces 0..3 in face-node order (faces 2 and 3
    reversed: compute_face_nodes, src/operators/operators_2d.rs:388-412)."""
    return [[a for a in range(n1)],
            [j * n1 + n1 - 1 for j in range(n1)],
            [(n1 - 1) * n1 + a for a in reversed(range(n1))],
            [j * n1 for j in reversed(range(n1))]]


def boundary_face_nodes(form: SWEDeviceForm2D, tag: int) -> list[int]:
    """The flat nodes of the boundary faces tagged ``tag``, each once, in
    element and face order (as TidalAtlas::boundary_tides numbers its slots,
    src/boundary/tidal_atlas.rs:598-630)."""
    mesh = form.mesh
    count: dict = {}
    for k, quad in enumerate(mesh.elements):
        for f in range(4):
            key = tuple(sorted((int(quad[f]), int(quad[(f + 1) % 4]))))
            count[key] = count.get(key, 0) + 1
    periodic = {(int(p[0]), int(p[1])) for p in mesh.periodic} | \
        {(int(p[2]), int(p[3])) for p in mesh.periodic}
    n1 = form.order + 1
    faces = face_node_lists(n1)
    seen, out = set(), []
    for k, quad in enumerate(mesh.elements):
        for f in range(4):
            key = tuple(sorted((int(quad[f]), int(quad[(f + 1) % 4]))))
            if count[key] > 1 or (k, f) in periodic:
                continue
            if mesh.face_tags is not None and int(mesh.face_tags[k][f]) != tag:
                continue
            for node in faces[f]:
                flat = k * n1 * n1 + node
                if flat not in seen:
                    seen.add(flat)
                    out.append(flat)
    return out


def synthetic_node_tides(form: SWEDeviceForm2D, tag: int = TAG_OPEN,
                         names=("M2", "S2", "N2", "K1", "O1"), seed: int = 2030,
                         velocity: bool = True, use_mean: bool = True,
                         max_transport_ratio: float | None = 2.5,
                         ramp_duration: float | None = 3600.0, by_position: bool = False):
    """BoundaryTides of a synthetic atlas on the boundary faces tagged
    ``tag``: per forced node, each constituent's elevation amplitude and
    phase vary smoothly along the boundary (amplitude 1 m for M2 scaled by
    the canonical ratios, ±20 % and ±15° along it), velocity constants of
    0.05–0.3 m/s, a mean level of a few cm and the source depth 0.8–1.2 times
    the node's own, all smooth along the boundary. ``by_position``: no
    slot_of_node (each face node takes the nearest slot)."""
    from .physics import NodeTidesBoundary

    ratio = {"M2": 1.0, "S2": 0.35, "N2": 0.2, "K2": 0.1, "K1": 0.1, "O1": 0.08, "P1": 0.03,
             "Q1": 0.02}
    rng = np.random.default_rng(seed)
    flats = boundary_face_nodes(form, tag)
    x, y = form.positions()
    x, y = x.reshape(-1)[flats], y.reshape(-1)[flats]
    length = max(float(np.ptp(x) + np.ptp(y)), 1.0)
    along = ((x - x.min()) + (y - y.min())) / length
    n, m = len(names), len(flats)
    coef = np.zeros((m, n, 6))
    for j, name in enumerate(names):
        amp = ratio.get(name, 0.05) * (1.0 + 0.2 * np.sin(2 * math.pi * along + rng.uniform(0, 6)))
        ph = math.radians(rng.uniform(0, 360)) + math.radians(15.0) * along
        coef[:, j, 0] = amp * np.cos(ph)
        coef[:, j, 1] = amp * np.sin(ph)
        for q in (2, 4):
            ua = rng.uniform(0.05, 0.3) * ratio.get(name, 0.05)
            uph = math.radians(rng.uniform(0, 360)) + math.radians(10.0) * along
            coef[:, j, q] = ua * np.cos(uph)
            coef[:, j, q + 1] = ua * np.sin(uph)
    omega = np.array([math.radians(tides.angular_speed(nm)) / 3600.0 for nm in names])
    f_rate = rng.uniform(-2e-10, 2e-10, n)
    bed = (form.bathymetry.reshape(-1)[flats] if form.bathymetry is not None else np.zeros(m))
    # smooth along the boundary, so coincident nodes of two faces agree
    depth = np.maximum(-bed, 0.5) * (1.0 + 0.2 * np.cos(2 * math.pi * along))
    mean = 0.025 + 0.02 * np.sin(3 * math.pi * along)
    slot_of_node = None
    if not by_position:
        slot_of_node = np.full(form.n_values, 0xFFFFFFFF, dtype=np.uint32)
        slot_of_node[flats] = np.arange(m, dtype=np.uint32)
    return NodeTidesBoundary(omega=omega, f_rate=f_rate, positions=np.column_stack([x, y]),
                             coefficients=coef, mean=mean,
                             source_depth=depth, slot_of_node=slot_of_node, velocity=velocity,
                             use_mean=use_mean, max_transport_ratio=max_transport_ratio,
                             ramp_duration=ramp_duration)


def synthetic_parent(form: SWEDeviceForm2D, tag: int = TAG_OPEN, t0: float = 0.0,
                     t1: float = 43_200.0, dt_snap: float = 3600.0, seed: int = 2031,
                     cubic: bool = True, velocity: bool = True,
                     max_transport_ratio: float | None = 2.5, reference_level: float = 0.1,
                     ramp_duration: float | None = 3600.0, by_position: bool = False,
                     band: int = 0):
    """An OceanModelState of a synthetic parent on the boundary faces tagged
    ``tag``: hourly snapshots (float32) from t0 to t1 of a parent whose ζ is
    a semidiurnal and a diurnal wave travelling along the boundary plus a
    slow surge, with depth-mean currents, and a parent depth 0.8–1.2 times
    the node's own. ``band`` extra slots off the boundary (not on_boundary)
    stand in for a relaxation band's nodes. ``by_position``: no
    slot_of_node."""
    from .physics import ParentBoundary

    rng = np.random.default_rng(seed)
    flats = boundary_face_nodes(form, tag)
    x, y = form.positions()
    x, y = x.reshape(-1)[flats], y.reshape(-1)[flats]
    length = max(float(np.ptp(x) + np.ptp(y)), 1.0)
    along = ((x - x.min()) + (y - y.min())) / length
    times = np.arange(t0, t1 + 0.5 * dt_snap, dt_snap)
    w1, w2 = 2 * math.pi / 44_714.0, 2 * math.pi / 86_164.0
    p1, p2 = rng.uniform(0, 2 * math.pi, 2)
    tt = times[None, :]
    a = along[:, None]
    zeta = (0.8 * np.cos(w1 * tt - 0.6 * a + p1) + 0.2 * np.cos(w2 * tt - 0.3 * a + p2)
            + 0.05 * np.sin(2 * math.pi * tt / 172_800.0))
    u = 0.3 * np.cos(w1 * tt - 0.6 * a + p1 + 0.7)
    v = 0.1 * np.sin(w1 * tt - 0.6 * a + p1 + 0.2)
    values = np.stack([zeta, u, v], axis=-1)
    positions = np.column_stack([x, y])
    bed = form.bathymetry.reshape(-1)[flats] if form.bathymetry is not None else np.zeros(len(x))
    depth = np.maximum(-bed, 0.5) * (1.0 + 0.2 * np.cos(2 * math.pi * along))
    on_boundary = np.ones(len(x), dtype=bool)
    if band:
        # band slots: inside the domain, far from the boundary's nodes
        positions = np.vstack([positions, positions[:band] + 1e5])
        values = np.concatenate([values, values[:band] * 0.5], axis=0)
        depth = np.concatenate([depth, depth[:band]])
        on_boundary = np.concatenate([on_boundary, np.zeros(band, dtype=bool)])
    slot_of_node = None
    if not by_position:
        slot_of_node = np.full(form.n_values, 0xFFFFFFFF, dtype=np.uint32)
        slot_of_node[flats] = np.arange(len(flats), dtype=np.uint32)
    return ParentBoundary(positions=positions, times=times,
                          values=values.astype(np.float32), parent_depth=depth,
                          on_boundary=on_boundary, slot_of_node=slot_of_node, cubic=cubic,
                          velocity=velocity, reference_level=reference_level,
                          max_transport_ratio=max_transport_ratio, ramp_duration=ramp_duration)


def synthetic_nesting(form: SWEDeviceForm2D, tag: int = TAG_OPEN, band_width: float = 4000.0,
                      rate: float = 1.0 / 1800.0, momentum_only: bool = False, **parent_kw):
    """A nesting of ``form`` in the synthetic parent (``synthetic_parent``):
    one series for the open boundary's nodes (weight 1) and for every node
    within ``band_width`` of them (weight (1 − d/W)², the relaxation band,
    as OceanModelState::new lays them out, src/boundary/ocean_nesting.rs:
    325-395). Returns the boundary condition and the relaxation band."""
    from .physics import RelaxationBand

    boundary = synthetic_parent(form, tag, by_position=False, **parent_kw)
    flats = boundary_face_nodes(form, tag)
    x, y = form.positions()
    x, y = x.reshape(-1), y.reshape(-1)
    bx, by = x[flats], y[flats]
    d = np.sqrt((x[:, None] - bx[None, :]) ** 2 + (y[:, None] - by[None, :]) ** 2).min(axis=1)
    on = np.zeros(form.n_values, dtype=bool)
    on[flats] = True
    band = np.flatnonzero(~on & (d < band_width))
    m = len(flats)
    # band slots take the nearest boundary node's series, scaled down inland
    nearest = np.argmin((x[band, None] - bx[None, :]) ** 2 + (y[band, None] - by[None, :]) ** 2,
                        axis=1)
    fall = (1.0 - 0.3 * d[band] / band_width)[:, None, None]
    values = np.concatenate([boundary.values, (boundary.values[nearest] * fall).astype(np.float32)])
    depth = np.concatenate([boundary.parent_depth, boundary.parent_depth[nearest]])
    positions = np.vstack([boundary.positions, np.column_stack([x[band], y[band]])])
    slot_of_node = np.full(form.n_values, 0xFFFFFFFF, dtype=np.uint32)
    slot_of_node[flats] = np.arange(m, dtype=np.uint32)
    slot_of_node[band] = m + np.arange(len(band), dtype=np.uint32)
    on_boundary = np.concatenate([np.ones(m, dtype=bool), np.zeros(len(band), dtype=bool)])
    weight = np.concatenate([np.ones(m), (1.0 - d[band] / band_width) ** 2])
    parent = dataclasses.replace(boundary, positions=positions, values=values, parent_depth=depth,
                                 on_boundary=on_boundary, slot_of_node=slot_of_node)
    return parent, RelaxationBand(parent=parent, weight=weight, rate=rate,
                                  momentum_only=momentum_only)


def synthetic_atmosphere(form: SWEDeviceForm2D, t0: float = 0.0, t1: float = 43_200.0,
                         dt_snap: float = 3600.0, epoch_unix: float = 1_750_000_000.0,
                         seed: int = 2033, depth_hpa: float = 25.0, radius: float | None = None,
                         max_wind: float = 22.0, background: tuple = (4.0, -2.0), **kw):
    """A GriddedAtmosphere of a synthetic storm over ``form``'s mesh,
    regridded onto its nodes as the reference's device holds one: a
    Gaussian low p − p_ref = −Δp·exp(−r²/R²) (its exact gradient), a
    cyclonic wind v_t = V·(r/R)·exp((1 − r²/R²)/2) around it plus a uniform
    background wind, the centre crossing the mesh's box diagonally between
    t0 and t1, snapshots every ``dt_snap`` (float32, Unix times from
    ``epoch_unix``). ``kw`` sets the GriddedAtmosphere's other fields."""
    from .physics import GriddedAtmosphere

    rng = np.random.default_rng(seed)
    x, y = form.positions()
    x, y = x.reshape(-1), y.reshape(-1)
    x0, x1, y0, y1 = x.min(), x.max(), y.min(), y.max()
    span = max(x1 - x0, y1 - y0, 1.0)
    R = radius if radius is not None else 0.35 * span
    times = np.arange(t0, t1 + 0.5 * dt_snap, dt_snap)
    frac = (times - t0) / max(t1 - t0, 1.0)
    jitter = rng.uniform(-0.1, 0.1, 2) * span
    cx = x0 - 0.2 * span + 1.4 * (x1 - x0 + 0.2 * span) * frac + jitter[0]
    cy = y0 + 0.3 * (y1 - y0) + 0.4 * (y1 - y0) * frac + jitter[1]
    dp = depth_hpa * 100.0
    values = np.empty((len(times), x.size, 5), dtype=np.float32)
    for n, (xc, yc) in enumerate(zip(cx, cy)):
        dx, dy = x - xc, y - yc
        r2 = (dx * dx + dy * dy) / (R * R)
        e = np.exp(-r2)
        p = -dp * e
        px, py = 2.0 * dp * e * dx / (R * R), 2.0 * dp * e * dy / (R * R)
        r = np.sqrt(dx * dx + dy * dy)
        vt = max_wind * np.sqrt(r2) * np.exp(0.5 * (1.0 - r2))
        inv = np.where(r > 0, 1.0 / np.maximum(r, 1e-12), 0.0)
        u = background[0] - vt * dy * inv
        v = background[1] + vt * dx * inv
        values[n] = np.stack([u, v, px, py, p], axis=-1)
    return GriddedAtmosphere(times=times + epoch_unix, values=values, epoch_unix=epoch_unix, **kw)


# -- the reference's split-form test setups ------------------------------------

L_TEST = 20_000.0


def smooth_bed(x, y):
    tau = 2.0 * math.pi / L_TEST
    return -200.0 + 150.0 * np.sin(tau * x) * np.cos(tau * y)


def xorshift_noise(n: int, seed: int = 0x9E37_79B9_7F4A_7C15) -> np.ndarray:
    """The reference tests' xorshift64 sequence, (seed >> 11)/2⁵³ per draw."""
    mask = (1 << 64) - 1
    out = np.empty(n)
    for i in range(n):
        seed ^= (seed << 13) & mask
        seed ^= seed >> 7
        seed ^= (seed << 17) & mask
        out[i] = (seed >> 11) / float(1 << 53)
    return out


def split_form_setup(order: int, periodic: bool, bed: str = "smooth", curved: bool = False,
                     numerics: int = abi.NUMERICS_FAST, formulation: int = abi.WET_DRY,
                     wet_dry: bool = False) -> SWEDeviceForm2D:
    """A 12 × 12 periodic mesh of [0, L]² or an 8 × 5 walled mesh of
    [0, L] × [0, L/2] (L = 20 km), with the smooth, cell-average or rough
    bed of the reference's tests; ``curved`` moves the vertices so every
    element is a general quadrilateral."""
    if periodic:
        mesh = uniform_periodic(0.0, L_TEST, 0.0, L_TEST, 12, 12)
    else:
        mesh = uniform_rectangle(0.0, L_TEST, 0.0, 0.5 * L_TEST, 8, 5)
    if curved:
        h_el = L_TEST / 12.0
        tau = 2.0 * math.pi / L_TEST

        def move(x, y):
            interior = (x > 0) & (x < L_TEST) & (y > 0) & (y < (L_TEST if periodic else 0.5 * L_TEST))
            a = 0.15 * h_el
            sx, sy = np.sin(3.0 * tau * x), np.sin(2.0 * tau * y)
            return (np.where(interior, x + a * sx * sy, x),
                    np.where(interior, y - 0.7 * a * sx * sy, y))
        mesh = move_vertices(mesh, move)
    form = SWEDeviceForm2D(mesh=mesh, order=order, numerics=numerics, formulation=formulation,
                           wet_dry=wet_dry, positivity_h_dry=1e-3 if wet_dry else None)
    x, y = node_positions(mesh, order)
    b = smooth_bed(x, y)
    if bed == "cell_average":
        b = np.repeat((b.sum(axis=1) / b.shape[1])[:, None], b.shape[1], axis=1)
    elif bed == "rough":
        b = b + 30.0 * (xorshift_noise(b.size).reshape(b.shape) - 0.5)
    form.bathymetry = b
    form.boundaries = {TAG_WALL: WallBoundary()}
    return form


def split_form_state(form: SWEDeviceForm2D, speed: float, eta: float = 0.3):
    """η = 0.3 m over the bed with the velocity speed·(cos·cos, ½ sin·cos)
    (src/solver/rhs/swe_2d_split_form.rs:1197-1214)."""
    tau = 2.0 * math.pi / L_TEST
    x, y = form.positions()
    h = eta - form.bathymetry
    u = speed * np.cos(tau * x) * np.cos(tau * y)
    v = 0.5 * speed * np.sin(tau * x) * np.cos(tau * y)
    return h.reshape(-1), (h * u).reshape(-1), (h * v).reshape(-1)


def shoreline_setup(order: int, periodic: bool, rough: bool, curved: bool = False,
                    numerics: int = abi.NUMERICS_FAST, formulation: int = abi.WET_DRY,
                    wet_dry: bool = False, h_min: float = 1e-6) -> SWEDeviceForm2D:
    """The reference's shoreline setup (src/solver/rhs/swe_2d_split_form.rs:1394-1417):
    B = −1 + 1.5 cos(τx) cos(τy), plus ±0.2 m of xorshift noise if ``rough``,
    so η = 0.3 leaves dry land and shorelines."""
    form = split_form_setup(order, periodic, "smooth", curved=curved, numerics=numerics,
                            formulation=formulation, wet_dry=wet_dry)
    form.h_min = h_min
    tau = 2.0 * math.pi / L_TEST
    x, y = form.positions()
    b = -1.0 + 1.5 * np.cos(tau * x) * np.cos(tau * y)
    if rough:
        b = b + 0.4 * (xorshift_noise(b.size, 0x2545_F491_4F6C_DD1D).reshape(b.shape) - 0.5)
    form.bathymetry = b
    return form


def shoreline_state(form: SWEDeviceForm2D, speed: float, eta: float = 0.3):
    """Lake at rest η = 0.3 (h = max(0, η − B)) with the test velocity field
    times ``speed`` at wet nodes (swe_2d_split_form.rs:1421-1437)."""
    h0, hu0, hv0 = split_form_state(form, speed, eta)
    h = np.maximum(eta - form.bathymetry.reshape(-1), 0.0)
    scale = np.where(h0 > 0.0, h / np.where(h0 > 0.0, h0, 1.0), 0.0)
    return h, hu0 * scale, hv0 * scale


def with_flow(case: Case, eta_amp: float = 0.5, u: float = 0.3, v: float = -0.1) -> tuple:
    """A flowing state on ``case``'s mesh: η = η_amp·cos(2πx/L_x) and a
    uniform velocity at the wet nodes, so that every field is O(1) (a state
    at rest has roundoff-level momentum, which no relative comparison can
    judge)."""
    x, _ = case.form.positions()
    lx = float(case.form.mesh.vertices[:, 0].max() - case.form.mesh.vertices[:, 0].min())
    b = case.form.bathymetry.reshape(x.shape)
    h = np.maximum(eta_amp * np.cos(2.0 * math.pi * x / lx) - b, 0.0)
    wet = h > 0.0
    return h.reshape(-1), np.where(wet, u * h, 0.0).reshape(-1), np.where(wet, v * h, 0.0).reshape(-1)
