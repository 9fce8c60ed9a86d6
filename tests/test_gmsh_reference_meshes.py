"""The reader on meshes Gmsh itself wrote, the reference's own fixtures
(tests/data/gmsh/), held to what the reference's tests assert of them
(tests/gmsh_mesh_test.rs:56-170, tests/local_time_stepping_test.rs:700-730),
and the oracle's multirate stepper on the farm-refined fjord. Skipped where
the reference repository is not present (it is read in place, never
copied)."""

import math

import numpy as np
import pytest

from dgcom_gb300 import gmsh
from dgcom_gb300.device import DeviceRun
from dgcom_gb300.mesh import TAG_OPEN, TAG_WALL, custom_tag, node_mass
from dgcom_gb300.physics import SWEDeviceForm2D, WallBoundary
from oracle_lib import oracle

# The bay's geometry (the fixture script's constants, as the reference's test states them)
LX, LY, COAST_AMP = 2000.0, 1200.0, 150.0
ISLAND = (1200.0, 650.0, 220.0, 150.0)


def bay(reference_data, name="bay_quads_v41.msh"):
    return gmsh.read_gmsh_mesh(reference_data(f"tests/data/gmsh/{name}"))


def test_three_formats_load_to_the_same_mesh(reference_data):
    ascii_mesh = bay(reference_data)
    for name in ("bay_quads_v41_binary.msh", "bay_quads_v22.msh"):
        other = bay(reference_data, name)
        # Gmsh writes 16 significant digits in ASCII, exact values in binary
        assert other.vertices.shape == ascii_mesh.vertices.shape
        assert np.abs(other.vertices - ascii_mesh.vertices).sum(axis=1).max() < 1e-12 * LX
        assert np.array_equal(other.elements, ascii_mesh.elements)
        assert np.array_equal(other.face_tags, ascii_mesh.face_tags)


def test_bay_geometry_and_tags(reference_data):
    mesh = bay(reference_data)
    assert mesh.n_elements == 192
    rows = gmsh.boundary_edges(mesh)
    on_boundary = np.zeros(mesh.vertices.shape[0], bool)
    on_boundary[rows[:, 2]] = on_boundary[rows[:, 3]] = True
    valence = np.bincount(mesh.elements.reshape(-1), minlength=mesh.vertices.shape[0])
    assert np.any(valence[~on_boundary] != 4)  # unstructured
    # the bay's area: rectangle − under the coastline − island, within 1 %
    area = node_mass(mesh, 3).sum()
    exact = LX * LY - 0.5 * COAST_AMP * LX - math.pi * ISLAND[2] * ISLAND[3]
    assert abs(area - exact) < 0.01 * exact

    def on_island(p):
        cx, cy, a, b = ISLAND
        return abs(((p[0] - cx) / a) ** 2 + ((p[1] - cy) / b) ** 2 - 1.0) < 1e-6

    lengths = {TAG_WALL: 0.0, TAG_OPEN: 0.0, custom_tag(13): 0.0}
    for _, _, va, vb, tag in rows:
        a, b = mesh.vertices[va], mesh.vertices[vb]
        length = math.hypot(*(b - a))
        if tag == TAG_WALL:  # "coast": the coastline and the island
            assert (on_island(a) and on_island(b)) or (a[1] <= COAST_AMP + 1 and b[1] <= COAST_AMP + 1)
        elif tag == TAG_OPEN:  # "open": west and north
            assert (a[0] == 0.0 and b[0] == 0.0) or (a[1] == LY and b[1] == LY)
        elif tag == custom_tag(13):  # "outflow": east
            assert a[0] == LX and b[0] == LX
        else:
            pytest.fail(f"boundary edge tagged {tag}")
        lengths[int(tag)] += length
    side = LY - 0.5 * COAST_AMP
    assert abs(lengths[TAG_OPEN] - (LX + side)) < 1e-9 * LX
    assert abs(lengths[custom_tag(13)] - side) < 1e-9 * LX
    a, b = ISLAND[2], ISLAND[3]
    h = ((a - b) / (a + b)) ** 2
    perimeter = math.pi * (a + b) * (1.0 + 3.0 * h / (10.0 + math.sqrt(4.0 - 3.0 * h)))
    assert LX + 0.97 * perimeter < lengths[TAG_WALL] < 1.1 * LX + perimeter


def test_quad_dominant_mesh_is_refused(reference_data):
    with pytest.raises(gmsh.UnsupportedElements) as err:
        bay(reference_data, "bay_quad_dominant_v41.msh")
    assert err.value.counts == [(2, 34)]
    assert "34 × 3-node triangle" in str(err.value)


def test_farm_refinement_saves_rhs_work(reference_data):
    """The farm-refined fjord (20 m quads at the farm, ≈ 450 m away), order
    1, walls, a bump at rest: up to 8 levels at CFL 0.8 for 10 s reach a
    finest level of at least 5 with more than 2× less RHS work than global
    steps at the finest step, and conserve mass."""
    mesh = gmsh.read_gmsh_mesh(reference_data("tests/data/gmsh/fjord_farm.msh"))
    assert mesh.n_elements == 3584
    form = SWEDeviceForm2D(mesh=mesh, order=1)
    x, y = form.positions()
    bed = -(30.0 + 120.0 * (1.0 - x / 12_000.0)) - 10.0 * np.sin(y / 2_000.0)
    form.bathymetry = bed
    form.boundaries = {int(t): WallBoundary() for t in np.unique(mesh.face_tags)}
    eta = 0.3 * np.exp(-((x - 6_000.0) ** 2 + (y - 3_000.0) ** 2) / 400.0 ** 2)
    h = np.maximum(eta - bed, 0.0).reshape(-1)
    q = (h, np.zeros_like(h), np.zeros_like(h))
    w = node_mass(mesh, 1).reshape(-1)
    ref = oracle(form)
    try:
        ref.upload(*q)
        rep = ref.run_with_callback(DeviceRun(span=(0.0, 10.0), cfl=0.8, levels=8))
        assert rep.success, rep.message
        out = ref.download()
    finally:
        ref.close()
    stats = rep.local_time_stepping
    assert stats.finest_level >= 5
    assert stats.global_evaluations / stats.element_evaluations > 2.0
    mass0, mass1 = float(w @ q[0]), float(w @ out[0])
    assert abs(mass1 - mass0) / mass0 < 1e-13
