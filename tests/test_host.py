"""Host-side logic: meshes, Hilbert order, node geometry, tides and the
workload generators."""

import math

import numpy as np

from dgcom_gb300 import cases, tides
from dgcom_gb300.mesh import (graded_jittered_box, hilbert_index, in_hilbert_order, node_mass,
                              node_positions, uniform_periodic, uniform_rectangle)


def test_uniform_rectangle_matches_the_reference_numbering():
    m = uniform_rectangle(0.0, 3.0, 0.0, 2.0, 3, 2)
    assert m.vertices.shape == (12, 2) and m.elements.shape == (6, 4)
    # element 0: vertices 0, 1, 5, 4 counter-clockwise (src/mesh/core/mesh2d.rs:244-250)
    assert list(m.elements[0]) == [0, 1, 5, 4]
    assert list(m.elements[4]) == [5, 6, 10, 9]


def test_periodic_pairs():
    m = uniform_periodic(0.0, 1.0, 0.0, 1.0, 3, 2)
    assert [tuple(p) for p in m.periodic] == [(2, 1, 0, 3), (5, 1, 3, 3), (3, 2, 0, 0),
                                             (4, 2, 1, 0), (5, 2, 2, 0)]


def test_hilbert_curve_visits_neighbours():
    cells = sorted((int(hilbert_index(np.array([x]), np.array([y]), 3)[0]), x, y)
                   for x in range(8) for y in range(8))
    for i, (a, b) in enumerate(zip(cells, cells[1:])):
        assert a[0] == i
        assert abs(a[1] - b[1]) + abs(a[2] - b[2]) == 1
    m = uniform_rectangle(0.0, 16.0, 0.0, 16.0, 16, 16)
    sorted_mesh, old = in_hilbert_order(m)
    assert sorted(old) == list(range(256))
    c = sorted_mesh.corners().mean(axis=1)
    steps = np.abs(np.diff(c, axis=0)).sum(axis=1)
    assert np.allclose(steps, 1.0)


def test_node_mass_sums_to_the_area():
    m = graded_jittered_box(2000.0, 1500.0, 20, 15, size_range=(80.0, 120.0), seed=3)
    for order in (1, 2, 3, 4):
        assert abs(node_mass(m, order).sum() - 2000.0 * 1500.0) < 1e-6 * 3e6
        x, y = node_positions(m, order)
        assert x.min() >= 0.0 and x.max() <= 2000.0 and y.min() >= 0.0 and y.max() <= 1500.0


def test_jittered_box_has_positive_jacobians():
    m = graded_jittered_box(20_000.0, 15_000.0, 60, 45, size_range=(250.0, 450.0), seed=11)
    assert (node_mass(m, 3) > 0.0).all()


def test_constituent_periods():
    # Schureman's speeds (deg/h): M2 28.9841042, S2 30, N2 28.4397295, K1 15.0410686
    for name, speed in (("M2", 28.9841042), ("S2", 30.0), ("N2", 28.4397295), ("K1", 15.0410686)):
        assert abs(tides.angular_speed(name) - speed) < 1e-6
    c = tides.constituent("M2", 1.0, 90.0)
    assert abs(tides.elevation([c], 0.25 * c.period) - 1.0) < 1e-12
    assert tides.elevation([c], 1800.0, ramp=3600.0) == 0.5 * tides.elevation([c], 1800.0)


def test_channel_workload():
    case = cases.tidal_channel()
    form = case.form
    assert form.mesh.n_elements == 4000 and form.order == 2
    b = form.bathymetry
    assert abs(b.min() + 20.0) < 1e-12 and abs(b.max() - 1.0) < 1e-12
    h = case.state[0]
    assert (h >= 0).all() and (h == 0).any()  # the head is dry at rest
    assert abs(form.boundaries[1].constituents[0].period / 3600.0 - 12.4206012) < 1e-6


def test_coastal_workload_is_seeded():
    a = cases.coastal_box(n_elements=5_000, order=3)
    b = cases.coastal_box(n_elements=5_000, order=3)
    assert np.array_equal(a.form.bathymetry, b.form.bathymetry)
    assert np.array_equal(a.form.mesh.vertices, b.form.mesh.vertices)
    assert a.form.bathymetry.min() >= -300.0 - 1e-9
    assert (a.state[0] == 0).any() and (a.state[0] > 0).any()
    assert abs(a.form.coriolis_f0 - 2 * 7.292115e-5 * math.sin(math.radians(63.0))) < 1e-18


def test_integer_pipe_compares_match_ieee(tmp_path):
    """The kernels' fp:: compares, minima and maxima give the IEEE result."""
    import shutil
    import subprocess
    from pathlib import Path

    gxx = shutil.which("g++")
    if gxx is None:
        import pytest

        pytest.skip("g++ not available")
    here = Path(__file__).resolve().parent
    exe = tmp_path / "fp64_bits_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(here.parent / "dgcom_gb300" / "csrc"),
                    str(here / "fp64_bits_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok ")


def test_reverse_point_functions_match_finite_differences(tmp_path):
    """Every reverse function of the adjoint (adjoint_point.cuh) against
    central differences of its forward function (point.cuh), host build."""
    import shutil
    import subprocess
    from pathlib import Path

    gxx = shutil.which("g++")
    if gxx is None:
        import pytest

        pytest.skip("g++ not available")
    here = Path(__file__).resolve().parent
    exe = tmp_path / "adjoint_point_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(here.parent / "dgcom_gb300" / "csrc"),
                    str(here / "adjoint_point_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("all ok")


def test_coastal_paving_is_an_unstructured_conforming_quad_mesh():
    """The coastal box's mesh: about the requested count, every interior
    edge shared by exactly two elements in opposite directions, positive
    Jacobians, the stretch below 3, element sizes over the three levels,
    vertex valences other than 4 (not a tensor grid), and the sides
    tagged (walls south, east and north, open to the west)."""
    from dgcom_gb300.mesh import TAG_OPEN, TAG_WALL, corner_jacobians, element_shape

    lx, ly = 200_000.0, 150_000.0
    mesh = cases.coastal_paving(40_000, 2026, lx, ly)
    assert abs(mesh.n_elements - 40_000) <= 400
    e = mesh.elements
    a, b = e.reshape(-1), np.roll(e, -1, axis=1).reshape(-1)
    fwd = {(int(p), int(q)) for p, q in zip(a, b)}
    assert len(fwd) == a.size  # no directed edge twice (orientation is consistent)
    interior = [(p, q) for p, q in fwd if (q, p) in fwd]
    boundary = [(p, q) for p, q in fwd if (q, p) not in fwd]
    assert len(interior) + len(boundary) == a.size
    v = mesh.vertices
    on_box = lambda i: (v[i, 0] in (0.0, lx)) or (v[i, 1] in (0.0, ly))  # noqa: E731
    assert all(on_box(p) and on_box(q) for p, q in boundary)
    # boundary faces tagged by side; the west side open
    tag_of = {}
    for k in range(mesh.n_elements):
        for f in range(4):
            tag_of[(int(e[k, f]), int(e[k, (f + 1) % 4]))] = int(mesh.face_tags[k, f])
    for p, q in boundary:
        west = v[p, 0] == 0.0 and v[q, 0] == 0.0
        assert tag_of[(p, q)] == (TAG_OPEN if west else TAG_WALL)
    assert corner_jacobians(mesh).min() > 0.0
    size, stretch = element_shape(mesh)
    assert stretch.max() < 3.0
    mean = np.sqrt(lx * ly / 40_000)
    lo, hi = np.percentile(size, [1, 99]) / mean * 173.2
    assert 70.0 < lo < 130.0 and 330.0 < hi < 470.0, (lo, hi)
    valence = np.bincount(a, minlength=v.shape[0])
    assert (valence == 3).any() and (valence > 4).any()


def test_dt_single_precision_filter_bound(tmp_path):
    """The dt pass's float rates (point.cuh node_rate_f32) stay within their
    stated error bound of the double rates, and the filter keeps every
    element's largest rate, on random nodes (host build)."""
    import shutil
    import subprocess
    from pathlib import Path

    gxx = shutil.which("g++")
    if gxx is None:
        import pytest

        pytest.skip("g++ not available")
    here = Path(__file__).resolve().parent
    exe = tmp_path / "dt_filter_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(here.parent / "dgcom_gb300" / "csrc"),
                    str(here / "dt_filter_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok ")


def test_sequential_breakdown_recovers_overhead_and_bound():
    """The ensemble bench's breakdown of the sequential arm: runs whose step
    costs overhead + nodes × cost give back both, the overhead's share, and
    the batching bound (sequential time over the members' work at the
    fastest run's throughput)."""
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench

    steps, overhead, cost = 10, 2e-4, 1e-9
    nodes = [16 * k for k in (5_000, 20_000, 80_000, 200_000)]
    runs = [(n // 16, 3, n, steps * (overhead + cost * n)) for n in nodes]
    b = bench.sequential_breakdown(runs, steps, batched_seconds=steps * cost * sum(nodes))
    assert abs(b["overhead_ms_per_run_step"] - 0.2) < 1e-9
    assert abs(b["ns_per_node_step"] - 1.0) < 1e-9
    seq = sum(overhead + cost * n for n in nodes)
    assert abs(b["overhead_share"] - 4 * overhead / seq) < 1e-12
    fastest = max(3 * n / (overhead + cost * n) for n in nodes)
    assert abs(b["bound_speedup"] - seq / (3 * sum(nodes) / fastest)) < 1e-9
    assert len(b["runs"]) == 4


def test_host_step_ready_lists(tmp_path):
    """The host-state step's ready lists (ready_lists in host_common.hpp)
    on scrambled grids with boundary gaps: every element, edge and boundary
    face listed once, in the chunk of the latest data it reads, in index
    order (tests/ready_lists_check.cpp, host build)."""
    import shutil
    import subprocess
    from pathlib import Path

    gxx = shutil.which("g++")
    if gxx is None:
        import pytest

        pytest.skip("g++ not available")
    here = Path(__file__).resolve().parent
    exe = tmp_path / "ready_lists_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", str(here.parent / "dgcom_gb300" / "csrc"),
                    str(here / "ready_lists_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok ")
