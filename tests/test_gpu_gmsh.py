"""A mesh that comes in through a Gmsh file runs on the device as it does
on the oracle: an unstructured-like graded box written as MSH 2.2 and as
binary MSH 4.1, read back (Hilbert order, tags from physical groups), with
a tide on the group tagged open and walls elsewhere."""

import numpy as np
import pytest

from dgcom_gb300 import abi, gmsh, tides
from dgcom_gb300.cases import Case, with_flow
from dgcom_gb300.device import DeviceRun, SWEPhysics2D
from dgcom_gb300.mesh import TAG_OPEN, TAG_WALL, custom_tag, graded_jittered_box
from dgcom_gb300.physics import SWEDeviceForm2D, TidalBoundary, WallBoundary, at_rest
from oracle_lib import oracle

pytestmark = pytest.mark.gpu


def bay_case(path, order):
    mesh = gmsh.read_gmsh_mesh(path)
    form = SWEDeviceForm2D(mesh=mesh, order=order)
    x, y = form.positions()
    form.bathymetry = -(1.0 + 24.0 * (1.0 - x / 6000.0) + 2.0 * np.sin(y / 700.0))
    form.manning_n = 0.025
    form.coriolis_f0 = 1.2e-4
    form.boundaries = {TAG_WALL: WallBoundary(), custom_tag(13): WallBoundary(),
                       TAG_OPEN: TidalBoundary([tides.constituent("M2", 0.8, 20.0)],
                                               ramp_duration=600.0)}
    return Case(form, at_rest(form, 0.0), 0.5, abi.SSP_RK3, 0.0)


@pytest.fixture(params=["v22", "v41_binary"])
def msh_path(request, tmp_path):
    m = graded_jittered_box(6000.0, 4000.0, 24, 16, size_range=(150.0, 400.0), jitter=0.2, seed=9,
                            sides=(TAG_WALL, custom_tag(13), TAG_WALL, TAG_OPEN))
    path = tmp_path / "bay.msh"
    if request.param == "v22":
        gmsh.write_gmsh_mesh(m, path)
    else:
        nodes = [(i + 1, float(x), float(y)) for i, (x, y) in enumerate(m.vertices)]
        quads = [(k + 1, *(int(v) + 1 for v in q)) for k, q in enumerate(m.elements)]
        rows = gmsh.boundary_edges(m)
        curve = {TAG_WALL: 1, custom_tag(13): 2, TAG_OPEN: 3}
        lines = [(len(quads) + i + 1, curve[int(t)], int(a) + 1, int(b) + 1)
                 for i, (_, _, a, b, t) in enumerate(rows)]
        path.write_bytes(gmsh.binary_msh41(
            nodes, quads, lines, {1: [7], 2: [13], 3: [8]},
            [(1, 7, "coast"), (1, 13, "outflow"), (1, 8, "ocean")]))
    return path


@pytest.mark.parametrize("order", [2, 3])
def test_gmsh_mesh_steps_like_the_oracle(msh_path, order):
    case = bay_case(msh_path, order)
    q = with_flow(case)
    dev, ref = SWEPhysics2D(case.form, 0), oracle(case.form)
    try:
        for s in (dev, ref):
            s.upload(*q)
        t = 300.0
        for _ in range(4):
            dt = ref.compute_dt_ssp(case.cfl)
            assert abs(dev.compute_dt_ssp(case.cfl) - dt) <= 1e-12 * dt
            for s in (dev, ref):
                s.step(t, dt)
            t += dt
        for a, b in zip(dev.download(), ref.download()):
            assert np.abs(a - b).max() <= 1e-12 * max(np.abs(b).max(), 1e-300)
    finally:
        dev.close()
        ref.close()


def test_gmsh_mesh_runs_with_local_time_stepping(msh_path):
    case = bay_case(msh_path, 2)
    q = with_flow(case)
    got = []
    for sim in (SWEPhysics2D(case.form, 0), oracle(case.form)):
        try:
            sim.upload(*q)
            rep = sim.run_with_callback(DeviceRun(span=(300.0, 1e9), cfl=0.5, levels=4,
                                                  max_steps=2))
            assert rep.n_steps == 2
            got.append((sim.download(), rep.local_time_stepping))
        finally:
            sim.close()
    (a, sa), (b, sb) = got
    assert sa.element_evaluations == sb.element_evaluations and sa.finest_level >= 1
    for x, y in zip(a, b):
        assert np.abs(x - y).max() <= 1e-12 * 2 ** sb.finest_level * max(np.abs(y).max(), 1e-300)
