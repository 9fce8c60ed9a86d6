"""Edge cases of the device path against the oracle or the exact answer:
a mesh of one element, a mesh with no water at all, the lowest and highest
orders under local time stepping, an ensemble of one member, an adjoint
without stations."""

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.adjoint import Adjoint
from dgcom_gb300.device import DeviceRun, SWEPhysics2D
from dgcom_gb300.ensemble import Ensemble
from dgcom_gb300.mesh import TAG_WALL, uniform_rectangle
from dgcom_gb300.physics import SWEDeviceForm2D, WallBoundary, at_rest
from oracle_lib import oracle
from test_multirate_oracle import basin

pytestmark = pytest.mark.gpu


def rel_err(got, want):
    return max(float(np.abs(g - w).max() / max(np.abs(w).max(), 1e-300)) for g, w in zip(got, want))


@pytest.mark.parametrize("levels", [0, 3])
def test_one_element_lake_stays_at_rest(levels):
    mesh = uniform_rectangle(0.0, 100.0, 0.0, 100.0, 1, 1)
    form = SWEDeviceForm2D(mesh=mesh, order=3)
    x, y = form.positions()
    form.bathymetry = -(5.0 + 0.5 * np.sin(x / 30.0) * np.cos(y / 40.0))
    form.boundaries = {TAG_WALL: WallBoundary()}
    q = at_rest(form, eta=0.2)
    dev = SWEPhysics2D(form, 0)
    try:
        dev.upload(*q)
        rep = dev.run_with_callback(DeviceRun(span=(0.0, 30.0), cfl=0.5, levels=levels))
        assert rep.success, rep.message
        h, hu, hv = dev.download()
    finally:
        dev.close()
    assert np.abs(h - q[0]).max() <= 1e-12 * q[0].max()
    assert np.abs(hu).max() <= 1e-12 and np.abs(hv).max() <= 1e-12


@pytest.mark.parametrize("levels", [0, 3])
def test_a_dry_mesh_lands_in_one_step(levels):
    """No water: every element step is unlimited, so the run takes one step
    to its end and nothing moves (a coarse step of one level when
    multirate)."""
    mesh = uniform_rectangle(0.0, 400.0, 0.0, 200.0, 4, 2)
    form = SWEDeviceForm2D(mesh=mesh, order=2)
    form.bathymetry = np.full((mesh.n_elements, 9), 1.0)  # land, 1 m above the datum
    form.boundaries = {TAG_WALL: WallBoundary()}
    q = at_rest(form)
    assert q[0].max() == 0.0
    dev = SWEPhysics2D(form, 0)
    try:
        dev.upload(*q)
        rep = dev.run_with_callback(DeviceRun(span=(0.0, 100.0), cfl=0.5, levels=levels))
        assert rep.success, rep.message
        assert rep.n_steps == 1 and rep.final_time == 100.0
        out = dev.download()
    finally:
        dev.close()
    for x in out:
        assert np.array_equal(x, np.zeros_like(x))


@pytest.mark.parametrize("order", [1, 4])
def test_multirate_at_the_lowest_and_highest_orders(order):
    form, q = basin(order=order)
    got = []
    for sim in (SWEPhysics2D(form, 0), oracle(form)):
        try:
            sim.upload(*q)
            rep = sim.run_with_callback(DeviceRun(span=(0.0, 1e9), cfl=0.5, levels=4, max_steps=1))
            assert rep.n_steps == 1
            got.append((sim.download(), rep.local_time_stepping))
        finally:
            sim.close()
    (a, sa), (b, sb) = got
    assert sa.element_evaluations == sb.element_evaluations
    assert rel_err(a, b) <= 1e-12 * 2 ** sb.finest_level


def test_an_ensemble_of_one_member_is_its_run():
    case = cases.tidal_channel(nx=20, ny=4, order=2)
    q = cases.with_flow(case)
    ens = Ensemble([case.form], 0)
    try:
        ens.upload(0, *q)
        reports, _ = ens.run(5, case.cfl, t_start=100.0)
        got = ens.download(0)
    finally:
        ens.close()
    dev = SWEPhysics2D(case.form, 0)
    try:
        dev.upload(*q)
        rep = dev.run_with_callback(DeviceRun(span=(100.0, 1e9), cfl=case.cfl, max_steps=5))
        want = dev.download()
    finally:
        dev.close()
    assert reports[0].n_steps == rep.n_steps == 5
    for a, b in zip(got, want):
        assert np.array_equal(a, b)


def test_an_adjoint_without_stations_has_no_gradient():
    case = cases.tidal_channel(nx=20, ny=4, order=2)
    form = case.form
    form.manning_n = np.full(form.n_values, 0.025)
    with Adjoint(form, 6, np.zeros((0, 2)), t_start=4000.0) as adj:
        J, eta, dts = adj.forward(cases.with_flow(case))
        g = adj.reverse()
    assert J == 0.0 and eta.shape == (6, 0) and np.all(dts > 0.0)
    for x in (g.h0, g.hu0, g.hv0, g.bed, g.manning):
        assert not np.any(x)
