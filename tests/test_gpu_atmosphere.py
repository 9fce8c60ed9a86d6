"""A weather model's wind and air pressure (the device form of
GriddedAtmosphere2D: the source term DeviceSource2D::Atmosphere and the
open boundaries' inverse-barometer raise, DeviceLevel::Atmosphere) on the
device against the oracle, through the C ABI: the RHS to TOL_RHS and a
stage to TOL with a storm crossing the tidal channel (wind and pressure,
either alone, ramped, three drag laws); the raise on a uniform tide, on
tides per node and on a parent series; the weather with a relaxation band;
runs of global and multirate steps; the span checked against the
snapshots; the ensemble and the adjoint refusing the weather."""

import dataclasses

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.adjoint import Adjoint
from dgcom_gb300.device import DeviceError, DeviceRun, SWEPhysics2D
from dgcom_gb300.ensemble import Ensemble
from dgcom_gb300.mesh import TAG_OPEN
from oracle_lib import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_RHS = 1e-10


def rel_err(got, want):
    return max(float(np.abs(g - w).max() / max(np.abs(w).max(), 1e-300)) for g, w in zip(got, want))


def setup(numerics=abi.NUMERICS_FAST, open_bc=None, raise_factor=None, relaxation=False, **kw):
    case = cases.tidal_channel(nx=24, ny=3, order=2, numerics=numerics)
    form = case.form
    weather = cases.synthetic_atmosphere(form, **kw)
    boundaries = dict(form.boundaries)
    band = None
    if relaxation:
        boundaries[TAG_OPEN], band = cases.synthetic_nesting(form, band_width=6000.0)
    elif open_bc == "node_tides":
        boundaries[TAG_OPEN] = cases.synthetic_node_tides(form)
    elif open_bc == "parent":
        boundaries[TAG_OPEN] = cases.synthetic_parent(form)
    if raise_factor is not None:
        boundaries[TAG_OPEN] = dataclasses.replace(boundaries[TAG_OPEN], raise_factor=raise_factor)
    form = dataclasses.replace(form, boundaries=boundaries, atmosphere=weather, relaxation=band)
    return case, form, cases.with_flow(case, eta_amp=0.3, u=0.3, v=0.05)


def check_rhs_and_stage(form, q, times=(1800.0, 7200.0, 9000.5)):
    dev, ref = SWEPhysics2D(form, 0), oracle(form)
    try:
        for s in (dev, ref):
            s.upload(*q)
        for t in times:  # in the tide's ramp, at a snapshot, between snapshots
            err = rel_err(dev.compute_rhs_into(t), ref.compute_rhs_into(t))
            assert err <= TOL_RHS, f"t {t}: RHS {err:.3e}"
        dt = ref.compute_dt_ssp(0.5)
        for s in (dev, ref):
            s.stage_where(base=0, input=0, out=1, time=times[-1], a=1.0, b=0.0, c=dt)
        err = rel_err(dev.download(1), ref.download(1))
        assert err <= TOL, f"stage {err:.3e}"
    finally:
        dev.close()
        ref.close()


@pytest.mark.parametrize("numerics", [abi.NUMERICS_FAST, abi.NUMERICS_EXACT])
@pytest.mark.parametrize("wind,pressure", [(True, True), (True, False), (False, True)])
@pytest.mark.parametrize("ramp", [None, 7200.0])
def test_source_matches_oracle(numerics, wind, pressure, ramp):
    case, form, q = setup(numerics, wind=wind, pressure=pressure, ramp_duration=ramp)
    check_rhs_and_stage(form, q)


@pytest.mark.parametrize("drag,cd", [(abi.DRAG_CONSTANT, 1.6e-3), (abi.DRAG_WU, 0.0),
                                     (abi.DRAG_YELLAND_TAYLOR, 0.0)])
def test_drag_laws_match_oracle(drag, cd):
    case, form, q = setup(abi.NUMERICS_EXACT, drag=drag, drag_cd=cd, max_wind=30.0)
    check_rhs_and_stage(form, q)


def test_the_source_changes_the_rhs():
    case, form, q = setup()
    plain = dataclasses.replace(form, atmosphere=None)
    dev = [SWEPhysics2D(f, 0) for f in (form, plain)]
    try:
        for d in dev:
            d.upload(*q)
        a, b = (d.compute_rhs_into(9000.5) for d in dev)
        assert np.array_equal(a[0], b[0])  # no mass source
        assert np.abs(a[1] - b[1]).max() > 1e-4  # a storm's wind and pressure gradient
    finally:
        for d in dev:
            d.close()


@pytest.mark.parametrize("numerics", [abi.NUMERICS_FAST, abi.NUMERICS_EXACT])
@pytest.mark.parametrize("open_bc", [None, "node_tides", "parent"])
@pytest.mark.parametrize("factor", [1.0, 0.25])
def test_raise_matches_oracle(numerics, open_bc, factor):
    case, form, q = setup(numerics, open_bc=open_bc, raise_factor=factor)
    check_rhs_and_stage(form, q)


def test_raise_only_atmosphere_and_no_level():
    """A weather that only raises the boundary (no source), and one without
    a pressure field (its level is 0: the unraised boundary's RHS)."""
    case, form, q = setup(raise_factor=1.0, source=False)
    check_rhs_and_stage(form, q)
    no_level = dataclasses.replace(form, atmosphere=dataclasses.replace(
        form.atmosphere, has_pressure=False))
    unraised = dataclasses.replace(form, boundaries={
        **form.boundaries, TAG_OPEN: dataclasses.replace(form.boundaries[TAG_OPEN],
                                                         raise_factor=None)})
    dev = [SWEPhysics2D(f, 0) for f in (no_level, unraised)]
    try:
        for d in dev:
            d.upload(*q)
        a, b = (d.compute_rhs_into(9000.5) for d in dev)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    finally:
        for d in dev:
            d.close()


@pytest.mark.parametrize("numerics", [abi.NUMERICS_FAST, abi.NUMERICS_EXACT])
def test_with_relaxation_band_matches_oracle(numerics):
    case, form, q = setup(numerics, relaxation=True, raise_factor=1.0)
    check_rhs_and_stage(form, q)


@pytest.mark.parametrize("levels", [0, 3])
@pytest.mark.parametrize("relaxation", [False, True])
def test_run_matches_oracle(levels, relaxation):
    case, form, q = setup(abi.NUMERICS_EXACT, raise_factor=1.0, relaxation=relaxation)
    out = []
    for sim in (SWEPhysics2D(form, 0), oracle(form)):
        try:
            sim.upload(*q)
            rep = sim.run_with_callback(DeviceRun(span=(4000.0, 4200.0), cfl=0.5, levels=levels))
            assert rep.success, rep.message
            out.append((sim.download(), rep.n_steps))
        finally:
            sim.close()
    (a, na), (b, nb) = out
    assert na == nb
    assert rel_err(a, b) <= 1e-10


def test_span_beyond_the_snapshots_is_refused():
    case, form, q = setup(t1=7200.0)
    dev = SWEPhysics2D(form, 0)
    try:
        dev.upload(*q)
        with pytest.raises(DeviceError):
            dev.run_with_callback(DeviceRun(span=(6000.0, 9000.0), cfl=0.5))
        with pytest.raises(DeviceError):
            dev.compute_rhs_into(7300.0)
        dev.compute_rhs_into(7200.0)
    finally:
        dev.close()


def test_ensemble_and_adjoint_refuse_the_weather():
    case, form, q = setup()
    with pytest.raises(DeviceError) as err:
        Ensemble([form, case.form])
    assert err.value.status == abi.ERR_UNSUPPORTED
    with pytest.raises(DeviceError) as err:
        Adjoint(form, 4, np.array([[10_000.0, 2_500.0]]), t_start=4000.0)
    assert err.value.status == abi.ERR_UNSUPPORTED
