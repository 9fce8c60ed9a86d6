"""A parent model's series as boundary data (DGSWE_BC_PARENT, the device
form of OceanModelState) on the device against the oracle, through the C
ABI: the RHS to TOL_RHS and a stage to TOL, linear and cubic in time,
elevation only or with the parent's currents and transport scaling, slots
by node or by the nearest boundary slot (band slots ignored); a run of
global steps; the span checked against the snapshots."""

import dataclasses

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.device import DeviceError, DeviceRun, SWEPhysics2D
from dgcom_gb300.mesh import TAG_OPEN
from oracle_lib import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_RHS = 1e-10


def rel_err(got, want):
    return max(float(np.abs(g - w).max() / max(np.abs(w).max(), 1e-300)) for g, w in zip(got, want))


def setup(numerics, **kw):
    case = cases.tidal_channel(nx=24, ny=3, order=2, numerics=numerics)
    form = case.form
    parent = cases.synthetic_parent(form, **kw)
    form = dataclasses.replace(form, boundaries={**form.boundaries, TAG_OPEN: parent})
    return case, form, cases.with_flow(case, eta_amp=0.3, u=0.3, v=0.05)


@pytest.mark.parametrize("numerics", [abi.NUMERICS_FAST, abi.NUMERICS_EXACT])
@pytest.mark.parametrize("cubic", [False, True])
@pytest.mark.parametrize("velocity,ratio", [(False, None), (True, None), (True, 2.5)])
@pytest.mark.parametrize("by_position", [False, True])
def test_rhs_and_stage_match_oracle(numerics, cubic, velocity, ratio, by_position):
    case, form, q = setup(numerics, cubic=cubic, velocity=velocity, max_transport_ratio=ratio,
                          by_position=by_position, band=3)
    dev, ref = SWEPhysics2D(form, 0), oracle(form)
    try:
        for s in (dev, ref):
            s.upload(*q)
        for t in (1800.0, 7200.0, 9000.5):  # in the ramp, at a snapshot, between
            err = rel_err(dev.compute_rhs_into(t), ref.compute_rhs_into(t))
            assert err <= TOL_RHS, f"t {t}: RHS {err:.3e}"
        dt = ref.compute_dt_ssp(0.5)
        for s in (dev, ref):
            s.stage_where(base=0, input=0, out=1, time=9000.5, a=1.0, b=0.0, c=dt)
        err = rel_err(dev.download(1), ref.download(1))
        assert err <= TOL, f"stage {err:.3e}"
    finally:
        dev.close()
        ref.close()


def test_run_matches_oracle_and_the_span_is_checked():
    case, form, q = setup(abi.NUMERICS_FAST)
    out = []
    for sim in (SWEPhysics2D(form, 0), oracle(form)):
        try:
            sim.upload(*q)
            rep = sim.run_with_callback(DeviceRun(span=(4000.0, 4300.0), cfl=0.5))
            assert rep.success, rep.message
            out.append((sim.download(), rep.n_steps))
        finally:
            sim.close()
    (a, na), (b, nb) = out
    assert na == nb
    assert rel_err(a, b) <= 1e-10
    dev = SWEPhysics2D(form, 0)
    try:
        dev.upload(*q)
        with pytest.raises(DeviceError):
            dev.run_with_callback(DeviceRun(span=(40_000.0, 50_000.0), cfl=0.5))
    finally:
        dev.close()


def nested(numerics, momentum_only=False, cubic=True):
    case = cases.tidal_channel(nx=24, ny=3, order=2, numerics=numerics)
    form = case.form
    parent, band = cases.synthetic_nesting(form, band_width=6000.0, cubic=cubic,
                                           momentum_only=momentum_only)
    form = dataclasses.replace(form, boundaries={**form.boundaries, TAG_OPEN: parent},
                               relaxation=band)
    return case, form, cases.with_flow(case, eta_amp=0.3, u=0.3, v=0.05)


@pytest.mark.parametrize("numerics", [abi.NUMERICS_FAST, abi.NUMERICS_EXACT])
@pytest.mark.parametrize("momentum_only", [False, True])
@pytest.mark.parametrize("cubic", [False, True])
def test_relaxation_band_matches_oracle(numerics, momentum_only, cubic):
    case, form, q = nested(numerics, momentum_only, cubic)
    dev, ref = SWEPhysics2D(form, 0), oracle(form)
    try:
        for s in (dev, ref):
            s.upload(*q)
        for t in (1800.0, 9000.5):
            err = rel_err(dev.compute_rhs_into(t), ref.compute_rhs_into(t))
            assert err <= TOL_RHS, f"t {t}: RHS {err:.3e}"
        dt = ref.compute_dt_ssp(0.5)
        for s in (dev, ref):
            s.stage_where(base=0, input=0, out=1, time=9000.5, a=1.0, b=0.0, c=dt)
        err = rel_err(dev.download(1), ref.download(1))
        assert err <= TOL, f"stage {err:.3e}"
    finally:
        dev.close()
        ref.close()


@pytest.mark.parametrize("levels", [0, 3])
def test_nested_run_matches_oracle(levels):
    case, form, q = nested(abi.NUMERICS_EXACT)
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
