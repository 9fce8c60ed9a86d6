"""Tides per boundary node (DGSWE_BC_NODE_TIDES, the device form of
BoundaryTides) on the device against the oracle, through the C ABI: the
RHS to TOL_RHS and a stage to TOL of each field (as the other boundary
conditions, test_gpu_parity.py), elevation only or with the tides'
velocity, with and without transport scaling, slots by node or by
position; a run of global steps and a multirate coarse step."""

import dataclasses

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.device import DeviceRun, SWEPhysics2D
from dgcom_gb300.mesh import TAG_OPEN
from oracle_lib import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_RHS = 1e-10


def rel_err(got, want):
    return max(float(np.abs(g - w).max() / max(np.abs(w).max(), 1e-300)) for g, w in zip(got, want))


def setup(numerics, velocity, ratio, by_position, order=2):
    case = cases.tidal_channel(nx=24, ny=3, order=order, numerics=numerics)
    form = case.form
    tides = cases.synthetic_node_tides(form, velocity=velocity, max_transport_ratio=ratio,
                                       by_position=by_position)
    form = dataclasses.replace(form, boundaries={**form.boundaries, TAG_OPEN: tides})
    return case, form, cases.with_flow(case, eta_amp=0.3, u=0.3, v=0.05)


@pytest.mark.parametrize("numerics", [abi.NUMERICS_FAST, abi.NUMERICS_EXACT])
@pytest.mark.parametrize("velocity,ratio", [(False, None), (True, None), (True, 2.5)])
@pytest.mark.parametrize("by_position", [False, True])
def test_rhs_and_stage_match_oracle(numerics, velocity, ratio, by_position):
    case, form, q = setup(numerics, velocity, ratio, by_position)
    dev, ref = SWEPhysics2D(form, 0), oracle(form)
    try:
        for s in (dev, ref):
            s.upload(*q)
        for t in (1800.0, 5000.0):  # during and after the ramp
            err = rel_err(dev.compute_rhs_into(t), ref.compute_rhs_into(t))
            assert err <= TOL_RHS, f"t {t}: RHS {err:.3e}"
        dt = ref.compute_dt_ssp(0.5)
        for s in (dev, ref):
            s.stage_where(base=0, input=0, out=1, time=5000.0, a=1.0, b=0.0, c=dt)
        err = rel_err(dev.download(1), ref.download(1))
        assert err <= TOL, f"stage {err:.3e}"
    finally:
        dev.close()
        ref.close()


def test_run_matches_oracle():
    case, form, q = setup(abi.NUMERICS_FAST, True, 2.5, False)
    out = []
    for sim in (SWEPhysics2D(form, 0), oracle(form)):
        try:
            sim.upload(*q)
            rep = sim.run_with_callback(DeviceRun(span=(4000.0, 4200.0), cfl=0.5))
            assert rep.success, rep.message
            out.append((sim.download(), rep.n_steps))
        finally:
            sim.close()
    (a, na), (b, nb) = out
    assert na == nb
    assert rel_err(a, b) <= 1e-10


def test_multirate_coarse_step_matches_oracle():
    case, form, q = setup(abi.NUMERICS_EXACT, True, None, False, order=3)
    out = []
    for sim in (SWEPhysics2D(form, 0), oracle(form)):
        try:
            sim.upload(*q)
            rep = sim.run_with_callback(DeviceRun(span=(4000.0, 1e9), cfl=0.5, levels=3,
                                                  max_steps=1))
            assert rep.n_steps == 1
            out.append((sim.download(), rep))
        finally:
            sim.close()
    (a, ra), (b, rb) = out
    assert ra.local_time_stepping.element_evaluations == rb.local_time_stepping.element_evaluations
    assert rel_err(a, b) <= 1e-12 * 2 ** rb.local_time_stepping.finest_level
