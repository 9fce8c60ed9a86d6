"""Local time stepping on the device (dgswe_run with run.levels > 0)
against the oracle's multirate stepper, through the C ABI.

Each coarse step starts both from the oracle's state (one coarse step per
run: max_steps = 1), so a difference cannot grow from step to step. A
coarse step of finest level L runs 2^L substeps of every stage on the
finest elements; the bar is TOL_STEP = 1e-12 × 2^L of each field's
largest value. The plans must agree exactly: the same work counts, the same
coarse step to 1e-13."""

import math

import numpy as np
import pytest

from dgcom_gb300 import abi
from dgcom_gb300.device import Cuda, DeviceRun, SWEPhysics2D
from dgcom_gb300.mesh import node_mass
from oracle_lib import oracle
from test_multirate_oracle import basin

pytestmark = pytest.mark.gpu


def rel_err(got, want):
    return max(float(np.abs(g - w).max() / max(np.abs(w).max(), 1e-300)) for g, w in zip(got, want))


def one_coarse_step(sim, state, t, levels, scheme, cfl=0.5):
    sim.upload(*state)
    rep = sim.run_with_callback(DeviceRun(span=(t, 1e9), cfl=cfl, levels=levels, max_steps=1,
                                          scheme=scheme))
    assert rep.n_steps == 1, rep.message
    return sim.download(), rep


@pytest.mark.parametrize("numerics", [abi.NUMERICS_FAST, abi.NUMERICS_EXACT])
@pytest.mark.parametrize("order,scheme", [(2, abi.SSP_RK3), (3, abi.SSP_RK3), (3, abi.SSP_RK43)])
def test_coarse_steps_match_oracle(numerics, order, scheme):
    form, q = basin(order=order)
    form.numerics = numerics
    dev, ref = SWEPhysics2D(form, 0), oracle(form)
    try:
        t = 0.0
        state = q
        finest = 0
        for step in range(4):
            got, rd = one_coarse_step(dev, state, t, 4, scheme)
            want, rr = one_coarse_step(ref, state, t, 4, scheme)
            sd, sr = rd.local_time_stepping, rr.local_time_stepping
            assert sd.finest_level == sr.finest_level, step
            assert sd.element_evaluations == sr.element_evaluations, step
            assert sd.line_local_elements == sr.line_local_elements, step
            assert abs(rd.final_time - rr.final_time) <= 1e-13 * max(rr.final_time - t, 1e-300)
            finest = max(finest, sr.finest_level)
            err = rel_err(got, want)
            assert err <= 1e-12 * 2 ** sr.finest_level, f"step {step}: {err:.3e}"
            state, t = want, rr.final_time
        assert finest >= 2
    finally:
        dev.close()
        ref.close()


def test_one_level_is_the_global_scheme_bit_for_bit():
    form, q = basin()
    dev = SWEPhysics2D(form, 0)
    try:
        dev.upload(*q)
        dt_min = float(dev.element_dt(0.5).min())
        cap = 1.5 * dt_min  # one level
        runs = []
        for levels in (0, 4):
            dev.upload(*q)
            rep = dev.run_with_callback(DeviceRun(span=(0.0, 8 * dt_min), cfl=0.5, levels=levels,
                                                  dt_max=cap))
            assert rep.success, rep.message
            runs.append((dev.download(), rep))
        (a, ra), (b, rb) = runs
        assert ra.n_steps == rb.n_steps and ra.final_time == rb.final_time
        assert rb.local_time_stepping.finest_level == 0
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    finally:
        dev.close()


def test_levels_conserve_mass_on_device():
    form, q = basin(wet_dry=False)
    form.manning_n = None
    mass = node_mass(form.mesh, form.order).reshape(-1)
    dev = SWEPhysics2D(form, 0)
    try:
        dev.upload(*q)
        rep = dev.run_with_callback(DeviceRun(span=(0.0, 60.0), cfl=0.5, levels=4))
        assert rep.success, rep.message
        s = rep.local_time_stepping
        assert s.finest_level >= 2
        assert s.element_evaluations < 0.8 * s.global_evaluations
        h = dev.download()[0]
    finally:
        dev.close()
    m0, m1 = float(mass @ q[0]), float(mass @ h)
    assert abs(m1 - m0) <= 1e-13 * m0


def test_case_device_runs_levels_to_its_callbacks():
    """CaseDevice::run_2d with DeviceRun::levels: the callbacks at the start
    and every interval, the end state in q, as the oracle's run."""
    form, q0 = basin()
    got = [x.copy() for x in q0]
    times = []
    rep = Cuda().run_2d(0, form, got, DeviceRun(span=(0.0, 50.0), cfl=0.5, interval=20.0,
                                                levels=3),
                        callback=lambda state, t: times.append(t))
    assert rep.success, rep.message
    assert times == [0.0, 20.0, 40.0]
    ref = oracle(form)
    try:
        ref.upload(*q0)
        rr = ref.run_with_callback(DeviceRun(span=(0.0, 50.0), cfl=0.5, interval=20.0, levels=3))
        want = ref.download()
    finally:
        ref.close()
    assert rep.n_steps == rr.n_steps
    assert rel_err(got, want) <= 1e-10
