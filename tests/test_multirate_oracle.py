"""Local time stepping in the oracle (its restatement of MultirateStepper
and SWEPhysics2D's element passes), on the CPU: the properties the
reference's module documentation states and its tests check
(src/time/multirate.rs:1-120, tests/local_time_stepping_test.rs):

- one level is the base scheme, bit for bit;
- mass is conserved to rounding across level interfaces (every face's
  flux at a finest substep and stage is the same from both sides);
- a run lands on its callback times exactly, with equal coarse steps;
- the levels save element evaluations against global steps at the finest
  level.

The oracle is test infrastructure; the GPU tests hold the device's
multirate runs to it."""

import math

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.device import DeviceRun
from dgcom_gb300.mesh import TAG_WALL, graded_jittered_box, node_mass
from dgcom_gb300.physics import SWEDeviceForm2D, WallBoundary
from oracle_lib import oracle


def basin(order=2, n=(12, 10), seed=5, wet_dry=True):
    """A closed, graded basin (walls) over a bed from 40 m to 2 m deep:
    element steps spread over several powers of two."""
    mesh = graded_jittered_box(4000.0, 3000.0, n[0], n[1], size_range=(120.0, 500.0), jitter=0.2,
                               seed=seed, sides=(TAG_WALL,) * 4)
    form = SWEDeviceForm2D(mesh=mesh, order=order)
    x, y = form.positions()
    form.bathymetry = -(2.0 + 38.0 * (x / 4000.0) ** 2 * (1.0 + 0.3 * np.sin(y / 500.0)))
    form.boundaries = {TAG_WALL: WallBoundary()}
    form.wet_dry = wet_dry
    form.manning_n = 0.02
    b = form.bathymetry.reshape(-1)
    eta = 0.3 * np.cos(2.0 * math.pi * x.reshape(-1) / 4000.0)
    h = np.maximum(eta - b, 0.0)
    return form, (h, 0.2 * h, -0.1 * h)


def run(form, state, levels, span, interval=None, dt_max=None, cfl=0.5):
    ref = oracle(form)
    try:
        ref.upload(*state)
        times = []
        rep = ref.run_with_callback(DeviceRun(span=span, cfl=cfl, levels=levels,
                                              interval=interval, dt_max=dt_max),
                                    lambda t, *q: times.append(t))
        return ref.download(), rep, times
    finally:
        ref.close()


def test_one_level_is_the_base_scheme_bit_for_bit():
    form, q = basin()
    ref = oracle(form)
    try:
        ref.upload(*q)
        dt_min = float(ref.element_dt(0.5).min())
    finally:
        ref.close()
    # a cap below twice the smallest step leaves one level
    cap = 1.5 * dt_min
    a, ra, _ = run(form, q, 0, (0.0, 6 * dt_min), dt_max=cap)
    b, rb, _ = run(form, q, 4, (0.0, 6 * dt_min), dt_max=cap)
    assert ra.n_steps == rb.n_steps and ra.final_time == rb.final_time
    assert rb.local_time_stepping.finest_level == 0
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_levels_conserve_mass_and_save_evaluations():
    form, q = basin(wet_dry=False)
    form.manning_n = None
    mass = node_mass(form.mesh, form.order).reshape(-1)
    out, rep, _ = run(form, q, 4, (0.0, 60.0))
    assert rep.success
    stats = rep.local_time_stepping
    assert stats.finest_level >= 2
    assert stats.element_evaluations < 0.8 * stats.global_evaluations
    m0, m1 = float(mass @ q[0]), float(mass @ out[0])
    assert abs(m1 - m0) <= 1e-13 * m0


def test_a_run_lands_on_its_callback_times():
    form, q = basin()
    _, rep, times = run(form, q, 3, (0.0, 50.0), interval=20.0)
    assert rep.success
    # the callbacks at the start and every interval (runner.rs:463-470)
    assert times == [0.0, 20.0, 40.0]
    assert rep.final_time == 50.0


@pytest.mark.parametrize("scheme", [abi.SSP_RK3, abi.SSP_RK43])
def test_levels_follow_the_element_steps(scheme):
    """Each coarse step's evaluations lie between the ideal (every element
    at its own stable step) and global steps at the finest level."""
    form, q = basin(order=3)
    ref = oracle(form)
    try:
        ref.upload(*q)
        rep = ref.run_with_callback(DeviceRun(span=(0.0, 40.0), cfl=0.5, levels=4, scheme=scheme))
    finally:
        ref.close()
    s = rep.local_time_stepping
    assert rep.success and s.steps > 0
    assert s.ideal_evaluations <= s.level_evaluations <= s.element_evaluations
    assert s.element_evaluations <= s.global_evaluations
    assert s.model_seconds == pytest.approx(40.0, rel=1e-12)
