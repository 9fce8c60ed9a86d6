"""The LocalTimeStepping pass entry points (dgswe_begin_coarse_step,
dgswe_stage_where, dgswe_finish_where, dgswe_depth_flags): coarse steps
planned on the host and taken pass by pass, as the reference's own
MultirateStepper drives its device backend (src/time/multirate.rs:1160-1331,
gpu/src/swe2d.rs:4403-4660), equal bit for bit to the library's own
multirate run, and to the oracle within the per-step tolerance."""

import numpy as np
import pytest

from dgcom_gb300 import abi
from dgcom_gb300.device import DeviceError, DeviceRun, SWEPhysics2D
from dgcom_gb300.multirate import HostStepper
from oracle_lib import oracle
from test_multirate_oracle import basin

pytestmark = pytest.mark.gpu


def host_steps(form, q, levels, scheme, n_steps, cfl=0.5, dt_max=None):
    dev = SWEPhysics2D(form, 0)
    stepper = HostStepper(dev, levels, scheme)
    try:
        dev.upload(*q)
        stepper.start()
        t, finest = 0.0, []
        for _ in range(n_steps):
            t, plan = stepper.step(t, 1e9, cfl, dt_max)
            finest.append(plan.finest)
        return dev.download(), t, finest
    finally:
        stepper.close()
        dev.close()


def library_run(sim, q, levels, scheme, n_steps, cfl=0.5, dt_max=None):
    try:
        sim.upload(*q)
        rep = sim.run_with_callback(DeviceRun(span=(0.0, 1e9), cfl=cfl, levels=levels,
                                              scheme=scheme, max_steps=n_steps, dt_max=dt_max))
        assert rep.n_steps == n_steps, rep.message
        return sim.download(), rep
    finally:
        sim.close()


@pytest.mark.parametrize("scheme", [abi.SSP_RK3, abi.SSP_RK43])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_host_planned_passes_are_the_library_run(scheme, order):
    form, q = basin(order=order)
    got, t, finest = host_steps(form, q, 4, scheme, 3)
    want, rep = library_run(SWEPhysics2D(form, 0), q, 4, scheme, 3)
    assert max(finest) >= 2, finest  # the basin spreads its elements over levels
    assert t == rep.final_time
    for a, b in zip(got, want):
        assert np.array_equal(a, b)


def test_host_planned_passes_against_the_oracle():
    form, q = basin(order=2)
    got, _, finest = host_steps(form, q, 4, abi.SSP_RK3, 2, dt_max=40.0)
    want, _ = library_run(oracle(form), q, 4, abi.SSP_RK3, 2, dt_max=40.0)
    scale = 2 ** max(finest)
    for a, b in zip(got, want):
        assert np.abs(a - b).max() <= 1e-12 * scale * max(np.abs(b).max(), 1e-300)


def test_depth_flags_are_the_nodes_depths():
    form, q = basin(order=2)
    dev = SWEPhysics2D(form, 0)
    try:
        dev.upload(*q)
        d = (1.0, 5.0, 0.0)
        flags = dev.depth_flags(*d)
        h = q[0].reshape(form.mesh.n_elements, -1)
        want = sum((np.all(h > di, axis=1).astype(np.uint8) << i) for i, di in enumerate(d))
        assert np.array_equal(flags, want)
        assert np.array_equal(dev.depth_flags(np.inf, -np.inf, 0.0) & 3,
                              np.full(form.mesh.n_elements, 2, np.uint8))
    finally:
        dev.close()


def test_passes_check_their_arguments():
    form, q = basin(order=2)
    dev = SWEPhysics2D(form, 0)
    try:
        dev.upload(*q)
        plan = abi.MultirateStage(0.0, 1.0, 0, 0, 0, 0, 0, 1.0, 0.0, 1.0, 0.0, 0, 0, 1, 0)
        with pytest.raises(DeviceError):  # no coarse step begun
            dev.multirate_stage(plan)
        K = form.mesh.n_elements
        levels = np.zeros(K, np.uint8)
        levels[: K // 2] = 1
        rates = np.tile(levels, (3, 1))
        rates[0, 0] = 0  # a rate below its element's level
        with pytest.raises(DeviceError):
            dev.begin_coarse_step(levels, rates)
        rates[0, 0] = 1
        dev.begin_coarse_step(levels, rates)
        with pytest.raises(DeviceError):  # finest is 1
            dev.multirate_stage(plan)
        plan.finest = 1
        plan.out = plan.input_buffer  # the stage would overwrite its input
        with pytest.raises(DeviceError):
            dev.multirate_stage(plan)
        with pytest.raises(DeviceError):
            dev.multirate_finish(0, 0)  # the sums cannot be the state
    finally:
        dev.close()
