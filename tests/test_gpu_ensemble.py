"""The ensemble driver through the C ABI: every member of a batched run
equals a run of that member alone (the single-mesh path, itself held to the
oracle by the parity tests), bit for bit, with mixed orders, a drying
channel and per-member Manning coefficients and tides."""

import ctypes as C

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.device import SWEPhysics2D
from dgcom_gb300.ensemble import Ensemble

pytestmark = pytest.mark.gpu

STEPS = 6
CFL = 0.5


def members(numerics):
    ms = cases.ensemble_members(4, seed=11, k_range=(60, 400), numerics=numerics)
    channel = cases.tidal_channel(nx=24, ny=4, order=3, numerics=numerics)  # a drying flat
    channel.form.coriolis_f0 = ms[0].form.coriolis_f0  # the physics options are shared
    ms.append(channel)
    return ms


def alone(form, state, steps, t_start=0.0):
    """``steps`` device-driven steps of one member on its own handle."""
    dev = SWEPhysics2D(form, 0)
    dev.upload(*state)
    cfg = abi.RunConfig()
    cfg.scheme = abi.SSP_RK3
    cfg.cfl = CFL
    cfg.t_start = t_start
    cfg.t_end = 1e300
    prof = abi.Profile()
    st = dev.lib.profile_steps(dev.handle, C.byref(cfg), steps, C.byref(prof))
    assert st == abi.OK, dev.lib.error_text(dev.handle, st)
    out = dev.download()
    dev.close()
    return out, prof.t_final


@pytest.mark.parametrize("numerics", [abi.NUMERICS_FAST, abi.NUMERICS_EXACT])
def test_members_equal_their_single_runs(numerics):
    ms = members(numerics)
    assert {c.form.order for c in ms} == {2, 3}
    states = [cases.with_flow(c) for c in ms]
    with Ensemble([c.form for c in ms]) as ens:
        assert ens.n_members == len(ms)
        for i, s in enumerate(states):
            assert ens.n_values(i) == s[0].size
            ens.upload(i, *s)
        reports, prof = ens.run(STEPS, CFL)
        assert prof.steps == STEPS and prof.total_ms > 0.0
        for i, c in enumerate(ms):
            want, t_want = alone(c.form, states[i], STEPS)
            got = ens.download(i)
            assert reports[i].success and reports[i].n_steps == STEPS
            assert reports[i].final_time == t_want
            for g, w in zip(got, want):
                assert np.array_equal(g, w), f"member {i}: max diff {np.abs(g - w).max()}"
            assert got[0].min() >= 0.0


def test_members_take_their_own_steps():
    ms = members(abi.NUMERICS_FAST)
    with Ensemble([c.form for c in ms]) as ens:
        for i, c in enumerate(ms):
            ens.upload(i, *cases.with_flow(c))
        reports, _ = ens.run(2, CFL)
    times = [r.final_time for r in reports]
    assert len(set(times)) == len(times)  # different meshes, different CFL steps
    assert all(r.dt_min > 0.0 and r.dt_max >= r.dt_min for r in reports)


def test_two_runs_continue_like_one():
    ms = members(abi.NUMERICS_FAST)[2:]
    states = [cases.with_flow(c) for c in ms]
    with Ensemble([c.form for c in ms]) as ens:
        for i, s in enumerate(states):
            ens.upload(i, *s)
        ens.run(2, CFL)
        reports, _ = ens.run(2, CFL, t_start=float("nan"))  # each member from its own time
        for i, c in enumerate(ms):
            want, t_want = alone(c.form, states[i], 4)
            assert reports[i].final_time == t_want
            assert all(np.array_equal(g, w) for g, w in zip(ens.download(i), want))


def test_mixed_order_members_match_the_oracle():
    """Each member of a batched run of mixed orders (two coastal boxes of
    order 2 and 3, and a drying channel of order 3) against the oracle
    stepping that member alone: every step from the same state, the
    member's own time step to 1e-13 and its state to 1e-12 of each field's
    largest value."""
    from oracle_lib import oracle

    ms = members(abi.NUMERICS_FAST)
    assert {c.form.order for c in ms} == {2, 3}
    states = [cases.with_flow(c) for c in ms]
    refs = [oracle(c.form) for c in ms]
    t = [0.0] * len(ms)
    try:
        with Ensemble([c.form for c in ms]) as ens:
            for i, s in enumerate(states):
                ens.upload(i, *s)
                refs[i].upload(*s)
            for step in range(5):
                reports, _ = ens.run(1, CFL, t_start=0.0 if step == 0 else float("nan"))
                for i, ref in enumerate(refs):
                    dt = ref.compute_dt_ssp(CFL)
                    ref.step(t[i], dt)
                    t[i] += dt
                    assert abs(reports[i].final_time - t[i]) <= 1e-13 * t[i], (i, step)
                    got, want = ens.download(i), ref.download()
                    for g, w in zip(got, want):
                        err = np.abs(g - w).max() / max(np.abs(w).max(), 1e-300)
                        assert err <= 1e-12, f"member {i} (order {ms[i].form.order}), step {step}: {err:.3e}"
                    ens.upload(i, *want)
    finally:
        for r in refs:
            r.close()
