"""dgswe_step_host: one step of a state held on the host, copied in and out
in element chunks beside the compute, against the same step taken call by
call (dgswe_upload, dgswe_element_dt, dgswe_step, dgswe_download): the
same bits and the same step, for both schemes and both numerics, on the
coastal box from rest and flowing, over several steps in a row."""

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.device import DeviceError, SWEPhysics2D

pytestmark = pytest.mark.gpu


def pinned(a):
    torch = pytest.importorskip("torch")
    out = torch.empty(a.size, dtype=torch.float64, pin_memory=True).numpy()
    out[:] = a
    return out


@pytest.mark.parametrize("numerics", [abi.NUMERICS_FAST, abi.NUMERICS_EXACT])
@pytest.mark.parametrize("scheme", [abi.SSP_RK3, abi.SSP_RK43])
@pytest.mark.parametrize("flowing", [False, True])
def test_step_host_equals_the_calls_it_replaces(numerics, scheme, flowing):
    case = cases.coastal_box(20_000, numerics=numerics)
    q0 = cases.with_flow(case) if flowing else case.state
    t0 = 7200.0 if flowing else 0.0
    a, b = SWEPhysics2D(case.form, 0), SWEPhysics2D(case.form, 0)
    try:
        host = [pinned(x) for x in q0]
        b.upload(*q0)
        t = t0
        for _ in range(4):
            dt = a.step_host(t, case.cfl, *host, scheme=scheme)
            want_dt = b.compute_dt_ssp(case.cfl, scheme)
            assert dt == want_dt
            b.step(t, want_dt, scheme)
            want = b.download()
            for g, w in zip(host, want):
                assert np.array_equal(g, w)
            for g, w in zip(a.download(), want):  # the handle's state holds it too
                assert np.array_equal(g, w)
            t += dt
    finally:
        a.close()
        b.close()


def test_step_host_caps_the_step_and_refuses_bad_arrays():
    case = cases.tidal_channel(nx=40, ny=4)
    dev = SWEPhysics2D(case.form, 0)
    try:
        q = [np.ascontiguousarray(x) for x in cases.with_flow(case)]
        dev.upload(*q)
        free = dev.compute_dt_ssp(case.cfl)
        dt = dev.step_host(0.0, case.cfl, *q, dt_max=0.25 * free)
        assert dt == 0.25 * free
        with pytest.raises(ValueError):
            dev.step_host(0.0, case.cfl, q[0][::2], q[1][::2], q[2][::2])
        with pytest.raises(DeviceError):
            dev.step_host(0.0, -1.0, *q)
    finally:
        dev.close()


@pytest.mark.parametrize("nx,ny", [(3, 2), (9, 1), (40, 4)])
def test_step_host_on_meshes_of_fewer_elements_than_chunks_and_more(nx, ny):
    """Meshes of 6, 9 and 160 elements: chunks left empty, chunks of one
    element, and every element's dt and every face's flux taken as its
    chunk arrives; the same bits as the call-by-call step."""
    case = cases.tidal_channel(nx=nx, ny=ny)
    q0 = cases.with_flow(case)
    a, b = SWEPhysics2D(case.form, 0), SWEPhysics2D(case.form, 0)
    try:
        host = [np.ascontiguousarray(x) for x in q0]
        b.upload(*q0)
        t = 0.0
        for _ in range(3):
            dt = a.step_host(t, case.cfl, *host)
            want_dt = b.compute_dt_ssp(case.cfl)
            assert dt == want_dt
            b.step(t, want_dt)
            for g, w in zip(host, b.download()):
                assert np.array_equal(g, w)
            t += dt
    finally:
        a.close()
        b.close()
