"""dgswe_compute_rhs_noalloc: the RHS of a state the caller already holds
on the device, computed without any allocation — for callers that cannot
call cudaMalloc while they step (a host whose own pool owns the device
budget, a loop where an allocation would synchronise or fail mid-run). Its
working memory is the library's fixed array, shared by every call.

Checked through the C ABI against dgswe_compute_rhs on the same states, on
two calls in a row (the second sees the first call's leftovers in the
shared array). Both run the same kernels on the same inputs, so the results
must be the same bits. The device's free memory and torch's allocator are
read around each call: nothing may change, except that the first call may
make the library's module resident (its fixed array, at most 64 MiB plus
the loader's rounding) where the CUDA runtime loads modules lazily.

This file is collected last, so a run that stops at the first failure has
run every other test before it."""

import ctypes as C
import dataclasses

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.device import SWEPhysics2D
from dgcom_gb300.mesh import TAG_OPEN

pytestmark = pytest.mark.gpu

ARRAY_BYTES = 64 << 20
LOADER_SLACK = 8 << 20


def _call(lib, dev, d_in, d_out, t, n):
    return lib.compute_rhs_noalloc(dev.handle, *(C.c_void_p(x.data_ptr()) for x in d_in), t,
                                   *(C.c_void_p(x.data_ptr()) for x in d_out), n)


def test_noalloc_rhs_matches_compute_rhs_twice_and_allocates_nothing():
    torch = pytest.importorskip("torch")
    case = cases.tidal_channel(nx=40, ny=8, order=3)
    dev = SWEPhysics2D(case.form, 0)
    lib = dev.lib
    n = dev.n_values
    states = [cases.with_flow(case), cases.with_flow(case, eta_amp=0.2, u=-0.4, v=0.15)]
    times = [0.0, 900.0]
    try:
        for call, (q, t) in enumerate(zip(states, times)):
            dev.upload(*q)
            want = dev.compute_rhs_into(t)
            d_in = [torch.from_numpy(np.ascontiguousarray(x)).to("cuda:0") for x in q]
            d_out = [torch.full((n,), float("nan"), dtype=torch.float64, device="cuda:0")
                     for _ in range(3)]
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info(0)[0]
            held0 = torch.cuda.memory_allocated(0)
            status = _call(lib, dev, d_in, d_out, t, n)
            assert status == abi.OK, lib.error_text(dev.handle, status)
            torch.cuda.synchronize()
            free1 = torch.cuda.mem_get_info(0)[0]
            assert torch.cuda.memory_allocated(0) == held0
            if call == 0:
                assert 0 <= free0 - free1 <= ARRAY_BYTES + LOADER_SLACK, (free0, free1)
            else:
                assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
            got = [x.cpu().numpy() for x in d_out]
            for g, w in zip(got, want):
                assert np.array_equal(g, w), (
                    f"call {call}: {np.count_nonzero(g != w)} values differ, "
                    f"largest by {np.nanmax(np.abs(g - w)):.3e}")
    finally:
        dev.close()


def test_noalloc_refuses_a_mesh_beyond_its_array():
    torch = pytest.importorskip("torch")
    # 120,000 elements at N = 3 need 76.8 MB, more than the 64 MiB array
    case = cases.coastal_box(n_elements=120_000, order=3)
    dev = SWEPhysics2D(case.form, 0)
    lib = dev.lib
    n = dev.n_values
    try:
        buf = torch.zeros(n, dtype=torch.float64, device="cuda:0")
        p = C.c_void_p(buf.data_ptr())
        status = lib.compute_rhs_noalloc(dev.handle, p, p, p, 0.0, p, p, p, n)
        assert status == abi.ERR_INVALID
        assert "working memory" in lib.error_text(dev.handle, status)
    finally:
        dev.close()


def test_noalloc_refuses_a_time_outside_the_forcing_snapshots():
    torch = pytest.importorskip("torch")
    case = cases.tidal_channel(nx=24, ny=3, order=2)
    parent = cases.synthetic_parent(case.form, t0=0.0, t1=43_200.0)
    form = dataclasses.replace(case.form, boundaries={**case.form.boundaries, TAG_OPEN: parent})
    dev = SWEPhysics2D(form, 0)
    lib = dev.lib
    n = dev.n_values
    try:
        q = cases.with_flow(case)
        d_in = [torch.from_numpy(np.ascontiguousarray(x)).to("cuda:0") for x in q]
        d_out = [torch.zeros(n, dtype=torch.float64, device="cuda:0") for _ in range(3)]
        torch.cuda.synchronize()
        status = _call(lib, dev, d_in, d_out, 50_000.0, n)
        assert status == abi.ERR_INVALID
        assert "snapshots" in lib.error_text(dev.handle, status)
        # inside the snapshots it is the handle's RHS
        dev.upload(*q)
        want = dev.compute_rhs_into(9000.5)
        status = _call(lib, dev, d_in, d_out, 9000.5, n)
        assert status == abi.OK, lib.error_text(dev.handle, status)
        for g, w in zip(d_out, want):
            assert np.array_equal(g.cpu().numpy(), w)
    finally:
        dev.close()
