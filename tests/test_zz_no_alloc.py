"""dgswe_compute_rhs_noalloc: the RHS of a state the caller already holds
on the device, computed without any allocation — for callers that cannot
call cudaMalloc while they step (a host whose own pool owns the device
budget, a loop where an allocation would synchronise or fail mid-run). Its
working memory is the library's fixed array, shared by every call.

Checked through the C ABI against dgswe_compute_rhs on the same states, at
the tolerance the RHS tests use, on two calls in a row (the second sees the
first call's leftovers in the shared array)."""

import ctypes as C

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.device import SWEPhysics2D

pytestmark = pytest.mark.gpu

TOL_RHS = 1e-10


def test_noalloc_rhs_matches_compute_rhs_twice():
    torch = pytest.importorskip("torch")
    case = cases.tidal_channel(nx=40, ny=8, order=3)
    dev = SWEPhysics2D(case.form, 0)
    lib = dev.lib
    n = dev.n_values
    states = [cases.with_flow(case), cases.with_flow(case, eta_amp=0.2, u=-0.4, v=0.15)]
    times = [0.0, 900.0]
    try:
        for q, t in zip(states, times):
            dev.upload(*q)
            want = dev.compute_rhs_into(t)
            d_in = [torch.from_numpy(np.ascontiguousarray(x)).to("cuda:0") for x in q]
            d_out = [torch.full((n,), float("nan"), dtype=torch.float64, device="cuda:0")
                     for _ in range(3)]
            torch.cuda.synchronize()
            status = lib.compute_rhs_noalloc(
                dev.handle, *(C.c_void_p(x.data_ptr()) for x in d_in), t,
                *(C.c_void_p(x.data_ptr()) for x in d_out), n)
            assert status == abi.OK, lib.error_text(dev.handle, status)
            got = [x.cpu().numpy() for x in d_out]
            for g, w in zip(got, want):
                assert np.all(np.isfinite(g))
                err = np.abs(g - w).max() / max(np.abs(w).max(), 1e-300)
                assert err <= TOL_RHS, f"relative difference {err:.3e}"
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
