"""The library's Standard-kernel helpers (dgswe_apply_diff_matrix,
dgswe_apply_lift, dgswe_coriolis_source, dgswe_combine_derivatives) on the
GPU, batched over elements, against the oracle's scalar forms of the
reference's helpers (src/solver/simd/kernels.rs) element by element: the
same bits, at the element sizes the reference's RHS bench times
(benches/rhs_swe_2d_bench.rs: 9, 16, 25 and 36 nodes)."""

import ctypes as C

import numpy as np
import pytest

from dgcom_gb300 import abi
from helpers_common import random_vec
from test_helpers import bind, ptr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
_dp = C.POINTER(C.c_double)
ELEMENTS = 3000


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0")


def vp(t):
    return C.c_void_p(t.data_ptr())


def batch(n, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.0, 1.0, n * ELEMENTS) * 10.0 ** rng.integers(-3, 4, n * ELEMENTS)


@pytest.mark.parametrize("n", [9, 16, 25, 36])
def test_diff_matrix_batched_equals_the_reference_helper(cuda_lib, n):
    ora = bind()
    d = random_vec(n * n, 42)
    f = [batch(n, s) for s in (1, 2, 3)]
    out = [torch.full((n * ELEMENTS,), float("nan"), dtype=torch.float64, device="cuda:0")
           for _ in range(3)]
    # the device copies must outlive the call: a dropped tensor's memory goes
    # back to torch's cache and the next copy would take it
    d_d, d_f = dev(d), [dev(x) for x in f]
    st = cuda_lib.apply_diff_matrix(0, vp(d_d), *map(vp, d_f), *map(vp, out), n, ELEMENTS)
    assert st == abi.OK, cuda_lib.helpers_last_error()
    got = [o.cpu().numpy() for o in out]
    want = [np.empty(n * ELEMENTS) for _ in range(3)]
    for e in range(ELEMENTS):
        s = slice(e * n, (e + 1) * n)
        views = [x[s] for x in f]
        outs = [np.empty(n) for _ in range(3)]
        ora.oracle_apply_diff_matrix(ptr(d), *map(ptr, views), *map(ptr, outs), n)
        for w, o in zip(want, outs):
            w[s] = o
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


@pytest.mark.parametrize("n", [9, 16, 25, 36])
def test_lift_batched_equals_the_reference_helper(cuda_lib, n):
    ora = bind()
    nf = int(round(n ** 0.5))
    lift = random_vec(n * nf, 42)
    diff = [batch(nf, s) for s in (4, 5, 6)]
    base = [batch(n, s) for s in (7, 8, 9)]
    scale = np.random.default_rng(3).uniform(0.1, 10.0, ELEMENTS)
    out = [dev(b) for b in base]
    d_lift, d_diff, d_scale = dev(lift), [dev(x) for x in diff], dev(scale)
    st = cuda_lib.apply_lift(0, vp(d_lift), *map(vp, d_diff), *map(vp, out), n, nf, vp(d_scale),
                             ELEMENTS)
    assert st == abi.OK, cuda_lib.helpers_last_error()
    got = [o.cpu().numpy() for o in out]
    want = [b.copy() for b in base]
    for e in range(ELEMENTS):
        s, sf = slice(e * n, (e + 1) * n), slice(e * nf, (e + 1) * nf)
        outs = [w[s].copy() for w in want]
        ora.oracle_apply_lift(ptr(lift), *[ptr(np.ascontiguousarray(x[sf])) for x in diff],
                              *map(ptr, outs), n, nf, float(scale[e]))
        for w, o in zip(want, outs):
            w[s] = o
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_coriolis_and_combine_equal_the_reference_helpers(cuda_lib):
    ora = bind()
    n = 16
    hu, hv = batch(n, 11), batch(n, 12)
    ohu, ohv = batch(n, 13), batch(n, 14)
    d_ohu, d_ohv = dev(ohu), dev(ohv)
    d_hu, d_hv = dev(hu), dev(hv)
    st = cuda_lib.coriolis_source(0, vp(d_hu), vp(d_hv), vp(d_ohu), vp(d_ohv), 1.2e-4,
                                  n * ELEMENTS)
    assert st == abi.OK, cuda_lib.helpers_last_error()
    ora.oracle_coriolis_source(ptr(hu), ptr(hv), ptr(ohu), ptr(ohv), 1.2e-4, n * ELEMENTS)
    assert np.array_equal(d_ohu.cpu().numpy(), ohu)
    assert np.array_equal(d_ohv.cpu().numpy(), ohv)

    ins = [batch(n, 20 + c) for c in range(12)]
    metric = np.random.default_rng(5).uniform(-0.02, 0.02, 4 * ELEMENTS)
    d_ins = [dev(x) for x in ins]
    arr = (C.c_void_p * 12)(*[t.data_ptr() for t in d_ins])
    out = [torch.empty(n * ELEMENTS, dtype=torch.float64, device="cuda:0") for _ in range(3)]
    d_metric = dev(metric)
    st = cuda_lib.combine_derivatives(0, arr, *map(vp, out), vp(d_metric), n, ELEMENTS)
    assert st == abi.OK, cuda_lib.helpers_last_error()
    got = [o.cpu().numpy() for o in out]
    for e in range(0, ELEMENTS, 7):
        s = slice(e * n, (e + 1) * n)
        views = [np.ascontiguousarray(x[s]) for x in ins]
        pa = (_dp * 12)(*map(ptr, views))
        outs = [np.empty(n) for _ in range(3)]
        ora.oracle_combine_derivatives(pa, *map(ptr, outs), *metric[4 * e:4 * e + 4], n)
        for g, o in zip(got, outs):
            assert np.array_equal(g[s], o)
