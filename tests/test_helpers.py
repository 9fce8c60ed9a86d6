"""The oracle's Standard-kernel helpers (the reference's scalar forms,
src/solver/simd/kernels.rs) against the reference's own tests of them
(kernels.rs:457-535) and against a plain restatement with every product
and sum rounded in the reference's order; and the library's helper entry
points refusing bad arguments without a GPU."""

import ctypes as C

import numpy as np

from helpers_common import random_vec
from oracle_lib import oracle_library

_dp = C.POINTER(C.c_double)


def ptr(a):
    return a.ctypes.data_as(_dp)


def bind():
    lib = oracle_library().cdll
    lib.oracle_apply_diff_matrix.argtypes = [_dp] * 7 + [C.c_int64]
    lib.oracle_apply_lift.argtypes = [_dp] * 7 + [C.c_int64, C.c_int64, C.c_double]
    lib.oracle_coriolis_source.argtypes = [_dp] * 4 + [C.c_double, C.c_int64]
    lib.oracle_combine_derivatives.argtypes = [C.POINTER(_dp)] + [_dp] * 3 + [C.c_double] * 4 + [
        C.c_int64]
    return lib


def test_diff_matrix_matches_the_reference_test():
    # test_apply_diff_matrix_scalar: a 3 × 3 element, D and fluxes from the
    # generator; out_h[0] equals the row-0 sum
    lib = bind()
    n = 9
    d = random_vec(n * n, 42)
    f = [random_vec(n, s) for s in (1, 2, 3)]
    out = [np.zeros(n) for _ in range(3)]
    lib.oracle_apply_diff_matrix(ptr(d), *map(ptr, f), *map(ptr, out), n)
    expected = 0.0
    for j in range(n):
        expected += d[j] * f[0][j]
    assert abs(out[0][0] - expected) <= 1e-12 * abs(expected)
    for i in range(n):  # every row, every field, the reference's order: bit for bit
        for v in range(3):
            s = 0.0
            for j in range(n):
                s += d[i * n + j] * f[v][j]
            assert out[v][i] == s


def test_lift_matches_the_reference_test():
    lib = bind()
    n, nf = 9, 3
    lift = random_vec(n * nf, 42)
    diff = [random_vec(nf, s) for s in (1, 2, 3)]
    out = [np.ones(n) for _ in range(3)]
    lib.oracle_apply_lift(ptr(lift), *map(ptr, diff), *map(ptr, out), n, nf, 0.5)
    assert np.any(np.abs(out[0] - 1.0) > 1e-10)  # test_apply_lift_scalar
    for i in range(n):
        for v in range(3):
            s = 0.0
            for fi in range(nf):
                s += lift[i * nf + fi] * diff[v][fi]
            assert out[v][i] == 1.0 + 0.5 * s


def test_coriolis_matches_the_reference_test():
    lib = bind()
    n = 8
    hu, hv = np.ones(n), np.full(n, 2.0)
    ohu, ohv = np.zeros(n), np.zeros(n)
    lib.oracle_coriolis_source(ptr(hu), ptr(hv), ptr(ohu), ptr(ohv), 1.2e-4, n)
    assert abs(ohu[0] - 2.4e-4) <= 1e-10 and abs(ohv[0] + 1.2e-4) <= 1e-10
    assert np.all(ohu == 1.2e-4 * 2.0) and np.all(ohv == -1.2e-4 * 1.0)


def test_combine_derivatives_is_the_negative_divergence():
    lib = bind()
    n = 16
    ins = [random_vec(n, 10 + c) for c in range(12)]
    out = [np.zeros(n) for _ in range(3)]
    arr = (_dp * 12)(*map(ptr, ins))
    rx, sx, ry, sy = 0.013, -0.002, 0.004, 0.011
    lib.oracle_combine_derivatives(arr, *map(ptr, out), rx, sx, ry, sy, n)
    for v in range(3):
        for i in range(n):
            div = ins[v][i] * rx + ins[3 + v][i] * sx + ins[6 + v][i] * ry + ins[9 + v][i] * sy
            assert out[v][i] == -div


def test_library_helpers_refuse_bad_arguments_before_the_device(cuda_lib):
    from dgcom_gb300 import abi

    z = C.c_void_p(0)
    st = cuda_lib.apply_diff_matrix(0, z, z, z, z, z, z, z, 16, 4)
    assert st == abi.ERR_INVALID
    assert "NULL" in cuda_lib.helpers_last_error().decode()
    buf = np.zeros(4)
    p = C.c_void_p(buf.ctypes.data)
    assert cuda_lib.apply_diff_matrix(0, p, p, p, p, p, p, p, 65, 1) == abi.ERR_INVALID
    assert cuda_lib.apply_lift(0, p, p, p, p, p, p, p, 4, 5, p, 1) == abi.ERR_INVALID
    assert cuda_lib.coriolis_source(0, p, p, p, p, 1e-4, -1) == abi.ERR_INVALID
