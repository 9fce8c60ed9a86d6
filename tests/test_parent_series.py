"""A parent model's series as boundary data (OceanModelState's device
form) in the oracle, on the CPU: the time stencil holds the reference's own
known answers (src/io/field_series.rs:187-223), and the boundary flux of a
parent at a snapshot time and at rest equals the uniform-elevation one."""

import ctypes as C
import dataclasses

import numpy as np
import pytest

from dgcom_gb300 import cases
from dgcom_gb300.mesh import TAG_OPEN
from oracle_lib import oracle, oracle_library

_dp = C.POINTER(C.c_double)


def stencil(times, t, cubic):
    lib = oracle_library()
    tt = np.ascontiguousarray(times, dtype=np.float64)
    idx = np.zeros(4, dtype=np.int64)
    w = np.zeros(4)
    n = lib.time_stencil(tt.ctypes.data_as(_dp), tt.size, t, 1 if cubic else 0,
                         idx.ctypes.data_as(C.POINTER(C.c_int64)), w.ctypes.data_as(_dp))
    return list(zip(idx[:n].tolist(), w[:n].tolist()))


def test_linear_stencil_brackets_without_clamping():
    times = [0.0, 10.0, 30.0]
    assert stencil(times, 20.0, False) == [(1, 0.5), (2, 0.5)]
    assert stencil(times, 30.0, False) == [(2, 1.0)]
    assert stencil(times, -1e-9, False) == []
    assert stencil(times, 30.1, True) == []
    assert len(stencil([5.0], 1e9, True)) == 1


def test_cubic_stencil_is_exact_for_polynomials():
    times = [0.0, 1.0, 2.5, 3.0, 5.0, 6.0]

    def cubic(t):
        return 1.0 - 2.0 * t + 0.3 * t * t - 0.05 * t * t * t

    def quadratic(t):
        return 1.0 - 2.0 * t + 0.3 * t * t

    for t in (1.2, 2.0, 2.9, 4.1):
        s = stencil(times, t, True)
        assert len(s) == 4
        assert abs(sum(w * cubic(times[k]) for k, w in s) - cubic(t)) < 1e-12
    for t in (0.4, 5.5):
        s = stencil(times, t, True)
        assert len(s) == 3
        assert abs(sum(w * quadratic(times[k]) for k, w in s) - quadratic(t)) < 1e-12


@pytest.mark.parametrize("cubic", [False, True])
def test_a_still_parent_is_the_still_boundary(cubic):
    """A parent at rest at level 0 without a datum shift gives the boundary
    of still water at level 0: the uniform tide with no constituents."""
    case = cases.tidal_channel(nx=24, ny=3, order=2)
    form = case.form
    form.bathymetry = form.bathymetry - 5.0
    q = cases.with_flow(case, eta_amp=0.3, u=0.3, v=0.05)
    parent = cases.synthetic_parent(form, cubic=cubic, reference_level=0.0, velocity=False)
    parent.values[:] = 0.0
    still = dataclasses.replace(form.boundaries[TAG_OPEN], constituents=[])
    out = []
    for bc in (still, parent):
        f = dataclasses.replace(form, boundaries={**form.boundaries, TAG_OPEN: bc})
        ref = oracle(f)
        try:
            ref.upload(*q)
            out.append(ref.compute_rhs_into(4321.0))
        finally:
            ref.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def nested(momentum_only=False, cubic=True):
    case = cases.tidal_channel(nx=24, ny=3, order=2)
    form = case.form
    form.bathymetry = form.bathymetry - 5.0
    q = cases.with_flow(case, eta_amp=0.3, u=0.3, v=0.05)
    parent, band = cases.synthetic_nesting(form, band_width=6000.0, cubic=cubic,
                                           momentum_only=momentum_only)
    form = dataclasses.replace(form, boundaries={**form.boundaries, TAG_OPEN: parent})
    return form, band, q


def rhs(form, q, t=9000.5):
    ref = oracle(form)
    try:
        ref.upload(*q)
        return ref.compute_rhs_into(t)
    finally:
        ref.close()


def test_a_band_of_zero_weight_changes_nothing():
    form, band, q = nested()
    base = rhs(form, q)
    zero = dataclasses.replace(band, weight=np.zeros_like(band.weight))
    for a, b in zip(base, rhs(dataclasses.replace(form, relaxation=zero), q)):
        assert np.array_equal(a, b)
    relaxed = rhs(dataclasses.replace(form, relaxation=band), q)
    assert np.abs(relaxed[1] - base[1]).max() > 0.0


def test_momentum_only_keeps_the_mass():
    form, band, q = nested(momentum_only=True)
    base = rhs(form, q)
    relaxed = rhs(dataclasses.replace(form, relaxation=band), q)
    assert np.array_equal(base[0], relaxed[0])
    assert np.abs(relaxed[1] - base[1]).max() > 0.0
