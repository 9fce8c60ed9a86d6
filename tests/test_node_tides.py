"""Tides per boundary node (BoundaryTides as the device form
DeviceExternal2D::Tides) in the oracle, on the CPU: constants equal at every
node with no velocity give the uniform harmonic tide's boundary, and the
slot of a face node is the one slot_of_node gives or the nearest."""

import dataclasses
import math

import numpy as np

from dgcom_gb300 import cases
from dgcom_gb300.mesh import TAG_OPEN
from dgcom_gb300.physics import NodeTidesBoundary
from oracle_lib import oracle


def channel():
    case = cases.tidal_channel(nx=24, ny=3, order=2)
    form = case.form
    form.bathymetry = form.bathymetry - 5.0
    return case, form, cases.with_flow(case, eta_amp=0.3, u=0.3, v=0.05)


def test_uniform_constants_equal_the_harmonic_tide():
    case, form, q = channel()
    bc = form.boundaries[TAG_OPEN]
    c = bc.constituents[0]
    # η = A cos(ωt + φ) = A cos φ cos ωt − A sin φ sin ωt (f = 1, no nodal drift)
    omega = 2.0 * math.pi / c.period
    flats = cases.boundary_face_nodes(form, TAG_OPEN)
    x, y = form.positions()
    pos = np.column_stack([x.reshape(-1)[flats], y.reshape(-1)[flats]])
    coef = np.zeros((len(flats), 1, 6))
    coef[:, 0, 0] = c.amplitude * math.cos(c.phase)
    coef[:, 0, 1] = -c.amplitude * math.sin(c.phase)
    node = NodeTidesBoundary(omega=np.array([omega]), f_rate=np.zeros(1), positions=pos,
                             coefficients=coef, ramp_duration=bc.ramp_duration)
    per_node = dataclasses.replace(form, boundaries={**form.boundaries, TAG_OPEN: node})
    out = []
    for f in (form, per_node):
        ref = oracle(f)
        try:
            ref.upload(*q)
            out.append(ref.compute_rhs_into(2500.0))
        finally:
            ref.close()
    for a, b in zip(*out):
        assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()


def test_slots_by_position_equal_slots_by_node():
    case, form, q = channel()
    out = []
    for by_position in (False, True):
        tides = cases.synthetic_node_tides(form, by_position=by_position)
        f = dataclasses.replace(form, boundaries={**form.boundaries, TAG_OPEN: tides})
        ref = oracle(f)
        try:
            ref.upload(*q)
            out.append(ref.compute_rhs_into(5000.0))
        finally:
            ref.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_velocity_constants_drive_the_boundary():
    """With the tides' velocity the boundary state differs from the
    elevation-only one (the external normal velocity enters the
    characteristic)."""
    case, form, q = channel()
    out = []
    for velocity in (False, True):
        tides = cases.synthetic_node_tides(form, velocity=velocity)
        f = dataclasses.replace(form, boundaries={**form.boundaries, TAG_OPEN: tides})
        ref = oracle(f)
        try:
            ref.upload(*q)
            out.append(ref.compute_rhs_into(5000.0))
        finally:
            ref.close()
    assert np.abs(out[0][1] - out[1][1]).max() > 0.0
