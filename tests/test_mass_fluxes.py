"""The RHS's mass fluxes (compute_rhs_swe_2d_mass_fluxes_into,
src/solver/rhs/swe_2d.rs:1017-1088) in the oracle, held to the reference's
own tests of them (swe_2d.rs:2267-2365, 2640-2775): the outputs leave the
RHS unchanged bit for bit; every face slot is written and every element
balances, ∫_K dh/dt = −∮_K F*_h, for both split forms with a dry region;
in every element that takes the subcells the interface and face mass
fluxes give dh/dt node by node (subcell_divergence_element), on rectangles
and on distorted quads, orders 1 to 3, and every other element's slots are
NaN. ``mass_flux_checks`` runs the same checks on any physics with the
ABI (the GPU tests give it the CUDA library)."""

from __future__ import annotations

import math

import numpy as np
import pytest

from dgcom_gb300 import abi
from dgcom_gb300.mesh import (TAG_WALL, QuadMesh, gll_nodes, gll_weights, node_mass,
                              node_positions, uniform_rectangle)
from dgcom_gb300.physics import SWEDeviceForm2D, WallBoundary
from oracle_lib import oracle, oracle_library

G = 10.0
TAU = 2.0 * math.pi


def face_sj(mesh: QuadMesh, order: int) -> np.ndarray:
    """|∂x/∂r| or |∂x/∂s| of the bilinear map at every face node, [K][4][N+1]
    (faces 0, 1, 2, 3 at s = −1, r = +1, s = +1, r = −1; faces 2 and 3 in
    reverse)."""
    x = gll_nodes(order)
    c = mesh.corners()  # [K][4][2]
    n1 = order + 1
    out = np.empty((mesh.n_elements, 4, n1))
    for face in range(4):
        for fi in range(n1):
            t = x[fi] if face < 2 else x[n1 - 1 - fi]
            r, s = [(t, -1.0), (1.0, t), (t, 1.0), (-1.0, t)][face]
            if face in (0, 2):
                d = 0.25 * (-(1 - s) * c[:, 0] + (1 - s) * c[:, 1] + (1 + s) * c[:, 2] - (1 + s) * c[:, 3])
            else:
                d = 0.25 * (-(1 - r) * c[:, 0] - (1 + r) * c[:, 1] + (1 + r) * c[:, 2] + (1 - r) * c[:, 3])
            out[:, face, fi] = np.hypot(d[:, 0], d[:, 1])
    return out


def setup(order, formulation, distorted=False, subcell_depth=1e-3, bed=lambda x, y: -1.0 + 2.0 * x):
    """The reference's test setups: the unit square in 4 × 4 quads (bumped
    for the distorted mesh), walls, g = 10, a bed rising to the east, η =
    0.2 + 0.05 sin 2πx over it and a rotational current."""
    mesh = uniform_rectangle(0.0, 1.0, 0.0, 1.0, 4, 4)
    if distorted:
        v = mesh.vertices.copy()
        bump = np.sin(TAU * v[:, 0]) * np.sin(TAU * v[:, 1])
        v[:, 0] += 0.06 * bump
        v[:, 1] -= 0.04 * bump
        mesh = QuadMesh(v, mesh.elements, mesh.periodic, mesh.face_tags)
    form = SWEDeviceForm2D(mesh=mesh, order=order, g=G, formulation=formulation,
                           subcell_depth=subcell_depth, wet_dry=False, positivity_h_dry=None,
                           boundaries={TAG_WALL: WallBoundary()})
    x, y = node_positions(mesh, order)
    b = bed(x, y)
    form.bathymetry = b
    eta = 0.2 + 0.05 * np.sin(TAU * x)
    h = np.maximum(eta - b, 0.0)
    u, v = 0.2 * np.cos(0.5 * TAU * y), 0.1 * np.sin(0.5 * TAU * x)
    return form, (h.reshape(-1), (h * u).reshape(-1), (h * v).reshape(-1))


def mass_flux_checks(make, form, q, subcell_depth=None):
    """The reference's checks of the mass fluxes on the physics ``make``
    builds; returns (rhs, face, subcell) for further comparisons."""
    sim = make(form)
    try:
        sim.upload(*q)
        plain = sim.compute_rhs_into(0.0)
        rhs, face, sub = sim.compute_rhs_mass_fluxes_into(0.0)
    finally:
        sim.close()
    for a, b in zip(rhs, plain):
        assert np.array_equal(a, b), "the mass flux outputs changed the RHS"
    assert np.isfinite(face).all(), "face slots not all written"
    n1 = form.order + 1
    nn = n1 * n1
    k_count = form.mesh.n_elements
    # ∫_K dh/dt = −∮_K F*_h
    volume = (node_mass(form.mesh, form.order).reshape(k_count, nn)
              * rhs[0].reshape(k_count, nn)).sum(axis=1)
    w = gll_weights(form.order)
    wf = np.stack([w, w, w[::-1], w[::-1]])
    outflow = (face_sj(form.mesh, form.order) * face * wf[None]).sum(axis=(1, 2))
    max_inflow = np.maximum.accumulate(np.abs(outflow))
    bound = 1e-12 * np.maximum(max_inflow, 1e-3)
    assert (np.abs(volume + outflow) < bound).all(), np.abs(volume + outflow).max()
    if subcell_depth is not None:
        lib = oracle_library()
        probe = oracle(form)
        try:
            hh = q[0].reshape(k_count, nn)
            hu, hv = q[1].reshape(k_count, nn), q[2].reshape(k_count, nn)
            dh = rhs[0].reshape(k_count, nn)
            n_sub, largest = 0, 0.0
            div = np.empty(nn)
            for k in range(k_count):
                if not (hh[k] < subcell_depth).any():
                    assert np.isnan(sub[k]).all(), f"element {k}"
                    continue
                assert np.isfinite(sub[k]).all(), f"element {k}"
                n_sub += 1
                status = lib.subcell_divergence(
                    probe.handle, k, *(np.ascontiguousarray(a).ctypes.data_as(
                        lib.subcell_divergence.argtypes[2]) for a in (hu[k], hv[k], sub[k],
                                                                       face[k].reshape(-1))),
                    div.ctypes.data_as(lib.subcell_divergence.argtypes[2]))
                assert status == abi.OK
                scale = max(1e-3, np.abs(div).max(), np.abs(dh[k]).max())
                largest = max(largest, float(np.abs(div + dh[k]).max() / scale))
            assert n_sub >= 4, "test regime: subcell elements"
            assert largest < 1e-12, f"dh/dt + div = {largest:.2e}"
        finally:
            probe.close()
    return rhs, face, sub


@pytest.mark.parametrize("formulation", [abi.ENTROPY_STABLE, abi.WET_DRY])
def test_face_mass_flux_balances_each_element(formulation):
    form, q = setup(2, formulation)
    mass_flux_checks(oracle, form, q)


@pytest.mark.parametrize("distorted", [False, True])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_subcell_mass_fluxes_give_the_mass_tendency_node_by_node(distorted, order):
    form, q = setup(order, abi.WET_DRY, distorted, subcell_depth=0.1,
                    bed=lambda x, y: -1.0 + 2.0 * x + 0.2 * y)
    mass_flux_checks(oracle, form, q, subcell_depth=0.1)
