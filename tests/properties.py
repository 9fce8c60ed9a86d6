"""The reference's own property tests of the split-form RHS
(src/solver/rhs/swe_2d_split_form.rs:1241-1700), restated against any
physics with the ABI (the oracle, or the CUDA library): ``make(form)`` gives
an object with upload / compute_rhs_into."""

from __future__ import annotations

import math

import numpy as np

from dgcom_gb300 import abi, cases
from dgcom_gb300.mesh import node_mass, uniform_periodic, uniform_rectangle, TAG_WALL
from dgcom_gb300.physics import SWEDeviceForm2D, WallBoundary

G = 9.81
SPLIT_FORMS = [abi.ENTROPY_CONSERVATIVE, abi.ENTROPY_STABLE, abi.WET_DRY]
BEDS = ["smooth", "cell_average", "rough"]


def rhs_of(make, form, q, time=0.0):
    s = make(form)
    try:
        s.upload(*q)
        return s.compute_rhs_into(time)
    finally:
        s.close()


def max_mom(rhs):
    return max(np.abs(rhs[1]).max(), np.abs(rhs[2]).max())


def integrate(form, values):
    m = node_mass(form.mesh, form.order).reshape(-1)
    return float(np.sum(m * values))


def lake_at_rest_any_nodal_bathymetry(make, orders=(1, 2, 3, 4)):
    """|dh/dt| < 1e-12, |d(hu)/dt| < 1e-9 (swe_2d_split_form.rs:1259-1290)."""
    for order in orders:
        for periodic in (True, False):
            for bed in BEDS:
                for formulation in SPLIT_FORMS:
                    form = cases.split_form_setup(order, periodic, bed, formulation=formulation)
                    rhs = rhs_of(make, form, cases.split_form_state(form, 0.0))
                    mh, mm = np.abs(rhs[0]).max(), max_mom(rhs)
                    assert mh < 1e-12 and mm < 1e-9, (order, periodic, bed, formulation, mh, mm)


def mass_conservation(make, orders=(1, 2, 3)):
    """|d(mass)/dt| / mass < 1e-14 on periodic meshes (swe_2d_split_form.rs:1315-1337)."""
    for order in orders:
        for bed in BEDS:
            for formulation in SPLIT_FORMS:
                form = cases.split_form_setup(order, True, bed, formulation=formulation)
                q = cases.split_form_state(form, 1.0)
                mass = integrate(form, q[0])
                rhs = rhs_of(make, form, q)
                rate = integrate(form, rhs[0])
                assert abs(rate) / mass < 1e-14, (order, bed, formulation, rate / mass)


def entropy_rate(form, q, rhs):
    h, hu, hv = q
    b = form.bathymetry.reshape(-1)
    wet = h > 1e-6
    u = np.where(wet, hu / np.where(wet, h, 1.0), 0.0)
    v = np.where(wet, hv / np.where(wet, h, 1.0), 0.0)
    w0 = G * (h + b) - 0.5 * (u * u + v * v)
    dot = w0 * rhs[0] + u * rhs[1] + v * rhs[2]
    return integrate(form, dot), integrate(form, np.abs(dot))


def entropy_conservation_and_stability(make, orders=(1, 2, 3)):
    """EntropyConservative keeps the energy (|dE/dt| < 1e-12 scale);
    EntropyStable and WetDry dissipate it (swe_2d_split_form.rs:1341-1390)."""
    for order in orders:
        for periodic in (True, False):
            for bed in BEDS:
                form = cases.split_form_setup(order, periodic, bed,
                                              formulation=abi.ENTROPY_CONSERVATIVE)
                h, hu, hv = cases.split_form_state(form, 1.0)
                nn = form.n_nodes
                offset = np.repeat(0.05 * (np.arange(form.mesh.n_elements) % 3), nn)
                q = (h + offset, hu, hv)
                rate, scale = entropy_rate(form, q, rhs_of(make, form, q))
                assert abs(rate) < 1e-12 * scale, ("EC", order, periodic, bed, rate, scale)
                for formulation in (abi.ENTROPY_STABLE, abi.WET_DRY):
                    form.formulation = formulation
                    rate, scale = entropy_rate(form, q, rhs_of(make, form, q))
                    assert rate < -1e-10 * scale, (formulation, order, periodic, bed, rate, scale)


def wet_dry_lake_at_rest_with_shorelines(make, orders=(1, 2, 3, 4)):
    """< 1e-14 in h, < 1e-13 in momentum at shorelines; the wet-only split
    form is not balanced there (swe_2d_split_form.rs:1480-1516)."""
    for order in orders:
        for periodic in (True, False):
            for rough in (False, True):
                form = cases.shoreline_setup(order, periodic, rough)
                q = cases.shoreline_state(form, 0.0)
                assert (q[0] == 0.0).any()
                rhs = rhs_of(make, form, q)
                mh, mm = np.abs(rhs[0]).max(), max_mom(rhs)
                assert mh < 1e-14 and mm < 1e-13, (order, periodic, rough, mh, mm)
                if not rough:
                    form.formulation = abi.ENTROPY_STABLE
                    assert max_mom(rhs_of(make, form, q)) > 1e-6


def wet_dry_lake_at_rest_with_films_below_h_min(make, orders=(1, 2, 3)):
    """Films of 5 mm under h_min = 1 cm keep their full pressure
    (swe_2d_split_form.rs:1518-1545)."""
    for order in orders:
        form = cases.shoreline_setup(order, True, False, h_min=1e-2)
        b = form.bathymetry
        form.bathymetry = np.where((b >= 0.25) & (b < 0.3), 0.3 - 5e-3, b)
        q = cases.shoreline_state(form, 0.0)
        assert np.any(np.abs(q[0] - 5e-3) < 1e-12)
        mm = max_mom(rhs_of(make, form, q))
        assert mm < 1e-13, (order, mm)


def wet_dry_mass_conservation_with_dry_regions(make, orders=(1, 2, 3)):
    """|d(mass)/dt| < 1e-14 ∫|dh/dt| (swe_2d_split_form.rs:1547-1570)."""
    for order in orders:
        for rough in (False, True):
            form = cases.shoreline_setup(order, True, rough)
            q = cases.shoreline_state(form, 1.0)
            rhs = rhs_of(make, form, q)
            rate = integrate(form, rhs[0])
            scale = integrate(form, np.abs(rhs[0]))
            assert abs(rate) < 1e-14 * scale, (order, rough, rate, scale)


def wet_dry_floods_a_dry_node_below_the_water(make):
    """A dry node below the water beside it floods (swe_2d_split_form.rs:1616-1678)."""
    order = 2
    n1 = order + 1
    stencils = [
        [(4.0, 0.0), (-3.8, 0.8), (0.35, 0.0), (-3.8, 0.8), (4.0, 0.0)],
        [(-3.0, 0.8), (0.5, 0.0), (-3.0, -0.2)],
    ]
    for nodes in stencils:
        nx = (len(nodes) - 1) // (n1 - 1)
        width = 100.0 * nx
        mesh = uniform_rectangle(0.0, width, 0.0, 100.0, nx, 1)
        form = SWEDeviceForm2D(mesh=mesh, order=order, wet_dry=False, positivity_h_dry=None,
                               boundaries={TAG_WALL: WallBoundary()})
        x, _ = form.positions()
        pos = np.rint(x / width * (len(nodes) - 1)).astype(int)
        b = np.array([nodes[p][0] for p in pos.reshape(-1)]).reshape(x.shape)
        eta = np.array([nodes[p][1] for p in pos.reshape(-1)]).reshape(x.shape)
        form.bathymetry = b
        h = np.maximum(eta - b, 0.0).reshape(-1)
        rhs = rhs_of(make, form, (h, np.zeros_like(h), np.zeros_like(h)))
        for idx, p in enumerate(pos.reshape(-1)):
            bb, ee = nodes[p]
            lo = max(p - 1, 0)
            around = nodes[lo:p + 2]
            below_water = any(ne > nb and ne > bb for nb, ne in around)
            if ee <= bb and below_water:
                assert rhs[0][idx] > 1e-3, (nodes, idx, rhs[0][idx])


def uniform_flow_flat_bottom_is_steady(make):
    """A uniform flow over a flat bed has zero RHS (< 1e-12) (swe_2d_split_form.rs:1680-1700)."""
    mesh = uniform_periodic(0.0, 1.0, 0.0, 1.0, 4, 4)
    for formulation in SPLIT_FORMS:
        form = SWEDeviceForm2D(mesh=mesh, order=3, formulation=formulation, wet_dry=False,
                               positivity_h_dry=None, boundaries={TAG_WALL: WallBoundary()})
        n = form.n_values
        h = np.full(n, 2.0)
        rhs = rhs_of(make, form, (h, 2.0 * np.full(n, 0.5), 2.0 * np.full(n, -0.2)))
        assert max(np.abs(r).max() for r in rhs) < 1e-12, formulation


ALL = [
    lake_at_rest_any_nodal_bathymetry,
    mass_conservation,
    entropy_conservation_and_stability,
    wet_dry_lake_at_rest_with_shorelines,
    wet_dry_lake_at_rest_with_films_below_h_min,
    wet_dry_mass_conservation_with_dry_regions,
    wet_dry_floods_a_dry_node_below_the_water,
    uniform_flow_flat_bottom_is_steady,
]
