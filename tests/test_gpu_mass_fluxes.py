"""dgswe_compute_rhs_mass_fluxes on the device: the reference's own checks
of the mass fluxes (the RHS unchanged bit for bit, every element balanced
by its faces' F*_h, the subcell elements' mass tendency node by node from
the interface fluxes, NaN elsewhere) on the device's outputs, and the
outputs against the oracle's: on the reference's test setups and on the
tidal channel's drying flat with a flowing state, FAST and EXACT."""

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.device import SWEPhysics2D
from oracle_lib import oracle
from test_mass_fluxes import mass_flux_checks, setup

pytestmark = pytest.mark.gpu

TOL_RHS = 1e-10


def device(form):
    return SWEPhysics2D(form, 0)


def close(got, want, what):
    nan_g, nan_w = np.isnan(got), np.isnan(want)
    assert np.array_equal(nan_g, nan_w), f"{what}: NaN slots differ"
    g, w = got[~nan_g], want[~nan_w]
    if w.size:
        err = np.abs(g - w).max() / max(np.abs(w).max(), 1e-300)
        assert err <= TOL_RHS, f"{what}: {err:.3e}"


@pytest.mark.parametrize("numerics", [abi.NUMERICS_FAST, abi.NUMERICS_EXACT])
@pytest.mark.parametrize("formulation", [abi.ENTROPY_STABLE, abi.WET_DRY])
def test_face_mass_balances_each_element(numerics, formulation):
    form, q = setup(2, formulation)
    form.numerics = numerics
    got = mass_flux_checks(device, form, q)
    want = mass_flux_checks(oracle, form, q)
    for a, b, what in zip(got, want, ("rhs", "face", "subcell")):
        close(np.asarray(a), np.asarray(b), what)


@pytest.mark.parametrize("numerics", [abi.NUMERICS_FAST, abi.NUMERICS_EXACT])
@pytest.mark.parametrize("distorted", [False, True])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_subcell_mass_fluxes_match_the_oracle(numerics, distorted, order):
    form, q = setup(order, abi.WET_DRY, distorted, subcell_depth=0.1,
                    bed=lambda x, y: -1.0 + 2.0 * x + 0.2 * y)
    form.numerics = numerics
    got = mass_flux_checks(device, form, q, subcell_depth=0.1)
    want = mass_flux_checks(oracle, form, q, subcell_depth=0.1)
    for a, b, what in zip(got[1:], want[1:], ("face", "subcell")):
        close(np.asarray(a), np.asarray(b), what)


@pytest.mark.parametrize("order", [2, 3])
def test_tidal_channel_drying_flat(order):
    case = cases.tidal_channel(nx=24, ny=3, order=order)
    q = cases.with_flow(case, eta_amp=0.3, u=0.3, v=0.05)
    out = []
    for make in (device, oracle):
        sim = make(case.form)
        try:
            sim.upload(*q)
            out.append(sim.compute_rhs_mass_fluxes_into(9000.5))
        finally:
            sim.close()
    (rhs, face, sub), (rhs_o, face_o, sub_o) = out
    for a, b in zip(rhs, rhs_o):
        close(a, b, "rhs")
    close(face, face_o, "face")
    close(sub, sub_o, "subcell")
    assert np.isfinite(sub).any(axis=1).sum() >= 3  # the shoreline column takes the subcells
