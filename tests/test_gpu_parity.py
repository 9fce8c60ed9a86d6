"""Parity of the CUDA path with the oracle (the CPU restatement of the
reference path), through the C ABI, on the reference's own test setups.

The bar the path is judged on is per stage: for each field of a stage
state, max |gpu − oracle| ≤ 1e-12 × max |oracle| after one stage (or one
step) from identical inputs (TOL). A right-hand side alone is the small
difference of large hydrostatic terms (g·h·∇h against g·h·∇B), so
reordered sums and FMA contraction move it by more of its own field's
largest value: the reference measured 1e-13 to 2e-11 for contraction alone
(gpu/src/gate.rs:1-22) and gates an RHS at 1e-9. Here an RHS is held to
TOL_RHS = 1e-10 of its field's largest value, and the stage state it makes
to TOL."""

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.device import SWEPhysics2D
from oracle_lib import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_RHS = 1e-10
NUMERICS = [abi.NUMERICS_FAST, abi.NUMERICS_EXACT]


def rel_err(got, want, floor=1e-300):
    return max(float(np.abs(g - w).max() / max(np.abs(w).max(), floor)) for g, w in zip(got, want))


def pair(form):
    return SWEPhysics2D(form, 0), oracle(form)


def check_stage(dev, ref, cfl=0.5):
    """Both from the same state: the first SSP-RK3 stage at the oracle's
    stable step, compared at TOL."""
    dt = ref.compute_dt_ssp(cfl)
    assert np.isfinite(dt) and dt > 0.0
    for s in (dev, ref):
        s.stage_where(base=0, input=0, out=1, time=0.0, a=1.0, b=0.0, c=dt)
    err = rel_err(dev.download(1), ref.download(1))
    assert err <= TOL, f"relative stage difference {err:.3e}"


@pytest.mark.parametrize("numerics", NUMERICS)
@pytest.mark.parametrize("formulation", [abi.WET_DRY, abi.ENTROPY_STABLE, abi.ENTROPY_CONSERVATIVE])
@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("curved", [False, True])
@pytest.mark.parametrize("bed", ["smooth", "rough"])
def test_rhs_matches_oracle_wet(numerics, formulation, order, periodic, curved, bed):
    form = cases.split_form_setup(order, periodic, bed, curved=curved, numerics=numerics,
                                  formulation=formulation)
    form.coriolis_f0 = 1.2e-4
    dev, ref = pair(form)
    q = cases.split_form_state(form, 1.0)
    dev.upload(*q)
    ref.upload(*q)
    err = rel_err(dev.compute_rhs_into(0.0), ref.compute_rhs_into(0.0))
    assert err <= TOL_RHS, f"relative RHS difference {err:.3e}"
    check_stage(dev, ref)


@pytest.mark.parametrize("numerics", NUMERICS)
@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("rough", [False, True])
@pytest.mark.parametrize("curved", [False, True])
def test_rhs_matches_oracle_shoreline(numerics, order, periodic, rough, curved):
    form = cases.shoreline_setup(order, periodic, rough, curved=curved, numerics=numerics)
    dev, ref = pair(form)
    q = cases.shoreline_state(form, 0.5)
    dev.upload(*q)
    ref.upload(*q)
    err = rel_err(dev.compute_rhs_into(0.0), ref.compute_rhs_into(0.0))
    assert err <= TOL_RHS, f"relative RHS difference {err:.3e}"
    check_stage(dev, ref)


@pytest.mark.parametrize("numerics", NUMERICS)
@pytest.mark.parametrize("order", [2, 3])
def test_stages_match_oracle_tidal_channel(numerics, order):
    case = cases.tidal_channel(nx=40, ny=4, order=order, numerics=numerics)
    dev, ref = pair(case.form)
    q = cases.with_flow(case)
    for s in (dev, ref):
        s.upload(*q)
    t = 0.0
    for step in range(5):
        dt_ref = ref.compute_dt_ssp(case.cfl)
        dt_dev = dev.compute_dt_ssp(case.cfl)
        assert abs(dt_dev - dt_ref) <= 1e-13 * dt_ref
        # the three stages one by one (stage_where), then finish
        for s in (dev, ref):
            s.stage_where(base=0, input=0, out=1, time=t, a=1.0, b=0.0, c=dt_ref)
            s.stage_where(base=0, input=1, out=2, time=t + dt_ref, a=0.75, b=0.25, c=0.25 * dt_ref)
            s.stage_where(base=0, input=2, out=3, time=t + 0.5 * dt_ref, a=1.0 / 3.0, b=2.0 / 3.0,
                          c=2.0 / 3.0 * dt_ref, acc=4, w=1.0, keep=0.0)
        for b in (1, 2, 3, 4):
            err = rel_err(dev.download(b), ref.download(b))
            assert err <= TOL, f"step {step}, buffer {b}: {err:.3e}"
        for s in (dev, ref):
            s.finish_where(4)
        err = rel_err(dev.download(), ref.download())
        assert err <= TOL, f"step {step}: {err:.3e}"
        # keep both on the oracle's state so every step starts identical
        dev.upload(*ref.download())
        t += dt_ref
    assert dev.negative_depth_clips() == ref.negative_depth_clips() == 0


@pytest.mark.parametrize("numerics", NUMERICS)
def test_fused_step_matches_oracle(numerics):
    case = cases.tidal_channel(nx=40, ny=4, order=2, numerics=numerics)
    dev, ref = pair(case.form)
    q = cases.with_flow(case)
    for s in (dev, ref):
        s.upload(*q)
    t = 0.0
    for _ in range(20):
        dt = ref.compute_dt_ssp(case.cfl)
        for s in (dev, ref):
            s.step(t, dt)
        err = rel_err(dev.download(), ref.download())
        assert err <= TOL
        dev.upload(*ref.download())
        t += dt


@pytest.mark.parametrize("numerics", NUMERICS)
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_element_dt_matches_oracle(numerics, order):
    form = cases.shoreline_setup(order, False, True, curved=True, numerics=numerics, wet_dry=True)
    dev, ref = pair(form)
    q = cases.shoreline_state(form, 0.5)
    dev.upload(*q)
    ref.upload(*q)
    for scheme in (abi.SSP_RK3, abi.SSP_RK43):
        a, b = dev.element_dt(0.9, scheme), ref.element_dt(0.9, scheme)
        finite = np.isfinite(b)
        assert np.array_equal(np.isfinite(a), finite)
        assert np.abs(a[finite] - b[finite]).max() <= 1e-13 * b[finite].max()


def test_shoreline_lake_at_rest_is_balanced_on_device():
    for order in (1, 2, 3, 4):
        form = cases.shoreline_setup(order, True, True)
        dev = SWEPhysics2D(form, 0)
        dev.upload(*cases.shoreline_state(form, 0.0))
        rh, rhu, rhv = dev.compute_rhs_into(0.0)
        assert np.abs(rh).max() < 1e-14 and max(np.abs(rhu).max(), np.abs(rhv).max()) < 1e-13


def test_lake_at_rest_any_bed_on_device():
    for order in (1, 2, 3, 4):
        for periodic in (True, False):
            for bed in ("smooth", "cell_average", "rough"):
                form = cases.split_form_setup(order, periodic, bed)
                dev = SWEPhysics2D(form, 0)
                dev.upload(*cases.split_form_state(form, 0.0))
                rh, rhu, rhv = dev.compute_rhs_into(0.0)
                assert np.abs(rh).max() < 1e-12
                assert max(np.abs(rhu).max(), np.abs(rhv).max()) < 1e-9
