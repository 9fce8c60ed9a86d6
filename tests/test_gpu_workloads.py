"""Parity of the CUDA path with the oracle on the plain workloads as they
are run and timed, through the C ABI:

- the coastal box (the unstructured quad paving with its random bed, its
  islands and the four-constituent tide at the open side, N = 3): a 20k-quad
  sample from rest (as the bench times it) and from its running tide (spun
  up on the device past the one-hour ramp), stage by stage, the element
  steps, and fused steps; and the full 1 M-quad box, one step stage by
  stage from rest and from a flowing state;
- the tidal channel at its full size (200 × 20 quads, N = 2, SSP-RK3,
  CFL 0.5) over a whole M2 cycle: every step against the oracle from the
  same state, then both running free with the stations compared.

Tolerance. A stage state's field is held to 1e-12 of the largest value the
field takes in the workload's running tide (TOL × scale). A state at rest
holds momentum of round-off size (≈ 1e-12 m²/s on this bed: the remainder
of g·h·∇h against g·h·∇B), which two correct implementations round
differently, so a state at rest cannot be judged relative to its own
momentum; its differences are measured against the same per-field scale as
the running tide's. The steps agree to 1e-13 relative."""


import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.case import Probe, locate
from dgcom_gb300.device import DeviceRun, SWEPhysics2D
from dgcom_gb300.mesh import TAG_OPEN
from oracle_lib import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_DT = 1e-13
NUMERICS = [abi.NUMERICS_FAST, abi.NUMERICS_EXACT]
SPIN_UP = 5400.0  # 1.5 h: the tide past its one-hour ramp


def field_errors(got, want, scale):
    """max |g − w| / scale per field (h, hu, hv)."""
    return [float(np.abs(g - w).max() / s) for g, w, s in zip(got, want, scale)]


def three_stages(dev, ref, t, dt):
    """The SSP-RK3 stages one by one (stage_where), then finish; the four
    buffers of each side."""
    for s in (dev, ref):
        s.stage_where(base=0, input=0, out=1, time=t, a=1.0, b=0.0, c=dt)
        s.stage_where(base=0, input=1, out=2, time=t + dt, a=0.75, b=0.25, c=0.25 * dt)
        s.stage_where(base=0, input=2, out=3, time=t + 0.5 * dt, a=1.0 / 3.0, b=2.0 / 3.0,
                      c=2.0 / 3.0 * dt, acc=4, w=1.0, keep=0.0)
    got = [dev.download(b) for b in (1, 2, 3)]
    want = [ref.download(b) for b in (1, 2, 3)]
    for s in (dev, ref):
        s.finish_where(4)
    got.append(dev.download())
    want.append(ref.download())
    return got, want


def compare_steps(dev, ref, t, n_steps, scale, cfl=0.5, fused=False):
    """``n_steps`` SSP-RK3 steps of both from the oracle's state (resynced
    every step); the worst per-field error and the worst dt difference."""
    worst, worst_dt = [0.0, 0.0, 0.0], 0.0
    for step in range(n_steps):
        dt_ref = ref.compute_dt_ssp(cfl)
        dt_dev = dev.compute_dt_ssp(cfl)
        worst_dt = max(worst_dt, abs(dt_dev - dt_ref) / dt_ref)
        if fused:
            for s in (dev, ref):
                s.step(t, dt_ref)
            pairs = [(dev.download(), ref.download())]
        else:
            pairs = list(zip(*three_stages(dev, ref, t, dt_ref)))
        for g, w in pairs:
            worst = [max(a, b) for a, b in zip(worst, field_errors(g, w, scale))]
        dev.upload(*ref.download())
        t += dt_ref
    return worst, worst_dt


@pytest.fixture(scope="module")
def box():
    """The 20k-quad coastal box, its state at rest and its running tide
    (spun up on the device to 1.5 h), and the running tide's per-field
    scale."""
    case = cases.coastal_box(20_000)
    dev = SWEPhysics2D(case.form, 0)
    try:
        dev.upload(*case.state)
        rep = dev.run_with_callback(DeviceRun(span=(0.0, SPIN_UP), cfl=case.cfl))
        assert rep.success and rep.negative_depth_clips == 0, rep.message
        flowing = dev.download()
    finally:
        dev.close()
    scale = [float(np.abs(f).max()) for f in flowing]
    return case, flowing, scale


def test_the_box_runs_a_tide_over_drying_islands(box):
    case, flowing, scale = box
    h = flowing[0].reshape(case.form.mesh.n_elements, -1)
    dry_nodes = (h <= 1e-6).mean()
    shallow_elements = (h < 1e-3).any(axis=1).mean()  # elements with subcells
    assert scale[1] > 10.0 and scale[2] > 10.0  # the tide moves tens of m²/s
    assert 0.001 < dry_nodes < 0.1 and shallow_elements > 0.001
    assert h.min() >= 0.0
    assert len(case.form.boundaries[TAG_OPEN].constituents) == 4


@pytest.mark.parametrize("numerics", NUMERICS)
@pytest.mark.parametrize("start", ["rest", "running"])
def test_coastal_box_stages_match_oracle(box, numerics, start):
    case, flowing, scale = box
    form = cases.coastal_box(20_000, numerics=numerics).form
    dev, ref = SWEPhysics2D(form, 0), oracle(form)
    try:
        q, t = (case.state, 0.0) if start == "rest" else (flowing, SPIN_UP)
        for s in (dev, ref):
            s.upload(*q)
        worst, worst_dt = compare_steps(dev, ref, t, 20, scale)
        print(f"box 20k {start} numerics {numerics}: per-field errors {worst}, dt {worst_dt:.2e}")
        assert max(worst) <= TOL, f"per-field errors {worst}"
        assert worst_dt <= TOL_DT, f"dt {worst_dt:.3e}"
        assert dev.negative_depth_clips() == ref.negative_depth_clips() == 0
        assert dev.download()[0].min() >= 0.0
    finally:
        dev.close()
        ref.close()


@pytest.mark.parametrize("start", ["rest", "running"])
def test_coastal_box_fused_steps_match_oracle(box, start):
    case, flowing, scale = box
    dev, ref = SWEPhysics2D(case.form, 0), oracle(case.form)
    try:
        q, t = (case.state, 0.0) if start == "rest" else (flowing, SPIN_UP)
        for s in (dev, ref):
            s.upload(*q)
        worst, worst_dt = compare_steps(dev, ref, t, 20, scale, fused=True)
        assert max(worst) <= TOL, f"per-field errors {worst}"
        assert worst_dt <= TOL_DT
    finally:
        dev.close()
        ref.close()


def test_coastal_box_element_steps_match_oracle(box):
    case, flowing, _ = box
    dev, ref = SWEPhysics2D(case.form, 0), oracle(case.form)
    try:
        for q in (case.state, flowing):
            for s in (dev, ref):
                s.upload(*q)
            a, b = dev.element_dt(case.cfl), ref.element_dt(case.cfl)
            finite = np.isfinite(b)
            assert np.array_equal(np.isfinite(a), finite)
            assert np.abs(a[finite] - b[finite]).max() <= TOL_DT * b[finite].max()
    finally:
        dev.close()
        ref.close()


def test_full_size_coastal_box_step_matches_oracle():
    """The benchmarked 1 M-quad box itself: one step stage by stage from
    rest at t = 0, and from a flowing state after the ramp."""
    case = cases.coastal_box(1_000_000)
    moving = cases.with_flow(case)
    scale = [float(np.abs(f).max()) for f in moving]
    dev, ref = SWEPhysics2D(case.form, 0), oracle(case.form)
    try:
        for q, t in ((case.state, 0.0), (moving, 7200.0)):
            for s in (dev, ref):
                s.upload(*q)
            worst, worst_dt = compare_steps(dev, ref, t, 1, scale)
            print(f"box 1M t={t}: per-field errors {worst}, dt {worst_dt:.2e}")
            assert max(worst) <= TOL, f"t {t}: per-field errors {worst}"
            assert worst_dt <= TOL_DT
    finally:
        dev.close()
        ref.close()


# -- the tidal channel over an M2 cycle ---------------------------------------

def station_probes(case):
    form = case.form
    probes = []
    for x, y in case.stations:
        k = locate(form.mesh, float(x), float(y))
        probes.append(Probe(form.mesh, form.order, k, float(x), float(y)))
    return probes


def station_eta(probes, form, state):
    n = form.mesh.n_elements
    h = state[0].reshape(n, -1)
    b = form.bathymetry.reshape(n, -1)
    return np.array([p.value(h) + p.value(b) for p in probes])


def test_tidal_channel_m2_cycle_matches_oracle():
    """The tidal channel as specified (200 × 20, N = 2, M2 of 1 m with a
    one-hour ramp, Manning 0.025, f = 1.26e-4, SSP-RK3 at CFL 0.5) over one
    M2 period from rest.

    Every step from the same state: the step's dt to 1e-13 and the stepped
    state to 1e-12 of each field's largest value over the cycle, no
    negative-depth clip on the flooding and draining flat, and h ≥ 0. Then
    both run free over the cycle, each with its own steps, and their
    station surfaces are compared every 30 minutes."""
    case = cases.tidal_channel()
    form = case.form
    period = form.boundaries[TAG_OPEN].constituents[0].period
    dev, ref = SWEPhysics2D(form, 0), oracle(form)
    try:
        for s in (dev, ref):
            s.upload(*case.state)
        t = 0.0
        n_steps = 0
        err = np.zeros(3)
        top = np.zeros(3)
        worst_dt = 0.0
        min_h = np.inf
        while t < period:
            dt = ref.compute_dt_ssp(case.cfl)
            worst_dt = max(worst_dt, abs(dev.compute_dt_ssp(case.cfl) - dt) / dt)
            for s in (dev, ref):
                s.step(t, dt)
            g, w = dev.download(), ref.download()
            err = np.maximum(err, [np.abs(a - b).max() for a, b in zip(g, w)])
            top = np.maximum(top, [np.abs(b).max() for b in w])
            min_h = min(min_h, float(g[0].min()))
            dev.upload(*w)
            t += dt
            n_steps += 1
        rel = err / top
        print(f"channel M2 cycle: {n_steps} steps, per-field errors {rel}, dt {worst_dt:.2e}")
        assert n_steps > 20_000
        assert rel.max() <= TOL, f"per-field errors over the cycle {rel} (scale {top})"
        assert worst_dt <= TOL_DT, f"dt {worst_dt:.3e}"
        assert min_h >= 0.0
        assert dev.negative_depth_clips() == 0 and ref.negative_depth_clips() == 0

        # both running free over the cycle, stations every 30 minutes
        probes = station_probes(case)
        series = {}
        for name, s in (("device", dev), ("oracle", ref)):
            s.upload(*case.state)
            rows = []
            rep = s.run_with_callback(DeviceRun(span=(0.0, period), cfl=case.cfl,
                                                interval=1800.0),
                                      lambda tt, h, hu, hv, rows=rows: rows.append(
                                          (tt, station_eta(probes, form, (h, hu, hv)))))
            assert rep.success and rep.negative_depth_clips == 0, rep.message
            series[name] = rows
        times = [r[0] for r in series["oracle"]]
        assert [r[0] for r in series["device"]] == pytest.approx(times, abs=1e-9)
        diff = np.array([np.abs(a[1] - b[1]).max()
                         for a, b in zip(series["device"], series["oracle"])])
        mouth = np.array([r[1][0] for r in series["oracle"]])
        print(f"free runs: station surfaces differ by at most {diff.max():.3e} m "
              f"(per half hour {np.array2string(diff, precision=2)})")
        assert np.abs(mouth).max() > 0.3  # the tide reached the stations
        assert diff.max() <= 1e-9, f"station surfaces differ by up to {diff.max():.3e} m"
    finally:
        dev.close()
        ref.close()
