"""PhysicsModule's implicit_damping and post_process as entry points of
their own (dgswe_implicit_damping, dgswe_post_process) against the
oracle's, through the C ABI, on the coastal box (20k quads, N = 3, its
drying islands): a stage value damped over a long dt with the rates frozen
at a flowing state, and a state pushed below the shoreline's depths
corrected in place, in both numerics variants.

Tolerance: each field to 1e-12 of its largest value (the FAST variant's
reciprocal and Manning rate are within an ulp, not the IEEE operations);
the clip counts exactly."""

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.device import SWEPhysics2D
from oracle_lib import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12
NUMERICS = [abi.NUMERICS_FAST, abi.NUMERICS_EXACT]


def errors(got, want):
    return [float(np.abs(g - w).max() / max(np.abs(w).max(), 1e-300)) for g, w in zip(got, want)]


@pytest.mark.parametrize("numerics", NUMERICS)
def test_implicit_damping_matches_oracle(numerics):
    case = cases.coastal_box(20_000, numerics=numerics)
    flow = cases.with_flow(case, eta_amp=0.5, u=0.4, v=-0.15)
    rng = np.random.default_rng(3)
    # a stage value near the flowing state, some of its nodes in the thin layer
    stage = [flow[0] * (1.0 + 0.01 * rng.standard_normal(flow[0].size)),
             flow[1] + 0.05 * rng.standard_normal(flow[1].size),
             flow[2] + 0.05 * rng.standard_normal(flow[2].size)]
    stage[0] = np.where(flow[0] > 0.0, np.abs(stage[0]), 0.0)
    dev, ref = SWEPhysics2D(case.form, 0), oracle(case.form)
    try:
        got = {}
        for name, s in (("device", dev), ("oracle", ref)):
            s.upload(*flow)                # from: the state buffer
            s.upload(*stage, buffer=1)     # the stage value
            s.implicit_damping(1, abi.STATE, 30.0)
            got[name] = s.download(1)
        err = errors(got["device"], got["oracle"])
        assert max(err) <= TOL, err
        # the damping acted: momentum fell where the friction and thin layer bite
        assert np.abs(got["oracle"][1]).sum() < np.abs(stage[1]).sum()
        assert np.array_equal(got["device"][0], stage[0])  # depth untouched
    finally:
        dev.close()
        ref.close()


@pytest.mark.parametrize("numerics", NUMERICS)
def test_post_process_matches_oracle(numerics):
    case = cases.coastal_box(20_000, numerics=numerics)
    flow = cases.with_flow(case, eta_amp=0.5, u=0.4, v=-0.15)
    # depths lowered by 3 mm: negative nodes at the shorelines (the limiter
    # and the clips), films under h_dry (correct_node's desingularisation)
    q = (flow[0] - 0.003, flow[1], flow[2])
    dev, ref = SWEPhysics2D(case.form, 0), oracle(case.form)
    try:
        got, clips = {}, {}
        for name, s in (("device", dev), ("oracle", ref)):
            s.upload(*q, buffer=2)
            before = s.negative_depth_clips()
            s.post_process(2)
            clips[name] = s.negative_depth_clips() - before
            got[name] = s.download(2)
        err = errors(got["device"], got["oracle"])
        assert max(err) <= TOL, err
        assert clips["device"] == clips["oracle"]
        assert (q[0] < 0.0).any() and got["device"][0].min() >= 0.0
    finally:
        dev.close()
        ref.close()


def test_entry_points_refuse_bad_arguments():
    case = cases.tidal_channel(nx=20, ny=2, order=2)
    dev = SWEPhysics2D(case.form, 0)
    try:
        lib = dev.lib
        assert lib.implicit_damping(dev.handle, 99, 0, 1.0) == abi.ERR_INVALID
        assert lib.implicit_damping(dev.handle, 1, 0, -1.0) == abi.ERR_INVALID
        assert lib.implicit_damping(dev.handle, 1, 0, float("nan")) == abi.ERR_INVALID
        assert lib.post_process(dev.handle, -1) == abi.ERR_INVALID
    finally:
        dev.close()
