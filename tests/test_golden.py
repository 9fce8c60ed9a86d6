"""The oracle against its committed outputs (tests/golden/oracle_regression.npz,
made by tests/golden/make_golden.py), and the CUDA library against the same
fixture: a change of either shows."""

import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).parent / "golden"
sys.path.insert(0, str(GOLDEN))
import make_golden  # noqa: E402


def rel(a, b):
    return max(float(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300)) for x, y in zip(a, b))


def test_oracle_matches_its_fixture():
    want = np.load(GOLDEN / "oracle_regression.npz")
    got = make_golden.outputs()
    for key in want.files:
        # same arithmetic; only the libm of another platform may move a last bit
        assert rel(got[key], want[key]) <= 1e-13, key


@pytest.mark.gpu
def test_device_matches_the_fixture():
    from dgcom_gb300 import cases
    from dgcom_gb300.device import SWEPhysics2D

    want = np.load(GOLDEN / "oracle_regression.npz")
    case = cases.tidal_channel(nx=20, ny=4)
    dev = SWEPhysics2D(case.form, 0)
    dev.upload(*cases.with_flow(case))
    dt = dev.compute_dt_ssp(case.cfl)
    assert abs(dt - want["channel_dt"][0]) <= 1e-13 * dt
    dev.step(600.0, want["channel_dt"][0])
    assert rel(dev.download(), want["channel_step"]) <= 1e-12
    form = cases.shoreline_setup(2, False, True, curved=True)
    dev = SWEPhysics2D(form, 0)
    dev.upload(*cases.shoreline_state(form, 0.5))
    assert rel(dev.compute_rhs_into(0.0), want["shoreline_rhs"]) <= 1e-10
