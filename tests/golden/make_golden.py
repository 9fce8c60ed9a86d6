"""Regenerates tests/golden/oracle_regression.npz: the oracle's outputs on
three small cases (the RHS of a curved shoreline mesh at N = 2, of a rough
walled mesh at N = 3, and one fused SSP-RK3 step of a coarse tidal channel
with flow), so that a change of the oracle itself shows. Run from the
repository root: python tests/golden/make_golden.py"""

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from dgcom_gb300 import cases  # noqa: E402
from oracle_lib import oracle  # noqa: E402


def outputs():
    out = {}
    form = cases.shoreline_setup(2, False, True, curved=True)
    o = oracle(form)
    o.upload(*cases.shoreline_state(form, 0.5))
    out["shoreline_rhs"] = np.stack(o.compute_rhs_into(0.0))
    o.close()
    form = cases.split_form_setup(3, False, "rough", curved=True)
    form.coriolis_f0 = 1.2e-4
    o = oracle(form)
    o.upload(*cases.split_form_state(form, 1.0))
    out["rough_rhs"] = np.stack(o.compute_rhs_into(0.0))
    o.close()
    case = cases.tidal_channel(nx=20, ny=4)
    o = oracle(case.form)
    o.upload(*cases.with_flow(case))
    dt = o.compute_dt_ssp(case.cfl)
    o.step(600.0, dt)
    out["channel_step"] = np.stack(o.download())
    out["channel_dt"] = np.array([dt])
    o.close()
    return out


if __name__ == "__main__":
    np.savez_compressed(Path(__file__).parent / "oracle_regression.npz", **outputs())
