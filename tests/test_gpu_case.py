"""A case file run on the device (``case.run_case``: the form, the state
and ``Cuda.run_2d`` with the stations sampled at every interval) against
the same case on the oracle, and its ``stations.csv``; with global steps
and with local time stepping."""

import csv

import numpy as np
import pytest

from dgcom_gb300 import case as C
from dgcom_gb300.device import DeviceRun
from oracle_lib import oracle
from test_case import BASIN, write

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("levels", [0, 3])
def test_a_case_on_the_device_is_the_case_on_the_oracle(tmp_path, levels):
    text = BASIN.replace('integrator = "ssp_rk3"',
                         f'integrator = "ssp_rk3"\nlocal_time_stepping_levels = {levels}')
    path = write(tmp_path, text)
    got = C.run_case(path)
    assert got.report.success, got.report.message
    case = C.load_case(path)
    form, q = C.build_form(case)
    ref = oracle(form)
    try:
        ref.upload(*q)
        rep = ref.run_with_callback(DeviceRun(span=(0.0, case.duration_s), cfl=case.cfl,
                                              interval=case.station_interval_s,
                                              scheme=case.scheme, levels=levels))
        assert rep.success and rep.n_steps == got.report.n_steps
        want = ref.download()
    finally:
        ref.close()
    for a, b in zip(got.state, want):
        scale = max(np.abs(b).max(), 1e-300)
        assert np.abs(a.reshape(-1) - b).max() <= 1e-10 * scale
    rows = list(csv.reader(open(case.output_dir / "stations.csv")))
    assert rows[0] == ["station", "time_s", "eta_m", "u_m_s", "v_m_s", "depth_m"]
    assert len(rows) == 1 + 2 * 4  # two stations at 0, 60, 120 and 180 s
    assert [float(r[1]) for r in rows[1::2]] == pytest.approx([0.0, 60.0, 120.0, 180.0])
    mouth = [float(r[2]) for r in rows[1::2]]
    assert mouth[0] == pytest.approx(0.0, abs=1e-12) and mouth[-1] != mouth[0]
