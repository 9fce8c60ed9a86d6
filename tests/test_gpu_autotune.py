"""dgswe_autotune: the kernels' launch shapes (the face kernel's threads per
block, the stage kernel's elements per block) change no result. Every
shape gives the default shapes' RHS, stage and run bit for bit, global
and multirate, on a drying channel (subcells, dry elements) at N = 2 and
3; the tuner returns one of its shapes with positive timings, and a run
after it (its step graph captured again) equals a run before it."""

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.device import DeviceRun, SWEPhysics2D

pytestmark = pytest.mark.gpu


def flowing(order):
    case = cases.tidal_channel(nx=24, ny=3, order=order)
    return case, cases.with_flow(case, eta_amp=0.3, u=0.3, v=0.05)


def outputs(form, q, face=None, stage=None, levels=0):
    dev = SWEPhysics2D(form, 0)
    try:
        dev.upload(*q)
        if face is not None:
            dev.autotune(1, face, stage)
        rhs = dev.compute_rhs_into(9000.5)
        dt = dev.compute_dt_ssp(0.5)
        dev.stage_where(base=0, input=0, out=1, time=9000.5, a=1.0, b=0.0, c=dt)
        staged = dev.download(1)
        rep = dev.run_with_callback(DeviceRun(span=(4000.0, 4150.0), cfl=0.5, levels=levels))
        assert rep.success, rep.message
        return rhs, staged, dev.download()
    finally:
        dev.close()


@pytest.mark.parametrize("order", [2, 3])
@pytest.mark.parametrize("levels", [0, 3])
def test_every_shape_gives_the_same_bits(order, levels):
    case, q = flowing(order)
    want = outputs(case.form, q, levels=levels)
    for face in (64, 128, 256):
        for stage in (0, 1, 2):
            got = outputs(case.form, q, face, stage, levels)
            for a, b in zip(got, want):
                for x, y in zip(a, b):
                    assert np.array_equal(x, y), f"face {face}, stage shape {stage}"


def test_tuner_picks_a_shape_and_runs_stay_the_same():
    case, q = flowing(3)
    runs = []
    for tune in (False, True):
        dev = SWEPhysics2D(case.form, 0)
        try:
            dev.upload(*q)
            rep = dev.run_with_callback(DeviceRun(span=(4000.0, 4100.0), cfl=0.5))
            assert rep.success
            if tune:
                t = dev.autotune(3)
                assert t["face_threads"] in (64, 128, 256)
                nn = 16
                assert t["stage_threads"] in (128 // nn * nn, 64 // nn * nn)
                assert all(ms > 0.0 for ms in t["face_ms"] + t["stage_ms"])
            rep = dev.run_with_callback(DeviceRun(span=(4100.0, 4200.0), cfl=0.5))
            assert rep.success
            runs.append(dev.download())
        finally:
            dev.close()
    for x, y in zip(*runs):
        assert np.array_equal(x, y)


def test_bad_shapes_are_refused():
    case, q = flowing(2)
    dev = SWEPhysics2D(case.form, 0)
    try:
        dev.upload(*q)
        t = abi.Tuning()
        assert dev.lib.autotune(dev.handle, 1, 100, -1, t) == abi.ERR_INVALID
        assert dev.lib.autotune(dev.handle, 0, -1, -1, t) == abi.ERR_INVALID
        assert dev.lib.autotune(dev.handle, 1, -1, 3, t) == abi.ERR_INVALID
    finally:
        dev.close()
