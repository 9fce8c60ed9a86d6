"""The weather forcing (GriddedAtmosphere2D's device form) in the oracle:
the reference's known answers for the drag laws, the wind stress, the
musl hypot and the inverse-barometer level
(src/source/swe_2d/wind.rs:385-460, src/math.rs:555-590,
src/source/swe_2d/gridded_atmosphere.rs:965-1060, 1340-1370), restated on
regridded snapshots; the element source of a lake at rest under a uniform
wind and pressure gradient; and the inverse-barometer raise of a
characteristic boundary equal to the same level given as its mean."""

import ctypes as C
import dataclasses
import math

import numpy as np
import pytest

from dgcom_gb300 import abi
from dgcom_gb300.mesh import TAG_OPEN, TAG_WALL, uniform_rectangle
from dgcom_gb300.physics import GriddedAtmosphere, SWEDeviceForm2D, TidalBoundary, WallBoundary
from oracle_lib import oracle, oracle_library

RHO_AIR, RHO_WATER, G = 1.225, 1025.0, 9.81
T0 = 1_750_000_000.0


def ulps(a, b):
    ia = np.frombuffer(np.float64(a).tobytes(), np.int64)[0]
    ib = np.frombuffer(np.float64(b).tobytes(), np.int64)[0]
    return abs(int(ia) - int(ib))


def test_hypot_known_answers():
    lib = oracle_library()
    assert lib.hypot(3.0, 4.0) == 5.0
    assert lib.hypot(-3.0, 0.0) == 3.0
    assert ulps(lib.hypot(1e300, 1e300), math.hypot(1e300, 1e300)) <= 1
    assert ulps(lib.hypot(1e-300, 3e-301), math.hypot(1e-300, 3e-301)) <= 1
    rng = np.random.default_rng(7)
    for a, b in zip(rng.uniform(-1e3, 1e3, 5000), rng.uniform(-1e-2, 1e-2, 5000)):
        assert ulps(lib.hypot(a, b), math.hypot(a, b)) <= 1


def test_drag_coefficients():
    lib = oracle_library()
    tol = 1e-12
    assert abs(lib.drag_coefficient(abi.DRAG_CONSTANT, 1.5e-3, 5.0) - 1.5e-3) < tol
    assert abs(lib.drag_coefficient(abi.DRAG_CONSTANT, 1.5e-3, 20.0) - 1.5e-3) < tol
    lp = lambda s: lib.drag_coefficient(abi.DRAG_LARGE_POND, 0.0, s)  # noqa: E731
    assert abs(lp(5.0) - 1.2e-3) < tol and abs(lp(11.0) - 1.2e-3) < tol
    assert abs(lp(15.0) - 1.465e-3) < tol
    cd_max = (0.49 + 0.065 * 25.0) * 1e-3
    assert abs(lp(25.0) - cd_max) < tol and abs(lp(40.0) - cd_max) < tol
    wu = lambda s: lib.drag_coefficient(abi.DRAG_WU, 0.0, s)  # noqa: E731
    assert abs(wu(10.0) - 1.45e-3) < tol and abs(wu(20.0) - 2.1e-3) < tol
    assert abs(lib.drag_coefficient(abi.DRAG_SMITH, 0.0, 10.0) - 1.24e-3) < tol
    yt = lambda s: lib.drag_coefficient(abi.DRAG_YELLAND_TAYLOR, 0.0, s)  # noqa: E731
    assert abs(yt(6.0) - 1.1e-3) < tol and abs(yt(10.0) - 1.21e-3) < tol


def source(h, u, v, px=0.0, py=0.0, drag=abi.DRAG_LARGE_POND, h_min=0.01):
    out = (C.c_double * 2)()
    oracle_library().atmosphere_source(h, u, v, px, py, drag, 0.0, RHO_AIR, RHO_WATER, h_min, out)
    return out[0], out[1]


def test_wind_stress_known_answers():
    su, sv = source(10.0, 10.0, 0.0)
    # τ_x = 1.225 · 1.2e-3 · 10 · 10 = 0.147 N/m², / 1025
    assert abs(su - 1.435e-4) < 1e-6 and sv == 0.0
    d = 10.0 / math.sqrt(2.0)
    su, sv = source(10.0, d, d)
    assert abs(su - sv) < 1e-10
    assert source(0.001, 20.0, 10.0) == (0.0, 0.0)  # below h_min: not forced
    # stronger wind, more stress
    assert source(10.0, 15.0, 0.0)[0] > source(10.0, 10.0, 0.0)[0]
    # the pressure gradient alone: −h ∂p/∂x / ρ
    su, sv = source(20.0, 0.0, 0.0, 0.015, -0.01)
    assert su == -20.0 * 0.015 / RHO_WATER and sv == 20.0 * 0.01 / RHO_WATER


def test_inverse_barometer_level():
    lib = oracle_library()
    assert abs(lib.inverse_barometer_level(100.0, 1.0, RHO_WATER) + 100.0 / (RHO_WATER * G)) < 1e-15
    assert lib.inverse_barometer_level(100.0, 0.0, RHO_WATER) == 0.0


def box(order=2, sides=(TAG_WALL,) * 4):
    """The reference's atmosphere test mesh: ±10 km, 4 × 4 quads."""
    mesh = uniform_rectangle(-10_000.0, 10_000.0, -10_000.0, 10_000.0, 4, 4, sides=sides)
    return SWEDeviceForm2D(mesh=mesh, order=order, wet_dry=False, positivity_h_dry=None,
                           boundaries={TAG_WALL: WallBoundary()})


def uniform_weather(form, wind=(10.0, 0.0), gradient=(0.01, 0.02), pressure=(100.0, 100.0),
                    **kw):
    """Two snapshots an hour apart, each uniform over the nodes: the
    reference test's weather (wind (10, 0) m/s; pressure rising 1 then 2 hPa
    per 10 km to the east)."""
    n = form.n_values
    values = np.zeros((2, n, 5), dtype=np.float32)
    for s in range(2):
        values[s, :, 0], values[s, :, 1] = wind
        values[s, :, 2] = gradient[s]
        values[s, :, 4] = pressure[s]
    return GriddedAtmosphere(times=np.array([T0, T0 + 3600.0]), values=values, epoch_unix=T0, **kw)


def rhs(form, h, t):
    sim = oracle(form)
    try:
        z = np.zeros(form.n_values)
        sim.upload(np.full(form.n_values, h), z, z)
        return sim.compute_rhs_into(t)
    finally:
        sim.close()


def test_element_source_is_wind_stress_and_pressure_gradient():
    form = box()
    h = 20.0
    form = dataclasses.replace(form, atmosphere=uniform_weather(form))
    rh, rhu, rhv = rhs(form, h, 1800.0)
    stress = RHO_AIR * 1.2e-3 * 100.0 / RHO_WATER
    expected = stress - h * 0.015 / RHO_WATER  # ∂p/∂x = 1.5 · 0.01 Pa/m at half past
    assert np.abs(rhu - expected).max() < 1e-9
    assert np.abs(rhv).max() < 1e-12 and np.abs(rh).max() < 1e-12
    # pressure only, ramped over 2 h: −ramp·h·∂p/∂x/ρ
    lib = oracle_library()
    weather = dataclasses.replace(form.atmosphere, wind=False, ramp_duration=7200.0)
    rh, rhu, rhv = rhs(dataclasses.replace(form, atmosphere=weather), h, 1800.0)
    ramp = lib.tidal_ramp(1800.0, 7200.0)
    assert 0.0 < ramp < 1.0
    assert np.abs(rhu + ramp * h * 0.015 / RHO_WATER).max() < 1e-9
    # switched off as a source (only a level for the boundaries): nothing
    weather = dataclasses.replace(form.atmosphere, source=False)
    rh, rhu, rhv = rhs(dataclasses.replace(form, atmosphere=weather), h, 1800.0)
    assert np.abs(rhu).max() < 1e-12


def test_nodes_below_h_min_are_not_forced():
    form = box()
    form = dataclasses.replace(form, atmosphere=uniform_weather(form, gradient=(0.0, 0.0)))
    _, rhu, _ = rhs(form, 0.005, 1800.0)
    assert np.abs(rhu).max() < 1e-12


@pytest.mark.parametrize("factor", [1.0, 0.25])
def test_raise_is_the_level_added_to_the_external_elevation(factor):
    """A characteristic boundary raised by a uniform pressure anomaly's
    inverse-barometer level gives the RHS of the same boundary with that
    level as its mean elevation, bit for bit."""
    form = box(sides=(TAG_WALL, TAG_WALL, TAG_WALL, TAG_OPEN))
    form.bathymetry = np.full((form.mesh.n_elements, form.n_nodes), -20.0)  # at rest: η = 0
    p = 1500.0  # Pa
    weather = uniform_weather(form, wind=(0.0, 0.0), gradient=(0.0, 0.0), pressure=(p, p),
                              source=False)
    level = -1.0 * np.float64(np.float32(p)) / (RHO_WATER * G)
    raised = dataclasses.replace(
        form, atmosphere=weather,
        boundaries={TAG_WALL: WallBoundary(),
                    TAG_OPEN: TidalBoundary([], ramp_duration=None, raise_factor=factor)})
    plain = dataclasses.replace(
        form, boundaries={TAG_WALL: WallBoundary(),
                          TAG_OPEN: TidalBoundary([], mean_elevation=factor * level,
                                                  ramp_duration=None)})
    for t in (0.0, 1800.0):
        a, b = rhs(raised, 20.0, t), rhs(plain, 20.0, t)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    # the raised boundary is not at rest: a 15 hPa anomaly lowers it ≈ 15 cm
    assert np.abs(rhs(raised, 20.0, 0.0)[0]).max() > 0.0
    # without a pressure field (has_level false) the level is 0
    no_level = dataclasses.replace(raised, atmosphere=dataclasses.replace(weather,
                                                                          has_pressure=False))
    assert np.abs(rhs(no_level, 20.0, 0.0)[0]).max() == 0.0
