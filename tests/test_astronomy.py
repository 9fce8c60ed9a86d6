"""Tidal astronomy (dgcom_gb300/astronomy.py) against the textbook values
the reference's tests hold its own to (src/tides/astronomy.rs:611-927,
src/time/clock.rs:143-215): Meeus' longitudes at J2000.0 and his Julian
date example, NOAA's tabulated speeds, S2's V₀ as solar time, the nodal
factors' extremes and families, Schureman's I and ξ, and the linear drift
through a run."""

import math

import pytest

from dgcom_gb300 import astronomy as A
from dgcom_gb300 import tides


def test_mean_longitudes_and_lunar_time_at_j2000():
    a = A.Arguments.at_julian_date(2_451_545.0)
    assert abs(a.s - 218.3164477) < 1e-4 and abs(a.h - 280.4664567) < 1e-4
    assert abs(a.p - 83.3530513) < 1e-3 and abs(a.n - 125.0445479) < 1e-4
    assert abs(a.p1 - 282.9373475) < 1e-3
    assert abs(a.tau - (15.0 * 12.0 + 280.4664567 - 218.3164477) % 360.0) < 1e-3


def test_julian_dates():
    assert abs(A.julian_date(1957, 10, 4, 19, 26, 24.0) - 2_436_116.31) < 1e-2  # Meeus 7.a
    assert abs(A.julian_date(2000, 1, 1, 12) - 2_451_545.0) < 1e-6
    clock = A.ModelClock("2000-01-01T12:00:00Z")
    assert abs(clock.julian_date(0.0) - 2_451_545.0) < 1e-9
    assert A.ModelClock("2025-06-01T00:00:00Z").epoch_unix == 1_748_736_000.0


SPEEDS = {"M2": 28.9841042, "S2": 30.0, "N2": 28.4397295, "K2": 30.0821373, "K1": 15.0410686,
          "O1": 13.9430356, "P1": 14.9589314, "Q1": 13.3986609, "M4": 57.9682084,
          "MS4": 58.9841042, "MN4": 57.4238337, "M6": 86.9523127, "Mf": 1.0980331,
          "Mm": 0.5443747, "Ssa": 0.0821373, "2N2": 27.8953548, "T2": 29.9589333,
          "MU2": 27.9682084, "NU2": 28.5125831, "LDA2": 29.4556253, "L2": 29.5284789}


def test_speeds_are_the_tabulated_ones():
    for name, speed in SPEEDS.items():
        assert abs(A.angular_speed(name) - speed) < 1e-6, name
        assert abs(A.constituent_period(name) * A.angular_speed(name) - 360.0 * 3600.0) < 1e-6
        assert A.canonical_name(name.lower()) == name
    assert abs(A.constituent_period("S2") - 12.0 * 3600.0) < 1e-9
    assert A.canonical_name("XX9") is None


def test_equilibrium_argument_advances_at_the_speed():
    jd0 = 2_451_545.0
    for name, period_h in [("M2", 12.4206012), ("S2", 12.0), ("N2", 12.6583482),
                           ("K2", 11.9672348), ("K1", 23.9344697), ("O1", 25.8193417),
                           ("P1", 24.0658902), ("Q1", 26.8683567), ("M4", 6.2103006),
                           ("M6", 4.1402004)]:
        v0 = A.nodal_correction(name, A.Arguments.at_julian_date(jd0)).v0_deg
        v1 = A.nodal_correction(name, A.Arguments.at_julian_date(jd0 + 1.0)).v0_deg
        rate = 360.0 / period_h * 24.0
        raw = v1 - v0
        raw += 360.0 * round((rate - raw) / 360.0)
        assert abs(360.0 / raw * 24.0 - period_h) < 1e-4, name


def test_s2_is_solar_time_and_solar_constituents_have_no_node():
    v0 = A.nodal_correction("S2", A.Arguments.at_julian_date(A.julian_date(2020, 6, 15))).v0_deg
    assert v0 < 1e-6 or abs(v0 - 360.0) < 1e-6
    v6 = A.nodal_correction("S2", A.Arguments.at_julian_date(A.julian_date(2020, 6, 15, 6)))
    assert abs(v6.v0_deg - 180.0) < 1e-6
    a = A.Arguments.at_julian_date(A.julian_date(2015, 3, 21))
    for name in ("S2", "P1", "Ssa"):
        c = A.nodal_correction(name, a)
        assert abs(c.f - 1.0) < 1e-12 and abs(c.u_deg) < 1e-12


def test_nodal_factor_extremes_and_families():
    f0, u0 = A.nodal_factors("M2", 0.0)
    f1, u1 = A.nodal_factors("M2", math.pi)
    assert abs(f0 - 0.9633) < 1e-3 and abs(u0) < 1e-12
    assert abs(f1 - 1.0379) < 1e-3 and abs(u1) < 1e-12
    assert abs(A.nodal_factors("K1", 0.0)[0] - 1.1128) < 1e-3
    assert abs(A.nodal_factors("K1", math.pi)[0] - 0.8816) < 1e-3
    assert abs(A.nodal_factors("O1", 0.0)[0] - 1.1827) < 1e-3
    assert abs(A.nodal_factors("O1", math.pi)[0] - 0.8057) < 1e-3
    a = A.Arguments.at_julian_date(A.julian_date(2010, 9, 1))
    m2, m4, m6 = (A.nodal_correction(n, a) for n in ("M2", "M4", "M6"))
    assert abs(m4.f - m2.f ** 2) < 1e-12 and abs(m6.f - m2.f ** 3) < 1e-12
    assert abs(m4.u_deg - 2 * m2.u_deg) < 1e-12 and abs(m6.u_deg - 3 * m2.u_deg) < 1e-12
    b = A.Arguments.at_julian_date(A.julian_date(2026, 6, 15))
    m2b = A.nodal_correction("M2", b)
    for name in ("N2", "2N2", "MU2", "NU2", "LDA2"):
        c = A.nodal_correction(name, b)
        assert (c.f, c.u_deg) == (m2b.f, m2b.u_deg)
    jd0 = A.julian_date(2000, 1, 1)
    f_a = A.nodal_correction("O1", A.Arguments.at_julian_date(jd0)).f
    f_b = A.nodal_correction("O1", A.Arguments.at_julian_date(jd0 + 6798.38)).f
    assert abs(f_a - f_b) < 2e-3  # one node cycle
    with pytest.raises(ValueError):
        A.nodal_correction("XYZ", a)


def test_lunar_intersection_and_l2():
    w, i = A.OBLIQUITY, A.MOON_INCLINATION
    incl, xi = A.lunar_intersection(0.0)
    assert abs(math.degrees(incl) - (w + i)) < 1e-9 and abs(xi) < 1e-12
    incl, xi = A.lunar_intersection(math.pi)
    assert abs(math.degrees(incl) - (w - i)) < 1e-9 and abs(xi) < 1e-9
    largest = max(abs(math.degrees(A.lunar_intersection(k / 3600 * 2 * math.pi)[1]))
                  for k in range(3600))
    assert abs(largest - 12.0) < 0.2
    for k in range(72):  # against Schureman's eqs. 213–214 written out
        n, p = math.radians(5.0 * k), math.radians(37.0 * k)
        incl, xi = A.lunar_intersection(n)
        t2 = math.tan(0.5 * incl) ** 2
        two_p = 2.0 * (p - xi)
        inv_ra = math.sqrt(1.0 - 12.0 * t2 * math.cos(two_p) + 36.0 * t2 * t2)
        r = math.degrees(math.atan2(math.sin(two_p), 1.0 / (6.0 * t2) - math.cos(two_p)))
        f, u = A.nodal_factors("L2", n, p)
        fm, um = A.nodal_factors("M2", n)
        assert abs(f - fm * inv_ra) < 1e-12 and abs(u - (um - r)) < 1e-9
    low = A.nodal_factors("L2", 0.0, 0.0)[0] / A.nodal_factors("M2", 0.0)[0]
    high = A.nodal_factors("L2", 0.0, 0.5 * math.pi)[0] / A.nodal_factors("M2", 0.0)[0]
    assert abs(low - 0.6104) < 1e-3 and abs(high - 1.3896) < 1e-3


def test_nodal_drift_follows_f_and_u():
    clock = A.ModelClock("2025-06-15T00:00:00Z")
    month, year = 30.0 * 86_400.0, 365.25 * 86_400.0
    for name, du_month, du_year, df_year in [("M2", 1e-3, 0.13, 2.5e-3), ("K1", 4e-3, 0.55, 7.5e-3)]:
        d = clock.nodal_drift(name)
        assert d.at(0.0) == A.nodal_correction(name, clock.arguments(0.0))
        for t, du in [(month, du_month), (year, du_year)]:
            exact = A.nodal_correction(name, clock.arguments(t))
            lin = d.at(t)
            assert abs(lin.u_deg - exact.u_deg) < du and abs(lin.f - exact.f) < df_year


def test_a_started_tide_carries_its_corrections():
    clock = A.ModelClock("2022-01-01T00:00:00Z")
    c = tides.constituent("K1", 0.1, 45.0, clock)
    d = clock.nodal_drift("K1")
    assert (c.f, c.u_deg, c.v0_deg) == (d.at_start.f, d.at_start.u_deg, d.at_start.v0_deg)
    assert 0.8 < c.f < 1.2
    # one period later the constituent repeats (f and u held)
    period = A.constituent_period("K1")
    e0 = c.f * c.amplitude * math.cos(c.phase + math.radians(c.v0_deg + c.u_deg))
    e1 = c.f * c.amplitude * math.cos(2 * math.pi + c.phase + math.radians(c.v0_deg + c.u_deg))
    assert abs(e0 - e1) < 1e-12 and abs(period / 3600.0 - 23.9344697) < 1e-6
