"""Tidal astronomy for boundary tides given with Greenwich phase lags and a
model start time: each constituent's equilibrium argument V₀ at the start
and its nodal factor f and phase u, drifting linearly through the run.

The same published method as the reference (src/tides/astronomy.rs,
src/time/clock.rs:78-117), restated:

- mean longitudes s (Moon), h (Sun), p (lunar perigee, s − M′), N (lunar
  ascending node) and p₁ (solar perigee, h − M) from Meeus' polynomials in
  Julian centuries from J2000.0 (Astronomical Algorithms, 2nd ed., eqs.
  22.x, 25.2, 47.1–47.7), with UTC for TT; the mean lunar time
  τ = 15°·(UT hours) + h − s;
- V₀ = Doodson's integer combination of (τ, s, h, p, p₁) plus Schureman's
  offset (±90° for the diurnals, 180° for λ2 and L2);
- f and u from Schureman's (1958, US C&GS SP 98) closed forms in N per
  nodal family (M2, K1, O1, K2, Mf, Mm, powers of M2), and for L2 M2's
  times 1 − 6 tan²(I/2)·e^{2i(p − ξ)} with the lunar orbit's inclination I
  to the equator and ξ from Schureman's eqs. 191–197;
- f(t) = f₀ + ḟ t and u(t) = u₀ + u̇ t, the rates by central differences
  over ±1 day, V₀ fixed at the start (NodalDrift).

The coefficients are the published ones (Meeus, Schureman, Doodson), so
they are necessarily the reference's too."""

from __future__ import annotations

import math
from dataclasses import dataclass
from datetime import datetime, timezone

# Secular rates of the mean longitudes, degrees per Julian century (Meeus)
S_RATE = 481_267.881_234_21   # Moon's mean longitude L′ (47.1)
H_RATE = 36_000.769_827_79    # Sun's mean longitude L₀ (25.2)
MP_RATE = 477_198.867_505_5   # Moon's mean anomaly M′ (47.4)
M_RATE = 35_999.050_290_9     # Sun's mean anomaly M (47.3)
HOURS_PER_CENTURY = 36_525.0 * 24.0
J2000 = 2_451_545.0
UNIX_EPOCH_JD = 2_440_587.5

OBLIQUITY = 23.452       # ω, Schureman (degrees)
MOON_INCLINATION = 5.145  # i of the Moon's orbit to the ecliptic (degrees)

# name → (Doodson coefficients of τ, s, h, p, p₁; offset in degrees; nodal family)
CONSTITUENTS = {
    "M2": ((2, 0, 0, 0, 0), 0.0, "M2"),
    "S2": ((2, 2, -2, 0, 0), 0.0, None),
    "N2": ((2, -1, 0, 1, 0), 0.0, "M2"),
    "K2": ((2, 2, 0, 0, 0), 0.0, "K2"),
    "2N2": ((2, -2, 0, 2, 0), 0.0, "M2"),
    "MU2": ((2, -2, 2, 0, 0), 0.0, "M2"),
    "NU2": ((2, -1, 2, -1, 0), 0.0, "M2"),
    "LDA2": ((2, 1, -2, 1, 0), 180.0, "M2"),
    "L2": ((2, 1, 0, -1, 0), 180.0, "L2"),
    "T2": ((2, 2, -3, 0, 1), 0.0, None),
    "K1": ((1, 1, 0, 0, 0), 90.0, "K1"),
    "O1": ((1, -1, 0, 0, 0), -90.0, "O1"),
    "P1": ((1, 1, -2, 0, 0), -90.0, None),
    "Q1": ((1, -2, 0, 1, 0), -90.0, "O1"),
    "M4": ((4, 0, 0, 0, 0), 0.0, 2),
    "MS4": ((4, 2, -2, 0, 0), 0.0, "M2"),
    "MN4": ((4, -1, 0, 1, 0), 0.0, 2),
    "M6": ((6, 0, 0, 0, 0), 0.0, 3),
    "Mf": ((0, 2, 0, 0, 0), 0.0, "Mf"),
    "Mm": ((0, 1, 0, -1, 0), 0.0, "Mm"),
    "Ssa": ((0, 0, 2, 0, 0), 0.0, None),
}


def canonical_name(name: str) -> str | None:
    """The conventional spelling of a supported constituent, matched
    case-insensitively; None if it is not supported."""
    key = name.strip().upper()
    for c in CONSTITUENTS:
        if c.upper() == key:
            return c
    return None


def _wrap(x: float) -> float:
    r = math.fmod(x, 360.0)
    return r + 360.0 if r < 0.0 else r


def julian_date(year: int, month: int, day: int, hour: int = 0, minute: int = 0,
                second: float = 0.0) -> float:
    """Julian Date of a Gregorian UTC instant (Meeus 7.1)."""
    y, m = (year - 1, month + 12) if month <= 2 else (year, month)
    a = math.floor(y / 100.0)
    b = 2.0 - a + math.floor(a / 4.0)
    frac = (hour + minute / 60.0 + second / 3600.0) / 24.0
    return math.floor(365.25 * (y + 4716.0)) + math.floor(30.6001 * (m + 1.0)) + day + b \
        - 1524.5 + frac


@dataclass
class Arguments:
    """Mean longitudes and the mean lunar time (degrees, in [0, 360))."""
    tau: float
    s: float
    h: float
    p: float
    n: float
    p1: float

    @staticmethod
    def at_julian_date(jd: float) -> "Arguments":
        t = (jd - J2000) / 36_525.0
        t2, t3, t4 = t * t, t * t * t, t * t * t * t
        s = 218.316_447_7 + S_RATE * t - 0.001_578_6 * t2 + t3 / 538_841.0 - t4 / 65_194_000.0
        h = 280.466_456_7 + H_RATE * t + 0.000_303_2 * t2
        mp = 134.963_396_4 + MP_RATE * t + 0.008_741_4 * t2 + t3 / 69_699.0 - t4 / 14_712_000.0
        m = 357.529_109_2 + M_RATE * t - 0.000_153_6 * t2 + t3 / 24_490_000.0
        node = 125.044_547_9 - 1_934.136_289_1 * t + 0.002_075_4 * t2 + t3 / 467_441.0 \
            - t4 / 60_616_000.0
        ut_hours = math.fmod(jd + 0.5, 1.0) * 24.0
        if ut_hours < 0.0:
            ut_hours += 24.0
        return Arguments(_wrap(15.0 * ut_hours + h - s), _wrap(s), _wrap(h), _wrap(s - mp),
                         _wrap(node), _wrap(h - m))


def angular_speed(name: str) -> float:
    """Degrees per mean solar hour: dV₀/dt from the longitudes' secular
    rates (τ′ = 15 + h′ − s′)."""
    c = CONSTITUENTS[canonical_name(name)][0]
    s = S_RATE / HOURS_PER_CENTURY
    h = H_RATE / HOURS_PER_CENTURY
    p = (S_RATE - MP_RATE) / HOURS_PER_CENTURY
    p1 = (H_RATE - M_RATE) / HOURS_PER_CENTURY
    tau = 15.0 + h - s
    return c[0] * tau + c[1] * s + c[2] * h + c[3] * p + c[4] * p1


def constituent_period(name: str) -> float:
    """Seconds: 360° / speed."""
    return 360.0 / angular_speed(name) * 3600.0


def lunar_intersection(n_rad: float) -> tuple[float, float]:
    """I and ξ (radians) at node longitude N (Schureman eqs. 191–197):
    cos I = cos ω cos i − sin ω sin i cos N and
    tan ½(N − ξ ± ν) = cos|sin ½(ω − i) / cos|sin ½(ω + i) · tan ½N."""
    w, i = math.radians(OBLIQUITY), math.radians(MOON_INCLINATION)
    incl = math.acos(math.cos(w) * math.cos(i) - math.sin(w) * math.sin(i) * math.cos(n_rad))
    n = math.pi - (math.pi - n_rad) % (2.0 * math.pi)  # N in (−π, π]: ½N on atan's branch
    t = math.tan(0.5 * n)
    a = math.atan(math.cos(0.5 * (w - i)) / math.cos(0.5 * (w + i)) * t)
    b = math.atan(math.sin(0.5 * (w - i)) / math.sin(0.5 * (w + i)) * t)
    return incl, n - (a + b)


def _m2(n: float) -> tuple[float, float]:
    return 1.0004 - 0.0373 * math.cos(n) + 0.0002 * math.cos(2 * n), -2.14 * math.sin(n)


def nodal_factors(family, n: float, p: float = 0.0) -> tuple[float, float]:
    """f and u (degrees) of a nodal family at node longitude N and lunar
    perigee p (radians; p only for L2)."""
    c, c2, c3 = math.cos(n), math.cos(2 * n), math.cos(3 * n)
    s, s2, s3 = math.sin(n), math.sin(2 * n), math.sin(3 * n)
    if family is None:
        return 1.0, 0.0
    if family == "M2":
        return _m2(n)
    if isinstance(family, int):
        f, u = _m2(n)
        return f ** family, family * u
    if family == "K1":
        return 1.0060 + 0.1150 * c - 0.0088 * c2 + 0.0006 * c3, -8.86 * s + 0.68 * s2 - 0.07 * s3
    if family == "O1":
        return 1.0089 + 0.1871 * c - 0.0147 * c2 + 0.0014 * c3, 10.80 * s - 1.34 * s2 + 0.19 * s3
    if family == "K2":
        return (1.0241 + 0.2863 * c + 0.0083 * c2 - 0.0015 * c3,
                -17.74 * s + 0.68 * s2 - 0.04 * s3)
    if family == "Mf":
        return 1.0429 + 0.4135 * c - 0.004 * c2, -23.7 * s + 2.7 * s2 - 0.4 * s3
    if family == "Mm":
        return 1.0 - 0.1300 * c + 0.0013 * c2, 0.0
    if family == "L2":
        fm, um = _m2(n)
        incl, xi = lunar_intersection(n)
        k = 6.0 * math.tan(0.5 * incl) ** 2
        two_p = 2.0 * (p - xi)
        re, im = 1.0 - k * math.cos(two_p), -k * math.sin(two_p)
        return fm * math.hypot(re, im), um + math.degrees(math.atan2(im, re))
    raise ValueError(f"unknown nodal family {family!r}")


@dataclass
class NodalCorrection:
    f: float
    u_deg: float
    v0_deg: float


def nodal_correction(name: str, a: Arguments) -> NodalCorrection:
    cname = canonical_name(name)
    if cname is None:
        raise ValueError(f"unsupported tidal constituent {name!r}")
    coef, offset, family = CONSTITUENTS[cname]
    v0 = _wrap(coef[0] * a.tau + coef[1] * a.s + coef[2] * a.h + coef[3] * a.p
               + coef[4] * a.p1 + offset)
    f, u = nodal_factors(family, math.radians(a.n), math.radians(a.p))
    return NodalCorrection(f, u, v0)


@dataclass
class NodalDrift:
    """f, u and V₀ at the start, and the rates of f and u (per second)."""
    at_start: NodalCorrection
    f_rate: float
    u_rate_deg: float

    def at(self, t: float) -> NodalCorrection:
        return NodalCorrection(self.at_start.f + self.f_rate * t,
                               self.at_start.u_deg + self.u_rate_deg * t, self.at_start.v0_deg)


class ModelClock:
    """Model time t (s) against UTC: t = 0 at ``start`` (ISO 8601, e.g.
    ``2025-06-15T00:00:00Z``)."""

    DAY = 86_400.0

    def __init__(self, start: str):
        text = start.strip()
        if text.endswith("Z") or text.endswith("z"):
            text = text[:-1] + "+00:00"
        try:
            when = datetime.fromisoformat(text)
        except ValueError:
            raise ValueError(f"run.start: not an ISO 8601 UTC time: {start!r}") from None
        if when.tzinfo is None:
            when = when.replace(tzinfo=timezone.utc)
        self.epoch_unix = when.timestamp()

    def julian_date(self, t: float) -> float:
        return UNIX_EPOCH_JD + (self.epoch_unix + t) / self.DAY

    def arguments(self, t: float) -> Arguments:
        return Arguments.at_julian_date(self.julian_date(t))

    def nodal_drift(self, name: str) -> NodalDrift:
        before = nodal_correction(name, self.arguments(-self.DAY))
        at = nodal_correction(name, self.arguments(0.0))
        after = nodal_correction(name, self.arguments(self.DAY))
        return NodalDrift(at, (after.f - before.f) / (2.0 * self.DAY),
                          (after.u_deg - before.u_deg) / (2.0 * self.DAY))
