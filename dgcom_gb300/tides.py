"""Tidal constituents of the harmonic open boundary, evaluated on the host
as the reference does (src/boundary/harmonic_tide.rs, src/tides/astronomy.rs):
a constituent's period is 360°/speed with the speed from its Doodson
coefficients and the secular rates of the mean longitudes (Meeus), not a
rounded period (12.42 h for M2 drifts ≈ 6° a year)."""

from __future__ import annotations

import math

from . import abi

# Secular rates of the mean longitudes, degrees per Julian century (Meeus):
# the Moon's s, the Sun's h, the Moon's perigee p (from s − p' with the
# Moon's mean anomaly), the Sun's perigee p1 (from h − the Sun's anomaly)
S_PER_CENTURY = 481_267.881_234_21
H_PER_CENTURY = 36_000.769_827_79
MP_PER_CENTURY = 477_198.867_505_5
M_PER_CENTURY = 35_999.050_290_9
HOURS_PER_CENTURY = 36_525.0 * 24.0

# Doodson coefficients (τ, s, h, p, p1) of the constituents the workloads use
DOODSON = {
    "M2": (2.0, 0.0, 0.0, 0.0, 0.0),
    "S2": (2.0, 2.0, -2.0, 0.0, 0.0),
    "N2": (2.0, -1.0, 0.0, 1.0, 0.0),
    "K2": (2.0, 2.0, 0.0, 0.0, 0.0),
    "K1": (1.0, 1.0, 0.0, 0.0, 0.0),
    "O1": (1.0, -1.0, 0.0, 0.0, 0.0),
    "P1": (1.0, 1.0, -2.0, 0.0, 0.0),
    "Q1": (1.0, -2.0, 0.0, 1.0, 0.0),
}


def angular_speed(name: str) -> float:
    """Degrees per mean solar hour: dV₀/dt with τ′ = 15 + h′ − s′."""
    c_tau, c_s, c_h, c_p, c_p1 = DOODSON[name]
    s = S_PER_CENTURY / HOURS_PER_CENTURY
    h = H_PER_CENTURY / HOURS_PER_CENTURY
    p = (S_PER_CENTURY - MP_PER_CENTURY) / HOURS_PER_CENTURY
    p1 = (H_PER_CENTURY - M_PER_CENTURY) / HOURS_PER_CENTURY
    tau = 15.0 + h - s
    return c_tau * tau + c_s * s + c_h * h + c_p * p + c_p1 * p1


def constituent_period(name: str) -> float:
    """Period in seconds, 360°/speed·3600."""
    return 360.0 / angular_speed(name) * 3600.0


def constituent(name: str, amplitude: float, phase_deg: float = 0.0) -> abi.TideConstituent:
    """A constituent with Greenwich lag ``phase_deg`` (η = A cos(ωt − G)),
    without nodal corrections."""
    c = abi.TideConstituent()
    c.amplitude = amplitude
    c.period = constituent_period(name)
    c.phase = -math.radians(phase_deg)
    c.f = 1.0
    c.f_rate = 0.0
    c.u_deg = 0.0
    c.u_rate_deg = 0.0
    c.v0_deg = 0.0
    return c


def tidal_ramp(t: float, duration: float | None) -> float:
    """Smooth start-up ramp 3τ² − 2τ³ (src/boundary/harmonic_tide.rs:24-32)."""
    if duration is None or not duration > 0.0:
        return 1.0
    tau = min(max(t / duration, 0.0), 1.0)
    return tau * tau * (3.0 - 2.0 * tau)


def elevation(constituents, t: float, mean: float = 0.0, ramp: float | None = None) -> float:
    """HarmonicTide::elevation (src/boundary/harmonic_tide.rs:124-136)."""
    tide = 0.0
    for c in constituents:
        f = c.f + c.f_rate * t
        u_deg = c.u_deg + c.u_rate_deg * t
        offset = (c.v0_deg + u_deg) * (math.pi / 180.0)
        tide += f * c.amplitude * math.cos(2.0 * math.pi / c.period * t + c.phase + offset)
    return mean + tidal_ramp(t, ramp) * tide
