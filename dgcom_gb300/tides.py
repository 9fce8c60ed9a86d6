"""Tidal constituents of the harmonic open boundary, evaluated on the host
as the reference does (src/boundary/harmonic_tide.rs, src/tides/astronomy.rs):
a constituent's period is 360°/speed with the speed from its Doodson
coefficients and the secular rates of the mean longitudes (Meeus), not a
rounded period (12.42 h for M2 drifts ≈ 6° a year); with a run start, its
equilibrium argument and nodal corrections (``astronomy``)."""

from __future__ import annotations

import math

from . import abi

from .astronomy import ModelClock, angular_speed, canonical_name, constituent_period  # noqa: F401


def constituent(name: str, amplitude: float, phase_deg: float = 0.0,
                clock: ModelClock | None = None) -> abi.TideConstituent:
    """A constituent with phase lag ``phase_deg``: η = f A cos(ωt + V₀ + u − G).
    With a ``clock`` (the run's start in UTC) the lag is Greenwich's and
    V₀, f and u are the start's, f and u drifting through the run
    (HarmonicTide with NodalDrift); without one, f = 1 and V₀ = u = 0."""
    c = abi.TideConstituent()
    c.amplitude = amplitude
    c.period = constituent_period(name)
    c.phase = -math.radians(phase_deg)
    c.f, c.f_rate, c.u_deg, c.u_rate_deg, c.v0_deg = 1.0, 0.0, 0.0, 0.0, 0.0
    if clock is not None:
        d = clock.nodal_drift(name)
        c.f, c.u_deg, c.v0_deg = d.at_start.f, d.at_start.u_deg, d.at_start.v0_deg
        c.f_rate, c.u_rate_deg = d.f_rate, d.u_rate_deg
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
