"""Analytic solutions the reference's own tests run the 2D SWE against,
restated for any physics with the ABI (the oracle, or the CUDA library):

- Thacker's planar oscillation in a paraboloid (tests/wet_dry_2d_test.rs:
  214-320, SWASHES parameters): the wet disc slides round the bowl, so the
  shoreline wets and dries everywhere. One period on an n × n P2 mesh with
  the wet/dry treatment at h_dry = 1e-5 m; the relative L1 depth error, the
  largest speed where h > 1 cm, the mass drift and the lowest depth.
- A travelling vortex on periodic meshes for the convergence orders of the
  split forms (tests/convergence_test.rs:1024-1240 measures them on a
  manufactured solution whose source term has no device form, so a source-
  free exact solution stands in: a cyclostrophic vortex h(r) = 1 −
  β²/(16π²g)·e^{2(1−r²)}, v_θ = (β/2π)·r·e^{1−r²}, carried by a uniform
  flow on a flat bed), on the reference's periodic meshes, uniform or
  distorted."""

from __future__ import annotations

import math

import numpy as np

from dgcom_gb300 import abi
from dgcom_gb300.device import DeviceRun
from dgcom_gb300.mesh import (TAG_WALL, QuadMesh, node_mass, node_positions, uniform_periodic,
                              uniform_rectangle)
from dgcom_gb300.physics import SWEDeviceForm2D, WallBoundary

G = 9.81


# -- Thacker ------------------------------------------------------------------

class Thacker:
    """Thacker (1981) planar surface in a paraboloid, SWASHES parameters
    (Delestre et al. 2013): a = 1, h0 = 0.1, η = 0.5, L = 4."""

    a, h0, eta, length = 1.0, 0.1, 0.5, 4.0

    @property
    def omega(self) -> float:
        return math.sqrt(2.0 * G * self.h0) / self.a

    @property
    def period(self) -> float:
        return 2.0 * math.pi / self.omega

    def bed(self, x, y):
        r2 = (x - 0.5 * self.length) ** 2 + (y - 0.5 * self.length) ** 2
        return -self.h0 * (1.0 - r2 / (self.a * self.a))

    def exact(self, x, y, t):
        w = self.omega
        xc, yc = x - 0.5 * self.length, y - 0.5 * self.length
        surface = self.eta * self.h0 / (self.a * self.a) * (
            2.0 * xc * math.cos(w * t) + 2.0 * yc * math.sin(w * t) - self.eta)
        h = surface - self.bed(x, y)
        wet = h > 0.0
        h = np.where(wet, h, 0.0)
        u = np.where(wet, -self.eta * w * math.sin(w * t), 0.0)
        v = np.where(wet, self.eta * w * math.cos(w * t), 0.0)
        return h, h * u, h * v


def thacker_form(n: int, numerics: int = abi.NUMERICS_FAST) -> SWEDeviceForm2D:
    """The reference's wet/dry Thacker setup: walls, P2, the WetDry split
    form with h_dry = 1e-5 m for the subcells, the wet/dry correction and
    the positivity-bounded step (the redundant positivity limiter of a
    wet/dry run), no friction, no Coriolis."""
    case = Thacker()
    mesh = uniform_rectangle(0.0, case.length, 0.0, case.length, n, n)
    form = SWEDeviceForm2D(mesh=mesh, order=2, g=G, formulation=abi.WET_DRY, subcell_depth=1e-5,
                           subcell_h_dry=1e-5, wet_dry=True, h_dry=1e-5, positivity_h_dry=1e-5,
                           boundaries={TAG_WALL: WallBoundary()}, numerics=numerics,
                           line_local_depth=None)
    x, y = node_positions(mesh, 2)
    form.bathymetry = case.bed(x, y)
    return form


def thacker_one_period(make, n: int, numerics: int = abi.NUMERICS_FAST):
    """(relative L1 depth error, max speed where h > 1 cm, mass drift,
    lowest depth seen, negative-depth clips) after one period at CFL 1."""
    case = Thacker()
    form = thacker_form(n, numerics)
    x, y = node_positions(form.mesh, 2)
    q0 = [a.reshape(-1) for a in case.exact(x, y, 0.0)]
    mass = node_mass(form.mesh, 2).reshape(-1)
    lowest = [float(q0[0].min())]

    def watch(t, h, hu, hv):
        lowest[0] = min(lowest[0], float(h.min()))

    sim = make(form)
    try:
        sim.upload(*q0)
        rep = sim.run_with_callback(DeviceRun(span=(0.0, case.period), cfl=1.0,
                                              interval=case.period / 64.0), watch)
        assert rep.success, rep.message
        h, hu, hv = sim.download()
    finally:
        sim.close()
    lowest[0] = min(lowest[0], float(h.min()))
    he = case.exact(x, y, case.period)[0].reshape(-1)
    exact_mass = float(np.sum(mass * he))
    error = float(np.sum(mass * np.abs(h - he))) / exact_mass
    wet = h > 1e-2
    speed = float((np.hypot(hu[wet], hv[wet]) / h[wet]).max())
    drift = abs(float(np.sum(mass * h)) - float(np.sum(mass * q0[0]))) / float(np.sum(mass * q0[0]))
    return error, speed, drift, lowest[0], rep.negative_depth_clips


# -- travelling vortex ----------------------------------------------------------

BETA, U_INF, V_INF, SIDE = 5.0, 1.0, 0.5, 10.0


def periodic_mesh(n: int, distorted: bool) -> QuadMesh:
    """periodic_mesh (tests/convergence_test.rs:1024-1039) on [−L/2, L/2]²:
    Mesh2D::uniform_periodic, its vertices moved by periodic bumps if
    distorted."""
    side = SIDE
    mesh = uniform_periodic(0.0, side, 0.0, side, n, n)
    if distorted:
        tau, a = 2.0 * math.pi / side, 0.04 * side
        v = mesh.vertices.copy()
        x, y = v[:, 0].copy(), v[:, 1].copy()
        sx, sy = np.sin(tau * x), np.sin(tau * y)
        v[:, 0] = x + a * sx * sy + 0.5 * a * np.sin(tau * y)
        v[:, 1] = y - 0.7 * a * sx * sy + 0.4 * a * np.sin(tau * x)
        mesh = QuadMesh(v, mesh.elements, mesh.periodic, mesh.face_tags)
    return mesh


def vortex(x, y, t):
    """The vortex centred at (L/2, L/2) at t = 0, carried by (U∞, V∞), its
    centre's nearest periodic image (the state is e^{−40}-small at the
    box's edge)."""
    xc = 0.5 * SIDE + U_INF * t
    yc = 0.5 * SIDE + V_INF * t
    dx = (x - xc + 0.5 * SIDE) % SIDE - 0.5 * SIDE
    dy = (y - yc + 0.5 * SIDE) % SIDE - 0.5 * SIDE
    r2 = dx * dx + dy * dy
    e = np.exp(1.0 - r2)
    h = 1.0 - BETA * BETA / (16.0 * math.pi * math.pi * G) * e * e
    u = U_INF - BETA / (2.0 * math.pi) * e * dy
    v = V_INF + BETA / (2.0 * math.pi) * e * dx
    return h, h * u, h * v


def vortex_form(n: int, order: int, formulation: int, distorted: bool,
                numerics: int = abi.NUMERICS_FAST) -> SWEDeviceForm2D:
    mesh = periodic_mesh(n, distorted)
    return SWEDeviceForm2D(mesh=mesh, order=order, g=G, formulation=formulation,
                           wet_dry=False, positivity_h_dry=None, numerics=numerics,
                           line_local_depth=None, boundaries={TAG_WALL: WallBoundary()})


def vortex_error(make, n: int, order: int, formulation: int, distorted: bool, cfl: float,
                 t_final: float = 0.5, numerics: int = abi.NUMERICS_FAST) -> float:
    """The L2 depth error at t_final of SSP-RK3 steps of equal length (the
    first step's CFL step, fitted to land on t_final), as the reference's
    convergence runs take them."""
    form = vortex_form(n, order, formulation, distorted, numerics)
    x, y = node_positions(form.mesh, order)
    q0 = [a.reshape(-1) for a in vortex(x, y, 0.0)]
    mass = node_mass(form.mesh, order).reshape(-1)
    sim = make(form)
    try:
        sim.upload(*q0)
        dt0 = sim.compute_dt_ssp(cfl)
        steps = max(1, math.ceil(t_final / dt0))
        dt = t_final / steps
        t = 0.0
        for _ in range(steps):
            sim.step(t, dt)
            t += dt
        h = sim.download()[0]
    finally:
        sim.close()
    he = vortex(x, y, t_final)[0].reshape(-1)
    return math.sqrt(float(np.sum(mass * (h - he) ** 2)))


def observed_orders(errors):
    return [math.log2(a / b) for a, b in zip(errors, errors[1:])]
