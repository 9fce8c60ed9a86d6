"""The discrete adjoint through the C ABI against finite differences of
the oracle (the CPU restatement of the reference forward).

J = Σ over steps and stations of η², on the tidal channel after its tide
ramp, with Manning's n per element. The forward's time steps are replayed
in the oracle: the adjoint is the derivative of the steps taken. Each
directional derivative g·d must match the central difference
(J(p+εd) − J(p−εd))/(2ε) to REL, with ε per parameter (a relative 1e-7 for
the state, 1e-6 for the bed, 1e-4 for n and the tide: a smaller step than
the curvature needs drowns the difference in J's rounding).

With a drying flat the run is not differentiable everywhere: dry nodes sit
at h = 0 exactly, where max(h, 0) and the dry tests have a kink, so the
one-sided differences differ there and the central one averages them. The
adjoint takes the branch each kink's forward took. Directions that do not
reach the shoreline within the run, and the parameters whose effect there
is small, are held to REL; at the shoreline the adjoint must lie within the
spread of the one-sided differences."""

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.adjoint import Adjoint
from dgcom_gb300.physics import TidalBoundary
from oracle_lib import oracle

pytestmark = pytest.mark.gpu

REL = 1e-6
STEPS = 8
T_START = 4000.0  # past the tide's one-hour ramp
STATIONS = [(2_000.0, 2_500.0), (10_000.0, 1_200.0), (25_000.0, 2_500.0), (40_000.0, 3_700.0),
            (47_000.0, 2_500.0)]
OPEN = 1  # the open boundary's index (conditions sorted by tag)


def setup(order: int, wet: bool, numerics=abi.NUMERICS_FAST):
    case = cases.tidal_channel(nx=24, ny=3, order=order, numerics=numerics)
    form = case.form
    if wet:
        form.bathymetry = form.bathymetry - 5.0  # 4 m at the shallow end: no drying
    rng = np.random.default_rng(7)
    n_el = rng.uniform(0.015, 0.035, form.mesh.n_elements)
    form.manning_n = np.repeat(n_el, (order + 1) ** 2)
    state = cases.with_flow(case, eta_amp=0.4, u=0.4, v=0.05)
    return case, form, state


def oracle_J(form, state, dts, elem, w):
    ref = oracle(form)
    try:
        ref.upload(*state)
        nn = w.shape[1]
        b = form.bathymetry.reshape(-1)
        t = T_START
        J = 0.0
        for dt in dts:
            ref.step(t, dt)
            t += dt
            h = ref.download()[0]
            for s in range(len(elem)):
                sl = slice(elem[s] * nn, (elem[s] + 1) * nn)
                J += float(np.dot(w[s], h[sl] + b[sl])) ** 2
    finally:
        ref.close()
    return J


def with_tide(form, amplitude=None, phase=None):
    bc = form.boundaries[OPEN]
    cons = list(bc.constituents)
    c0 = type(cons[0])()
    for name, _ in type(c0)._fields_:
        setattr(c0, name, getattr(cons[0], name))
    if amplitude is not None:
        c0.amplitude = amplitude
    if phase is not None:
        c0.phase = phase
    cons[0] = c0
    new = dict(form.boundaries)
    new[OPEN] = TidalBoundary(cons, mean_elevation=bc.mean_elevation,
                              ramp_duration=bc.ramp_duration, incoming_wave=bc.incoming_wave)
    import dataclasses

    return dataclasses.replace(form, boundaries=new)


def central(f, eps):
    return (f(eps) - f(-eps)) / (2.0 * eps)


def check(name, adj, fd, rel):
    err = abs(adj - fd) / max(abs(fd), abs(adj), 1e-300)
    assert err <= rel, f"{name}: adjoint {adj:.12e} fd {fd:.12e} rel {err:.2e}"


def run(form, state, steps=STEPS):
    with Adjoint(form, steps, STATIONS, cfl=0.5, t_start=T_START) as adj:
        J, eta, dts = adj.forward(state)
        elem, w = adj.station_weights()
        g = adj.reverse()
    return J, dts, elem, w, g


@pytest.mark.parametrize("order", [2, 3])
def test_gradient_matches_oracle_finite_differences_wet(order):
    import dataclasses

    case, form, state = setup(order, True)
    nn = (order + 1) ** 2
    J, dts, elem, w, g = run(form, state)
    assert np.all(dts > 0.0)
    J0 = oracle_J(form, state, dts, elem, w)
    assert abs(J - J0) <= 1e-10 * abs(J0)  # the device forward is the oracle's
    rng = np.random.default_rng(11)
    for k, name in [(0, "h0"), (1, "hu0"), (2, "hv0")]:
        d = rng.standard_normal(state[0].size)
        eps = 1e-7 * float(np.abs(state[k]).max())

        def J_of(e, k=k, d=d):
            st = list(state)
            st[k] = state[k] + e * d
            return oracle_J(form, tuple(st), dts, elem, w)

        check(name, float(np.dot([g.h0, g.hu0, g.hv0][k], d)), central(J_of, eps), REL)
    n0 = np.asarray(form.manning_n)
    d_el = rng.standard_normal(form.mesh.n_elements)
    d = np.repeat(d_el, nn)
    fd = central(lambda e: oracle_J(dataclasses.replace(form, manning_n=n0 + e * d), state, dts,
                                    elem, w), 1e-4 * float(n0.max()))
    check("manning", float(np.dot(g.manning_per_element(nn), d_el)), fd, REL)
    x, y = form.positions()
    d = np.sin(x.reshape(-1) / 7_000.0) * np.cos(y.reshape(-1) / 3_000.0)
    b0 = form.bathymetry.reshape(-1)
    fd = central(lambda e: oracle_J(dataclasses.replace(form, bathymetry=(b0 + e * d).reshape(
        form.bathymetry.shape)), state, dts, elem, w), 1e-6 * float(np.abs(b0).max()))
    check("bed", float(np.dot(g.bed, d)), fd, REL)
    c0 = form.boundaries[OPEN].constituents[0]
    fd = central(lambda e: oracle_J(with_tide(form, amplitude=c0.amplitude + e), state, dts, elem,
                                    w), 1e-4 * c0.amplitude)
    check("amplitude", float(g.tide[OPEN, 0, 0]), fd, REL)
    fd = central(lambda e: oracle_J(with_tide(form, phase=c0.phase + e), state, dts, elem, w), 1e-4)
    check("phase", float(g.tide[OPEN, 0, 1]), fd, REL)


def test_gradient_with_a_drying_flat():
    import dataclasses

    case, form, state = setup(2, False)
    nn = 9
    J, dts, elem, w, g = run(form, state)
    x, y = form.positions()
    x = x.reshape(-1)
    rng = np.random.default_rng(3)
    h0 = state[0]
    wet = h0 > 1e-3
    # away from the shoreline (x < 40 km; the flat dries near 48 km)
    for k, name in [(0, "h0"), (1, "hu0")]:
        d = rng.standard_normal(h0.size) * wet * (x < 40e3)
        eps = 1e-7 * float(np.abs(state[k]).max())

        def J_of(e, k=k, d=d):
            st = list(state)
            st[k] = state[k] + e * d
            return oracle_J(form, tuple(st), dts, elem, w)

        check(name + " far", float(np.dot([g.h0, g.hu0][k], d)), central(J_of, eps), REL)
    # the tide and Manning's n everywhere, the bed everywhere (a continuous field)
    c0 = form.boundaries[OPEN].constituents[0]
    fd = central(lambda e: oracle_J(with_tide(form, amplitude=c0.amplitude + e), state, dts, elem,
                                    w), 1e-4 * c0.amplitude)
    check("amplitude", float(g.tide[OPEN, 0, 0]), fd, REL)
    fd = central(lambda e: oracle_J(with_tide(form, phase=c0.phase + e), state, dts, elem, w), 1e-4)
    check("phase", float(g.tide[OPEN, 0, 1]), fd, REL)
    n0 = np.asarray(form.manning_n)
    d_el = rng.standard_normal(form.mesh.n_elements)
    d = np.repeat(d_el, nn)
    fd = central(lambda e: oracle_J(dataclasses.replace(form, manning_n=n0 + e * d), state, dts,
                                    elem, w), 1e-4 * float(n0.max()))
    check("manning", float(np.dot(g.manning_per_element(nn), d_el)), fd, REL)
    xx, yy = form.positions()
    d = np.sin(xx.reshape(-1) / 7_000.0) * np.cos(yy.reshape(-1) / 3_000.0)
    b0 = form.bathymetry.reshape(-1)
    fd = central(lambda e: oracle_J(dataclasses.replace(form, bathymetry=(b0 + e * d).reshape(
        form.bathymetry.shape)), state, dts, elem, w), 1e-6 * float(np.abs(b0).max()))
    check("bed", float(np.dot(g.bed, d)), fd, 10 * REL)


def test_gradient_through_the_wet_dry_paths():
    """Thin films instead of dry land (h of 2e-4 to 8e-4 m, between h_min
    and h_dry) and a seeded generic state (no node exactly at a threshold,
    no ties in a minimum, a maximum or a limiter's extremum test): the subcell volume term, the wet/dry
    limiter, thin-layer damping and desingularisation all run, and the run
    is differentiable at the base point, so the central differences hold
    the adjoint to REL along directions that cover the films."""
    import dataclasses

    case, form, state = setup(2, False)
    film = state[0] < 1e-3
    rng = np.random.default_rng(17)
    # a generic state: the flowing one is uniform across the channel, so
    # nodes at one x are equal and the subcell limiter sits on its kink
    h_film = rng.uniform(2e-4, 8e-4, film.size)  # distinct depths: no ties in a minimum
    wet_h = state[0] * (1.0 + 0.02 * rng.standard_normal(film.size))
    h0 = np.where(film, h_film, wet_h)
    u0 = np.where(film, rng.uniform(-0.05, 0.05, film.size), 0.4 + 0.05 * rng.standard_normal(film.size))
    v0 = np.where(film, rng.uniform(-0.05, 0.05, film.size), 0.05 * rng.standard_normal(film.size))
    hu0 = h0 * u0
    hv0 = h0 * v0
    st0 = (h0, hu0, hv0)
    J, dts, elem, w, g = run(form, st0)
    x, _ = form.positions()
    x = x.reshape(-1)
    rng = np.random.default_rng(5)
    near = x > 44e3
    for k, name in [(0, "h0"), (1, "hu0")]:
        d = rng.standard_normal(h0.size) * near
        if k == 0:
            d = d * np.where(film, 1e-4, 1.0)  # the films stay between the thresholds
        eps = 1e-7 * float(np.abs(st0[k]).max())

        def J_of(e, k=k, d=d):
            st = list(st0)
            st[k] = st0[k] + e * d
            return oracle_J(form, tuple(st), dts, elem, w)

        check(name + " shore", float(np.dot([g.h0, g.hu0][k], d)), central(J_of, eps), REL)


def test_checkpoint_segments_give_the_same_gradient():
    case, form, state = setup(2, False)
    with Adjoint(form, STEPS, STATIONS, t_start=T_START) as full:
        full.forward(state)
        g1 = full.reverse()
        assert full.stats().stride == 1
    state_bytes = 3 * 8 * state[0].size
    # step-start segments: each step's stages computed twice in the reverse
    with Adjoint(form, STEPS, STATIONS, t_start=T_START, memory_budget=6.5 * state_bytes) as seg:
        seg.forward(state)
        g2 = seg.reverse()
        st = seg.stats()
        assert st.stride > 1 and not st.full_segments and st.recomputed_steps > STEPS
    # full segments every 4 steps: each step computed once
    with Adjoint(form, STEPS, STATIONS, t_start=T_START, memory_budget=44 * state_bytes,
                 checkpoint_every=4) as seg:
        seg.forward(state)
        g3 = seg.reverse()
        st = seg.stats()
        assert st.stride == 4 and st.full_segments and st.recomputed_steps == STEPS
    for g in (g2, g3):
        for a, b in [(g1.h0, g.h0), (g1.bed, g.bed), (g1.manning, g.manning)]:
            assert np.abs(a - b).max() <= 1e-12 * max(np.abs(a).max(), 1e-300)


def test_replayed_steps_give_the_recorded_functional():
    case, form, state = setup(3, True)
    with Adjoint(form, STEPS, STATIONS, t_start=T_START) as adj:
        J, eta, dts = adj.forward(state)
        J2, eta2, dts2 = adj.forward(state, dts=dts)
    assert np.array_equal(dts, dts2)
    assert abs(J - J2) <= 1e-14 * abs(J)


def test_a_sweep_without_the_bed_gradient_gives_the_others():
    """dgswe_adjoint_reverse with no bed output skips the bed's λ; the state,
    Manning and tide gradients stay those of a full sweep (to the atomic
    sums' ordering, 1e-12), on a drying flat (subcell and limiter paths)."""
    case, form, state = setup(2, False)
    with Adjoint(form, STEPS, STATIONS, t_start=T_START) as adj:
        adj.forward(state)
        full = adj.reverse()
        part = adj.reverse(bed=False)
    assert np.abs(full.bed).max() > 0.0 and not part.bed.any()
    for a, b in [(full.h0, part.h0), (full.hu0, part.hu0), (full.hv0, part.hv0),
                 (full.manning, part.manning), (full.tide, part.tide)]:
        assert np.abs(a - b).max() <= 1e-12 * max(np.abs(a).max(), 1e-300)
