"""The batched adjoint of an ensemble (dgswe_adjoint_create_ensemble) and
the parameter update between sweeps (dgswe_adjoint_set_parameters).

An ensemble's adjoint runs every member's forward and reverse sweep in
one batch; member by member it must give what the member's own adjoint
gives: the same time steps and misfit bit for bit (the forward kernels
are the same and the members' sums run in the same order), and the same
gradients up to the order of the atomic additions of the reverse sweep.
The gradients the ensemble gives are also checked against central
differences of the ensemble's own forward with its time steps replayed,
the parameters moved by dgswe_adjoint_set_parameters."""

import dataclasses

import numpy as np
import pytest

from dgcom_gb300 import cases
from dgcom_gb300.adjoint import Adjoint
from dgcom_gb300.mesh import TAG_OPEN
from dgcom_gb300.physics import TidalBoundary

pytestmark = pytest.mark.gpu

STEPS = 24
T_START = 3600.0  # the tide fully ramped; from a flowing state (Manning's n matters)


def members(n=3, k_range=(300, 900), n_stations=5):
    ms = cases.adjoint_ensemble_members(n_members=n, k_range=k_range, n_stations=n_stations)
    forms = [m.case.form for m in ms]
    # and one station in the first column of elements, which the tide on the
    # open (western) side reaches within the run
    own = [np.vstack([m.stations, [[50.0, 0.5 * f.mesh.vertices[:, 1].max()]]])
           for m, f in zip(ms, forms)]
    stations = np.vstack(own)
    member = np.repeat(np.arange(n), [x.shape[0] for x in own]).astype(np.int32)
    flows = [cases.with_flow(m.case, eta_amp=0.5, u=0.4, v=-0.15) for m in ms]
    state = tuple(np.concatenate([f[c] for f in flows]) for c in range(3))
    return ms, forms, stations, member, state


def open_row(form):
    """The open boundary's row among a form's conditions (sorted by tag)."""
    return sorted(form.boundaries).index(TAG_OPEN)


def test_ensemble_adjoint_equals_each_members_own():
    ms, forms, stations, member, state = members()
    with Adjoint.ensemble(forms, STEPS, stations, member, t_start=T_START) as ens:
        J, eta, dts = ens.forward(state)
        Jm = ens.member_J()
        g = ens.reverse()
        slices = [ens.member_slice(m) for m in range(len(forms))]
        tides = [ens.member_tide(g.tide, m) for m in range(len(forms))]
    assert dts.shape == (STEPS, len(forms))
    assert np.all(dts > 0.0)
    assert J == pytest.approx(float(Jm.sum()), rel=1e-14)
    for m, f in enumerate(forms):
        sel = member == m
        sl = slices[m]
        with Adjoint(f, STEPS, stations[sel], t_start=T_START) as one:
            J1, eta1, dts1 = one.forward(tuple(x[sl] for x in state))
            g1 = one.reverse()
        assert np.array_equal(dts[:, m], dts1), m
        assert np.array_equal(eta[:, sel], eta1), m
        assert Jm[m] == J1, m
        for name in ("h0", "hu0", "hv0", "bed", "manning"):
            a, b = getattr(g, name)[sl], getattr(g1, name)
            tol = 1e-11 * max(float(np.abs(b).max()), 1e-300)
            assert np.abs(a - b).max() <= tol, (m, name, float(np.abs(a - b).max()), tol)
        nc = len(f.boundaries)
        a, b = tides[m], g1.tide[:nc]
        assert np.abs(a - b).max() <= 1e-11 * max(float(np.abs(b).max()), 1e-300), (m, "tide")


def test_set_parameters_equals_a_new_form():
    ms, forms, stations, member, state = members(n=1, k_range=(400, 400))
    form = forms[0]
    ms0 = ms[0]
    row = open_row(form)
    with Adjoint(form, STEPS, stations, t_start=T_START) as adj:
        J0, _, dts = adj.forward(state)
        tide = adj.tide_parameters()
        tide[row] = ms0.tide_obs
        adj.set_parameters(manning=ms0.manning_obs, tide=tide)
        J1, _, dts1 = adj.forward(state, dts=dts)
        adj.set_parameters(manning=np.asarray(form.manning_n), tide=adj.tide_parameters())
        J2, _, _ = adj.forward(state, dts=dts)
    bc = form.boundaries[TAG_OPEN]
    cons = []
    for i, c in enumerate(bc.constituents):
        k = type(c)()
        for name, _ in type(c)._fields_:
            setattr(k, name, getattr(c, name))
        k.amplitude, k.phase = ms0.tide_obs[i]
        cons.append(k)
    new = dict(form.boundaries)
    new[TAG_OPEN] = TidalBoundary(cons, mean_elevation=bc.mean_elevation,
                                  ramp_duration=bc.ramp_duration, incoming_wave=bc.incoming_wave)
    moved = dataclasses.replace(form, boundaries=new, manning_n=ms0.manning_obs)
    with Adjoint(moved, STEPS, stations, t_start=T_START) as fresh:
        Jf, _, _ = fresh.forward(state, dts=dts)
    assert J1 == Jf
    assert J2 == J0
    assert J1 != J0


def test_ensemble_gradient_matches_finite_differences():
    ms, forms, stations, member, state = members()
    nn = (forms[0].order + 1) ** 2
    rng = np.random.default_rng(5)
    with Adjoint.ensemble(forms, STEPS, stations, member, t_start=T_START) as ens:
        # observations from the perturbed forcing, at the same step times
        tide0 = ens.tide_parameters()
        n0 = np.concatenate([np.asarray(f.manning_n) for f in forms])
        tide_obs = tide0.copy()
        c0 = 0
        for m, f in enumerate(forms):
            tide_obs[c0 + open_row(f)] = ms[m].tide_obs
            c0 += len(f.boundaries)
        n_obs = np.concatenate([m.manning_obs for m in ms])
        _, _, dts = ens.forward(state)
        ens.set_parameters(manning=n_obs, tide=tide_obs)
        _, eta_obs, _ = ens.forward(state, dts=dts)
        ens.set_parameters(manning=n0, tide=tide0)
        J, _, _ = ens.forward(state, dts=dts, eta_obs=eta_obs)
        assert J > 0.0
        g = ens.reverse()

        def J_at(manning=None, tide=None):
            ens.set_parameters(manning=manning, tide=tide)
            return ens.forward(state, dts=dts, eta_obs=eta_obs)[0]

        # Manning's n per element of member 1, a random direction. The step
        # is 3e-3 of n: J ≈ 0.02 carries roundoff of ≈ 1e-15, which steps of
        # 1e-4 and below turn into FD errors of 1e-5 and more, while steps of
        # 1e-2 to 3e-3 agree with the adjoint to ≈ 1e-7 in every direction
        # tried (truncation is below that)
        sl = ens.member_slice(1)
        d = np.zeros_like(n0)
        d[sl] = np.repeat(rng.standard_normal((sl.stop - sl.start) // nn), nn)
        eps = 3e-3 * float(n0.max())
        fd = (J_at(manning=n0 + eps * d) - J_at(manning=n0 - eps * d)) / (2 * eps)
        J_at(manning=n0)
        adj = float(np.dot(g.manning, d))
        assert abs(adj - fd) <= 1e-6 * max(abs(fd), abs(adj)), (adj, fd)
        # member 2's eight constituents: amplitudes and phases together
        row = sum(len(f.boundaries) for f in forms[:2]) + open_row(forms[2])
        dt = np.zeros_like(tide0)
        dt[row] = rng.standard_normal(dt[row].shape)
        eps = 1e-4  # metres and radians: J is far more curved here, and dJ larger
        fd = (J_at(tide=tide0 + eps * dt) - J_at(tide=tide0 - eps * dt)) / (2 * eps)
        adj = float(np.sum(g.tide * dt))
        assert abs(adj - fd) <= 1e-6 * max(abs(fd), abs(adj)), (adj, fd)


def test_ensemble_gradient_matches_the_oracle_forward():
    """The batched gradient for one member against central differences of
    the oracle (the CPU restatement of the reference forward) running that
    member alone over the member's own time steps: Manning's n per element
    of member 1 in a random direction, at 1e-6."""
    from oracle_lib import oracle

    ms, forms, stations, member, state = members()
    nn = (forms[0].order + 1) ** 2
    rng = np.random.default_rng(11)
    with Adjoint.ensemble(forms, STEPS, stations, member, t_start=T_START) as ens:
        tide0 = ens.tide_parameters()
        n0 = np.concatenate([np.asarray(f.manning_n) for f in forms])
        tide_obs = tide0.copy()
        c0 = 0
        for m, f in enumerate(forms):
            tide_obs[c0 + open_row(f)] = ms[m].tide_obs
            c0 += len(f.boundaries)
        n_obs = np.concatenate([m.manning_obs for m in ms])
        _, _, dts = ens.forward(state)
        ens.set_parameters(manning=n_obs, tide=tide_obs)
        _, eta_obs, _ = ens.forward(state, dts=dts)
        ens.set_parameters(manning=n0, tide=tide0)
        ens.forward(state, dts=dts, eta_obs=eta_obs)
        g = ens.reverse()
        sl = ens.member_slice(1)
        st_elem, st_w = ens.station_weights()
    mine = np.nonzero(member == 1)[0]
    k0 = sl.start // nn
    form1 = forms[1]
    q1 = tuple(np.ascontiguousarray(x[sl]) for x in state)
    b1 = form1.bathymetry.reshape(-1)

    def J_oracle(manning):
        ref = oracle(dataclasses.replace(form1, manning_n=manning))
        try:
            ref.upload(*q1)
            t, J = T_START, 0.0
            for n in range(STEPS):
                ref.step(t, float(dts[n, 1]))
                t += float(dts[n, 1])
                h = ref.download()[0]
                for s in mine:
                    k = int(st_elem[s]) - k0
                    eta = float(np.dot(st_w[s], h[k * nn:(k + 1) * nn] + b1[k * nn:(k + 1) * nn]))
                    J += (eta - float(eta_obs[n, s])) ** 2
        finally:
            ref.close()
        return J

    n1 = np.asarray(form1.manning_n, dtype=np.float64).reshape(-1)
    d1 = np.repeat(rng.standard_normal(n1.size // nn), nn)
    eps = 3e-3 * float(n0.max())
    fd = (J_oracle(n1 + eps * d1) - J_oracle(n1 - eps * d1)) / (2 * eps)
    adj = float(np.dot(g.manning[sl], d1))
    assert abs(adj - fd) <= 1e-6 * max(abs(fd), abs(adj)), (adj, fd)
