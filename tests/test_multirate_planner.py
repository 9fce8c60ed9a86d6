"""The multirate level planner on the host (dgswe_planner_*, no device),
held to the known answers of the reference's own tests of
MultirateStepper (src/time/multirate.rs:1350-1805): the levels and coarse
step, the caps, the landing fit, the jump limit, the stage rates spread one
face per stage or node by node along GLL lines, the pass lists, and the kept
plan equal to one made afresh.

A mesh of separate quads (no face neighbours) checks assign_levels alone,
as the reference's test does without a mesh; rows of unit quads are the
reference's Mesh2D::uniform_rectangle rows."""

import math

import numpy as np
import pytest

from dgcom_gb300 import abi
from dgcom_gb300.mesh import QuadMesh, uniform_rectangle
from dgcom_gb300.multirate import Planner
from dgcom_gb300.physics import SWEDeviceForm2D

INF = math.inf


def separate_quads(n: int) -> QuadMesh:
    """n unit quads that share no vertex: every face on the boundary."""
    verts, elems = [], []
    for k in range(n):
        x = 2.0 * k
        verts += [(x, 0.0), (x + 1.0, 0.0), (x + 1.0, 1.0), (x, 1.0)]
        elems.append((4 * k, 4 * k + 1, 4 * k + 2, 4 * k + 3))
    return QuadMesh(np.array(verts), np.array(elems, dtype=np.int64), np.zeros((0, 4), np.int64),
                    np.zeros((n, 4), dtype=np.int32))


def planner(mesh, max_levels, order=1, scheme=abi.SSP_RK3):
    return Planner(SWEDeviceForm2D(mesh=mesh, order=order), max_levels, scheme)


def row(n):
    return uniform_rectangle(0.0, float(n), 0.0, 1.0, n, 1)


def test_levels_are_powers_of_two_below_the_coarse_step(cuda_lib):
    # multirate.rs:1350-1366
    dts = [1.0, 0.3, 0.26, 0.1, INF, 0.55]
    with planner(separate_quads(6), 8) as p:
        plan = p.assign(dts)
    assert plan.finest == 3
    assert plan.dt == 0.8
    assert list(plan.levels) == [0, 2, 2, 3, 0, 1]
    for level, dt_k in zip(plan.levels, dts):
        dt_l = plan.dt / 2 ** int(level)
        assert dt_l <= dt_k
        assert level == 0 or 2.0 * dt_l > dt_k


def test_levels_respect_the_caps(cuda_lib):
    # multirate.rs:1368-1388
    mesh = separate_quads(2)
    with planner(mesh, 2) as p:
        plan = p.assign([1.0, 0.1])
        assert (plan.dt, plan.finest) == (0.4, 2)
        assert list(plan.levels) == [0, 2]
    with planner(mesh, 8) as p:
        plan = p.assign([1.0, 0.1], dt_cap=0.25)
        assert (plan.dt, plan.finest) == (0.2, 1)
        assert list(plan.levels) == [0, 1]
    with planner(mesh, 0) as p:
        plan = p.assign([1.0, 0.1])
        assert (plan.dt, plan.finest) == (0.1, 0)
        assert list(plan.levels) == [0, 0]
    with planner(separate_quads(3), 4) as p:
        plan = p.assign([INF] * 3)
        assert plan.dt == INF and plan.finest == 0
        assert list(plan.levels) == [0, 0, 0]


def test_lists_hold_the_elements_at_or_above_each_key_in_order(cuda_lib):
    # multirate.rs:1389-1406: keys [0, 2, 1, 2, 0, 3] as levels
    with planner(separate_quads(6), 8) as p:
        plan = p.assign([8.0, 2.0, 4.0, 2.0, 8.0, 1.0])
    assert list(plan.levels) == [0, 2, 1, 2, 0, 3]
    key = plan.rates.shape[0]  # the levels' list
    assert [plan.at_or_above(key, d) for d in range(4)] == [
        [0, 1, 2, 3, 4, 5], [1, 2, 3, 5], [1, 3, 5], [5]]
    # the order itself: largest key first, index order within a key
    assert list(plan.order[key]) == [5, 1, 3, 2, 0, 4]


def test_rates_spread_one_face_per_stage(cuda_lib):
    # multirate.rs:1415-1430
    with planner(row(6), 2) as p:
        _, rates = p.spread([0, 0, 0, 0, 0, 2])
    assert [list(r) for r in rates] == [[0, 0, 0, 0, 2, 2], [0, 0, 0, 2, 2, 2],
                                        [0, 0, 2, 2, 2, 2]]


def test_rates_spread_over_the_stage_stencil(cuda_lib):
    # multirate.rs:1468-1486 (one RHS stencil per stage)
    with planner(row(8), 2) as p:
        plan = p.assign([4.0] * 7 + [2.0])
    assert list(plan.levels) == [0] * 7 + [1]
    assert list(plan.rates[0]) == [0, 0, 0, 0, 0, 0, 1, 1]
    assert list(plan.rates[2]) == [0, 0, 0, 0, 1, 1, 1, 1]
    # 3 stages × 8 elements × 2 finest substeps against the evaluations
    assert 48.0 / plan.evaluations == 48.0 / (3.0 * 8.0 + 2.0 + 3.0 + 4.0)


def line_rates(line_local):
    """multirate.rs:1488-1506: node rates of a row of 6 P2 elements whose
    last is on level 2, four stages."""
    with planner(row(6), 2, order=2, scheme=abi.SSP_RK43) as p:
        _, rates = p.spread([0, 0, 0, 0, 0, 2], line_local=line_local)
    return [list(r) for r in rates]


def test_line_local_rates_cross_an_element_in_two_stages(cuda_lib):
    assert line_rates([True] * 6) == [[0, 0, 0, 0, 2, 2], [0, 0, 0, 0, 2, 2],
                                      [0, 0, 0, 2, 2, 2], [0, 0, 0, 2, 2, 2]]


def test_rates_of_whole_elements_spread_one_face_per_stage(cuda_lib):
    assert line_rates([False] * 6) == [[0, 0, 0, 0, 2, 2], [0, 0, 0, 2, 2, 2],
                                       [0, 0, 2, 2, 2, 2], [0, 2, 2, 2, 2, 2]]


def test_whole_elements_among_line_local_ones(cuda_lib):
    assert line_rates([True, True, True, True, False, True]) == [
        [0, 0, 0, 0, 2, 2], [0, 0, 0, 2, 2, 2], [0, 0, 0, 2, 2, 2], [0, 0, 2, 2, 2, 2]]
    assert line_rates([True, True, True, False, True, True]) == [
        [0, 0, 0, 0, 2, 2], [0, 0, 0, 0, 2, 2], [0, 0, 0, 2, 2, 2], [0, 0, 2, 2, 2, 2]]


def test_a_landing_takes_equal_steps_with_their_own_levels(cuda_lib):
    # multirate.rs:1606-1651
    dts = [8.0, 8.0, 8.0, 8.0, 4.0, 2.0, 1.0, 1.0]
    with planner(row(8), 8) as p:
        plan = p.assign(dts)
        assert plan.dt == 8.0
        assert list(plan.levels) == [0, 0, 0, 0, 1, 2, 3, 3]
        assert 3.0 * plan.inverse_dt_sum == 3.0 * 3.25
        assert plan.level_evaluations / 8.0 == 3.0 * plan.inverse_dt_sum
        plan = p.assign(dts, landing=20.0)
        assert plan.dt == 20.0 / 3.0
        assert plan.stable_step == 8.0
        assert list(plan.levels) == [0, 0, 0, 0, 1, 2, 3, 3]
        for level, dt_k in zip(plan.levels, dts):
            assert plan.dt / 2 ** int(level) <= dt_k
        plan = p.assign(dts, landing=3.0)
        assert plan.dt == 3.0
        assert list(plan.levels) == [0, 0, 0, 0, 0, 1, 2, 2]
        assert plan.finest == 2
        assert plan.level_evaluations == 3 * 15
        plan = p.assign(dts, landing=8.0)
        assert plan.dt == 8.0
        assert list(plan.levels) == [0, 0, 0, 0, 1, 2, 3, 3]


def test_kept_plans_are_those_made_afresh(cuda_lib):
    # multirate.rs:1653-1708, with the face stencil
    mesh = row(16)
    a = [300.0] * 15 + [19.0]
    b = list(a)
    b[7] = 40.0
    sequence = [(a, None), (a, None), (a, 1e3), (b, None), (b, None), (a, None), (a, 60.0)]
    with planner(mesh, 3) as kept:
        for i, (dts, cap) in enumerate(sequence):
            k = kept.assign(dts, dt_cap=cap)
            with planner(mesh, 3) as fresh:
                f = fresh.assign(dts, dt_cap=cap)
            assert k.dt == f.dt and k.finest == f.finest
            assert np.array_equal(k.levels, f.levels)
            assert np.array_equal(k.rates, f.rates)
            assert np.array_equal(k.order, f.order)
            assert k.evaluations == f.evaluations
            if i == 0:
                assert list(k.levels[13:]) == [1, 2, 3], "the limit raised the levels"


def test_a_bound_caps_the_coarse_step(cuda_lib):
    # multirate.rs:1781-1804: the module's bound enters as the cap
    with planner(row(4), 8) as p:
        plan = p.assign([500.0, 4.0, 2.0, 1.0], dt_cap=4.0)
        assert plan.dt == 4.0
        assert list(plan.levels) == [0, 0, 1, 2]
        assert p.assign([500.0, 4.0, 2.0, 1.0]).dt == 256.0


def test_level_jumps_are_limited_to_one(cuda_lib):
    # multirate.rs:1806-1815
    with planner(row(6), 3) as p:
        levels, _ = p.spread([0, 0, 0, 0, 0, 3], limit=True)
        assert list(levels) == [0, 0, 0, 1, 2, 3]
        levels, _ = p.spread([2, 0, 0, 0, 1, 0], limit=True)
        assert list(levels) == [2, 1, 0, 0, 1, 0]


@pytest.mark.parametrize("seed", [3, 4])
def test_plan_invariants_on_a_jittered_mesh(cuda_lib, seed):
    """On an unstructured mesh: every element steps within its own step,
    neighbours differ by at most a level, rates grow by stage and are at
    least the level, and each list is a prefix of its key's order."""
    from dgcom_gb300.mesh import graded_jittered_box

    mesh = graded_jittered_box(1000.0, 800.0, 12, 10, size_range=(50.0, 120.0), jitter=0.2,
                               seed=seed)
    rng = np.random.default_rng(seed)
    dts = np.exp(rng.uniform(0.0, math.log(40.0), mesh.n_elements))
    with planner(mesh, 6, order=3) as p:
        plan = p.assign(dts)
    assert plan.dt == dts.min() * 2 ** plan.finest
    for level, dt_k in zip(plan.levels, dts):
        assert plan.dt / 2 ** int(level) <= dt_k
    assert np.all(plan.rates[0] >= plan.levels)
    assert np.all(plan.rates[1] >= plan.rates[0]) and np.all(plan.rates[2] >= plan.rates[1])
    for key in range(4):
        values = plan.levels if key == 3 else plan.rates[key]
        ordered = values[plan.order[key]]
        assert np.all(np.diff(ordered.astype(int)) <= 0)


def test_substep_depths_are_the_schedule():
    """The passes of a coarse step of finest level L: substep p's stages
    run on the elements rated at least depth(p), and the substeps of the
    elements of level at least depth(p + 1) end after it
    (MultirateStepper::schedule, src/time/multirate.rs:1160-1210)."""
    from dgcom_gb300.multirate import substep_depth

    assert [substep_depth(p, 0) for p in range(2)] == [0, 0]
    assert [substep_depth(p, 2) for p in range(5)] == [0, 2, 1, 2, 0]
    assert [substep_depth(p, 3) for p in range(9)] == [0, 3, 2, 3, 1, 3, 2, 3, 0]
    # an element of level l starts a substep every 2^(L-l) finest substeps
    L = 4
    for level in range(L + 1):
        starts = [p for p in range(1 << L) if substep_depth(p, L) <= level]
        assert starts == list(range(0, 1 << L, 1 << (L - level)))
