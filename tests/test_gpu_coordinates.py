"""Scenarios far from the coordinate origin, bit for bit against the oracle.

The float32 pre-checks that skip non-interacting pairs and wall segments
work on positions relative to the scenario's grid origin, with extents raised
by the positions' magnitudes (csrc/cd_cull.cuh).  These tests move the
hallway (400 Circular agents, two walls) and the room (2000 ThreeCircle
agents, five walls) to UTM-like coordinates, (5e5, 7e6) m, and require every
force-stage variant to reproduce the oracle's full step bit for bit, and a
20-step rollout to stay identical.  A crowd 7e6 m from its grid origin (all
agents clamped into one border cell, relative coordinates near the 1e7 m
bound) must stay identical too, and a crowd beyond the bound is rejected.
"""
import numpy as np
import pytest

from crowddynamics_gb300 import _native as N
from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.engine import batch_from_scenarios
from crowddynamics_gb300.simulation.agents import shoulders
from test_gpu_parity import assert_identical, device_step, moving, oracle_step

pytestmark = pytest.mark.gpu

UTM = (5e5, 7e6)


def translated(scen, offset, bounds=None):
    """The scenario moved by `offset` (agents, shoulders, walls and grid)."""
    a = scen.agents.copy()
    a['position'] = a['position'] + np.asarray(offset)
    if scen.body == 'three_circle':
        shoulders(a)
    w = scen.walls.copy()
    w['p0'] = w['p0'] + np.asarray(offset)
    w['p1'] = w['p1'] + np.asarray(offset)
    x0, y0, x1, y1 = scen.bounds
    if bounds is None:
        bounds = (x0 + offset[0], y0 + offset[1], x1 + offset[0], y1 + offset[1])
    return S.Scenario(scen.name + '_moved', a, w, bounds, scen.cell_size, scen.dt_min,
                      scen.dt_max, scen.steps, scen.seed, dict(scen.extra))


CASES = {
    'hallway': lambda: translated(S.hallway(), UTM),
    'hallway_moving': lambda: translated(moving(S.hallway()), UTM),
    'room_moving': lambda: translated(moving(S.room()), UTM),
}


@pytest.mark.parametrize('name', sorted(CASES))
@pytest.mark.parametrize('variant', range(15))
def test_utm_full_step_every_variant(oracle, native, name, variant):
    scen = CASES[name]()
    noise = S.draw_noise(scen.agents, np.random.default_rng(21))
    got, dt_g = device_step(scen, N.NODE_ALL, noise, variant=variant)
    exact, dt_e = oracle_step(oracle, scen, N.NODE_ALL, noise, exact=True)
    assert dt_g == dt_e
    assert_identical(got, exact, 'variant %d' % variant)


@pytest.mark.parametrize('name', ['hallway_moving', 'room_moving'])
def test_utm_rollout(oracle, native, name):
    scen = CASES[name]()
    nodes = N.NODE_ALL & ~N.NODE_FLUCTUATION
    b, agents, _ = batch_from_scenarios([scen])
    b.run(20, nodes)
    got = agents.copy()
    b.download(got)
    b.close()
    ref = scen.agents.copy()
    grid = oracle.make_grid(*scen.grid)
    with oracle.exact_math():
        for _ in range(20):
            oracle.step(ref, grid, scen.walls, flags=2 | 4 | 8 | 16 | 32 | 64,
                        dt_min=scen.dt_min, dt_max=scen.dt_max)
    assert_identical(got, ref, 'rollout')


@pytest.mark.parametrize('variant', [0, 6, 10])
def test_crowd_far_from_its_grid(oracle, native, variant):
    """A 2 x 2 grid at the origin and a crowd 7e6 m away: every agent sits in
    one border cell, every pair is a candidate, and the raised extents keep
    every pair the reference evaluates."""
    base = moving(S.room(n=300, size=15.0, seed=4))
    scen = translated(base, UTM, bounds=(0.0, 0.0, 2 * base.cell_size, 2 * base.cell_size))
    noise = S.draw_noise(scen.agents, np.random.default_rng(22))
    got, dt_g = device_step(scen, N.NODE_ALL, noise, variant=variant)
    exact, dt_e = oracle_step(oracle, scen, N.NODE_ALL, noise, exact=True)
    assert dt_g == dt_e
    assert_identical(got, exact, 'variant %d' % variant)


def test_crowd_beyond_the_range_is_rejected(native):
    from crowddynamics_gb300.exceptions import InvalidValue
    base = S.hallway(n=50, width=10.0, height=10.0, seed=2)
    scen = translated(base, (2e7, 0.0), bounds=(0.0, 0.0, 10.0, 10.0))
    b, agents, _ = batch_from_scenarios([scen])
    with pytest.raises(InvalidValue, match='1e7 m'):
        b.step(N.NODE_AGENT_AGENT, want_dt=True)
    b.close()
