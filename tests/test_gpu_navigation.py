"""Navigation on the device (CD_NODE_NAVIGATION): the reference's meshgrid
indicer + getdefault lookup, against the golden fixture made from the
reference's own code and against the oracle (exact-math mode: bit-identical)
inside full steps and through MultiAgentSimulation."""
import os

import numpy as np
import pytest

from crowddynamics_gb300 import _native as N
from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.engine import DeviceBatch, batch_from_scenarios, grid_for_bounds
from crowddynamics_gb300.simulation import logic as L
from crowddynamics_gb300.simulation.agents import Agents
from crowddynamics_gb300.simulation.field import Field
from crowddynamics_gb300.simulation.multiagent import MultiAgentSimulation
from test_gpu_parity import assert_identical

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


def test_device_navigation_matches_golden(native):
    d = np.load(os.path.join(GOLDEN, 'navigation.npz'))
    b = d['bounds']
    for body in ('circular', 'three_circle'):
        a = d[body + '_before'].copy()
        batch = DeviceBatch(body, [dict(n_agents=len(a), n_walls=0,
                                         grid=grid_for_bounds((-3.0, -1.0, 10.0, 8.0), 3.6))])
        batch.upload(a)
        batch.set_direction_maps(0, d['dir_x'], d['dir_y'], b[0], b[1], float(d['step']))
        batch.step(N.NODE_NAVIGATION)
        batch.download(a)
        batch.close()
        want = d[body + '_after']
        assert np.array_equal(a['target_direction'], want['target_direction']), body
        assert np.array_equal(a['position'], want['position'])


def nav_room(seed=5):
    """ThreeCircle room whose agents follow the exit map (target 0) or a
    seeded random field (target 1); a fifth have no target."""
    scen = S.room(n=300, size=14.0, seed=seed)
    a = scen.agents
    rng = np.random.default_rng(seed)
    a['target'] = rng.choice([-1, 0, 0, 1, 1], len(a))
    mx, my, step = S.room_exit_direction_map(14.0, 14.0, 6.4, 7.6, step=0.1)
    ang = rng.uniform(0, 2 * np.pi, mx.shape)
    maps = (np.stack([mx, np.cos(ang)]), np.stack([my, np.sin(ang)]))
    return scen, maps, step


@pytest.mark.parametrize('variant', [None, 0, 7, 10])
def test_navigation_steps_match_oracle(oracle, native, variant):
    scen, (mx, my), step = nav_room()
    b, agents, _ = batch_from_scenarios([scen])
    if variant is not None:
        b.set_variant(variant)
    b.set_direction_maps(0, mx, my, 0.0, 0.0, step)
    ref = scen.agents.copy()
    grid = oracle.make_grid(*scen.grid)
    rng = np.random.default_rng(3)
    nodes = N.NODE_ALL | N.NODE_NAVIGATION
    with oracle.exact_math():
        for _ in range(20):
            nf, nm = S.draw_noise(ref, rng)
            b.set_noise(nf, nm)
            b.step(nodes)
            oracle.step(ref, grid, scen.walls, nf, nm, flags=oracle.ORC_FULL | oracle.ORC_NAVIGATION,
                        dt_min=scen.dt_min, dt_max=scen.dt_max, nav=(mx, my, 0.0, 0.0, step))
    got = agents.copy()
    b.download(got)
    b.close()
    assert_identical(got, ref, 'navigation steps')
    assert np.array_equal(got['target_direction'], ref['target_direction'])


def test_simulation_navigation_node(oracle, native):
    scen, (mx, my), step = nav_room(seed=6)
    sim = MultiAgentSimulation(agents=Agents(array=scen.agents.copy()),
                               field=Field(domain=scen.bounds, obstacles=scen.walls),
                               rng=np.random.default_rng(8))
    nav = L.Navigation(sim)
    nav.direction_maps = [(mx[0], my[0]), (mx[1], my[1])]
    nav.step = step
    sim.logic = L.Reset(sim) << (L.Integrator(sim, dt_min=0.001, dt_max=0.01) << (
        L.Fluctuation(sim), L.Adjusting(sim) << (nav, L.Orientation(sim)),
        L.AgentAgentInteractions(sim, max_agent_radius=0.35), L.AgentObstacleInteractions(sim)))
    cell = sim.logic['AgentAgentInteractions'].cell_size
    grid = oracle.make_grid(*grid_for_bounds(scen.bounds, cell))
    ref = scen.agents.copy()
    rng = np.random.default_rng(8)
    with oracle.exact_math():
        for _ in range(10):
            sim.update()
            nf, nm = S.draw_noise(ref, rng)
            oracle.step(ref, grid, scen.walls, nf, nm, flags=oracle.ORC_FULL | oracle.ORC_NAVIGATION,
                        dt_min=0.001, dt_max=0.01, nav=(mx, my, 0.0, 0.0, step))
    assert_identical(sim.agents.array, ref, 'simulation with navigation')
    assert np.array_equal(sim.agents.array['target_direction'], ref['target_direction'])


def test_direction_maps_rejected(native):
    scen, (mx, my), step = nav_room()
    b, _, _ = batch_from_scenarios([scen])
    from crowddynamics_gb300.exceptions import InvalidValue
    with pytest.raises(InvalidValue):
        b.set_direction_maps(1, mx, my, 0.0, 0.0, step)          # no scenario 1
    with pytest.raises(InvalidValue):
        b.set_direction_maps(0, mx, my, 0.0, 0.0, 0.0)           # step 0
    with pytest.raises(InvalidValue):
        b.set_direction_maps(0, mx, my[:, :-1], 0.0, 0.0, step)  # shapes differ
    b.close()
