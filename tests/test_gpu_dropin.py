"""The reference-facing host API on the device: the function-level drop-ins
(core/interactions.py, core/integrator.py, core/motion/adjusting.py,
core/steering/orientation.py) and MultiAgentSimulation with the standard
node tree, each against the oracle (exact-math mode: bit-identical)."""
import math

import numpy as np
import pytest

from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.core import interactions as I, integrator as G
from crowddynamics_gb300.core.motion import adjusting as A
from crowddynamics_gb300.core.steering import orientation as OR
from crowddynamics_gb300.exceptions import InvalidType
from crowddynamics_gb300.simulation import logic as L
from crowddynamics_gb300.simulation.agents import Agents
from crowddynamics_gb300.simulation.field import Field
from crowddynamics_gb300.simulation.multiagent import MultiAgentSimulation
from crowddynamics_gb300.core._device_call import position_grid
from test_gpu_parity import assert_identical
from test_reference_kat import validation_agents

pytestmark = pytest.mark.gpu


@pytest.fixture(params=['hallway', 'room'])
def scen(request):
    return S.hallway(n=150, width=20.0, height=8.0, seed=4) if request.param == 'hallway' \
        else S.room(n=200, size=12.0, seed=5)


def test_agent_agent_block_list(oracle, native, scen):
    a = scen.agents.copy()
    I.agent_agent_block_list(a, scen.cell_size)
    ref = scen.agents.copy()
    with oracle.exact_math():
        oracle.agent_agent_block_list(ref, oracle.make_grid(*position_grid(ref, scen.cell_size)))
    assert_identical(a, ref)


def test_agent_obstacle(oracle, native, scen):
    a = scen.agents.copy()
    I.agent_obstacle(a, scen.walls)
    ref = scen.agents.copy()
    with oracle.exact_math():
        oracle.agent_obstacle(ref, scen.walls)
    assert_identical(a, ref)


def test_adjust_orient_integrate(oracle, native, scen):
    a = scen.agents.copy()
    ref = scen.agents.copy()
    with oracle.exact_math():
        if scen.body == 'three_circle':
            OR.orient_towards_target_direction(a)
            oracle.orient_towards_target_direction(ref)
            A.torque_adjust_agents(a)
            oracle.torque_adjust_agents(ref)
        A.force_adjust_agents(a)
        oracle.force_adjust_agents(ref)
        assert_identical(a, ref, 'adjust')
        dt_probe = G.adaptive_timestep(a, 0.001, 0.01)
        assert dt_probe == oracle.adaptive_timestep(ref, 0.001, 0.01)
        dt = G.velocity_verlet_integrator(a, 0.001, 0.01)
        assert dt == oracle.velocity_verlet_integrator(ref, 0.001, 0.01)
    assert_identical(a, ref, 'integrate')


def test_invalid_and_empty(native):
    bad = np.zeros(3, dtype=[('position', 'f8', 2)])
    with pytest.raises(InvalidType):
        I.agent_agent_block_list(bad, 3.6)
    with pytest.raises(InvalidType):
        I.agent_obstacle(bad, S.walls_array([((0, 0), (1, 0))]))
    from crowddynamics_gb300.simulation.agents import new_agents
    for model in ('circular', 'three_circle'):
        e = new_agents(0, model)
        I.agent_agent_block_list(e, 3.6)
        assert G.velocity_verlet_integrator(e, 0.001, 0.01) == 0.01
        one = new_agents(1, model)
        one['mass'] = 1.0
        I.agent_agent_block_list(one, 3.6)
        assert np.all(one['force'] == 0)


def standard_tree(sim, noise=True):
    kids = [L.Adjusting(sim) << L.Orientation(sim), L.AgentAgentInteractions(sim, max_agent_radius=0.35),
            L.AgentObstacleInteractions(sim)]
    if noise:
        kids.insert(0, L.Fluctuation(sim))
    return L.Reset(sim) << (L.Integrator(sim, dt_min=0.001, dt_max=0.01) << tuple(kids))


def test_simulation_matches_oracle(oracle, native, scen):
    rng_seed = 17
    sim = MultiAgentSimulation(agents=Agents(array=scen.agents.copy()),
                               field=Field(domain=scen.bounds, obstacles=scen.walls),
                               rng=np.random.default_rng(rng_seed))
    sim.logic = standard_tree(sim)
    cell = sim.logic['AgentAgentInteractions'].cell_size
    from crowddynamics_gb300.engine import grid_for_bounds
    grid = oracle.make_grid(*grid_for_bounds(scen.bounds, cell))
    ref = scen.agents.copy()
    rng = np.random.default_rng(rng_seed)
    t = 0.0
    with oracle.exact_math():
        for k in range(30):
            sim.update()
            nf, nm = S.draw_noise(ref, rng)
            t += oracle.step(ref, grid, scen.walls, nf, nm, dt_min=0.001, dt_max=0.01)
    assert sim.data['iterations'] == 30
    assert sim.data['time_tot'] == t
    assert_identical(sim.agents.array, ref, 'simulation')
    # host edits between updates reach the device
    sim.agents.array['velocity'] *= 0.5
    ref['velocity'] *= 0.5
    with oracle.exact_math():
        sim.update()
        nf, nm = S.draw_noise(ref, rng)
        oracle.step(ref, grid, scen.walls, nf, nm, dt_min=0.001, dt_max=0.01)
    assert_identical(sim.agents.array, ref, 'after host edit')
    sim.close()


@pytest.mark.parametrize('model', ['circular', 'three_circle'])
def test_validation_scenarios(native, model):
    """examples/tests/test_validation.py:32-57 through MultiAgentSimulation:
    a free walker covers >= 10 m in 1000 steps; in a head-on encounter
    agent 0 covers >= 8 m."""
    sim = MultiAgentSimulation(agents=Agents(array=validation_agents(model, [0.0], [(0.0, 0.0)])),
                               field=Field(domain=(-20, -20, 40, 20)))
    sim.logic = L.Reset(sim) << L.Integrator(sim) << L.Adjusting(sim) << L.Orientation(sim)
    start = sim.agents.array['position'].copy()
    sim.exit_condition = lambda s: s.data['iterations'] == 1000
    sim.run()
    d = np.hypot(*(sim.agents.array['position'] - start).T)
    assert d[0] >= 10.0 or np.isclose(d[0], 10.0)

    sim = MultiAgentSimulation(
        agents=Agents(array=validation_agents(model, [0.0, math.pi], [(0.0, 0.0), (5.0, 0.0)])),
        field=Field(domain=(-20, -20, 40, 20)), rng=np.random.default_rng(0))
    sim.logic = L.Reset(sim) << (L.Integrator(sim) << (
        L.Fluctuation(sim), L.Adjusting(sim) << L.Orientation(sim), L.AgentAgentInteractions(sim)))
    start = sim.agents.array['position'].copy()
    sim.exit_condition = lambda s: s.data['iterations'] == 1000
    sim.run()
    d = np.hypot(*(sim.agents.array['position'] - start).T)
    assert d[0] >= 8.0 or np.isclose(d[0], 8.0)
