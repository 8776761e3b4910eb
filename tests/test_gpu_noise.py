"""Fluctuation noise drawn on the device (cd_set_noise_mode): bit-identical
to the oracle's copy of the same generator (cd_noise.h), inside single steps,
rollouts, CUDA-graph runs and MultiAgentSimulation."""
import numpy as np
import pytest

from crowddynamics_gb300 import _native as N
from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.engine import batch_from_scenarios, grid_for_bounds
from crowddynamics_gb300.simulation import logic as L
from crowddynamics_gb300.simulation.agents import Agents
from crowddynamics_gb300.simulation.field import Field
from crowddynamics_gb300.simulation.multiagent import MultiAgentSimulation
from test_gpu_parity import assert_identical

pytestmark = pytest.mark.gpu

SEED = 0x5eed1234abcd


def scenarios():
    return {'hallway': S.hallway(n=300, seed=3), 'room': S.room(n=400, size=16.0, seed=4)}


@pytest.mark.parametrize('name', ['hallway', 'room'])
def test_device_noise_equals_oracle(oracle, native, name):
    scen = scenarios()[name]
    b, agents, _ = batch_from_scenarios([scen])
    b.set_noise_mode(True, SEED, 41)
    for k in (42, 43):
        b.upload(scen.agents)
        b.set_noise_mode(True, SEED, k - 1)
        b.step(N.NODE_FLUCTUATION)                 # force = noise (initial force is zero)
        got = agents.copy()
        b.download(got)
        f, m = oracle.device_noise(scen.agents, SEED, k)
        assert np.array_equal(got['force'], f), k
        if m is not None:
            assert np.array_equal(got['torque'], m), k
    b.close()


@pytest.mark.parametrize('name', ['hallway', 'room'])
@pytest.mark.parametrize('graph', [False, True])
def test_rollout_with_device_noise(oracle, native, name, graph):
    scen = scenarios()[name]
    b, agents, _ = batch_from_scenarios([scen])
    b.set_noise_mode(True, SEED, 100)
    if graph:
        b.run(15, N.NODE_ALL)
    else:
        for _ in range(15):
            b.step(N.NODE_ALL)
    got = agents.copy()
    b.download(got)
    b.close()
    ref = scen.agents.copy()
    grid = oracle.make_grid(*scen.grid)
    with oracle.exact_math():
        for k in range(15):
            nf, nm = oracle.device_noise(ref, SEED, 101 + k)
            oracle.step(ref, grid, scen.walls, nf, nm, dt_min=scen.dt_min, dt_max=scen.dt_max)
    assert_identical(got, ref, 'device-noise rollout')


def test_simulation_device_noise(oracle, native):
    scen = scenarios()['room']
    sim = MultiAgentSimulation(agents=Agents(array=scen.agents.copy()),
                               field=Field(domain=scen.bounds, obstacles=scen.walls),
                               device_noise_seed=SEED)
    sim.logic = L.Reset(sim) << (L.Integrator(sim, dt_min=0.001, dt_max=0.01) << (
        L.Fluctuation(sim), L.Adjusting(sim) << L.Orientation(sim),
        L.AgentAgentInteractions(sim, max_agent_radius=0.35), L.AgentObstacleInteractions(sim)))
    cell = sim.logic['AgentAgentInteractions'].cell_size
    grid = oracle.make_grid(*grid_for_bounds(scen.bounds, cell))
    ref = scen.agents.copy()
    with oracle.exact_math():
        for k in range(8):
            sim.update()
            nf, nm = oracle.device_noise(ref, SEED, k + 1)
            oracle.step(ref, grid, scen.walls, nf, nm, dt_min=0.001, dt_max=0.01)
    assert_identical(sim.agents.array, ref, 'simulation with device noise')


def test_device_noise_distribution_at_scale(native):
    stats = pytest.importorskip('scipy.stats')
    scen = S.large_field(n=100_000)
    a = scen.agents
    a['std_rand_force'] = 1.0
    a['mass'] = 1.0
    a['std_rand_torque'] = 1.0
    a['inertia_rot'] = 1.0
    b, agents, _ = batch_from_scenarios([scen])
    b.upload(a)
    b.set_noise_mode(True, 99, 0)
    b.step(N.NODE_FLUCTUATION)
    got = agents.copy()
    b.download(got)
    b.close()
    mag = np.hypot(*got['force'].T)
    assert mag.max() <= 3.0 and np.abs(got['torque']).max() <= 3.0
    assert stats.kstest(mag, stats.truncnorm(0, 3).cdf).pvalue > 1e-4
    assert stats.kstest(got['torque'], stats.truncnorm(-3, 3).cdf).pvalue > 1e-4


def test_host_noise_still_required_without_device_mode(native):
    from crowddynamics_gb300.exceptions import InvalidValue
    scen = scenarios()['hallway']
    b, _, _ = batch_from_scenarios([scen])
    with pytest.raises(InvalidValue):
        b.run(1, N.NODE_ALL)
    with pytest.raises(InvalidValue):
        b.step(N.NODE_ALL)
    b.close()
