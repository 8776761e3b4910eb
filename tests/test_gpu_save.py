"""SaveSimulationData with asynchronous device snapshots: the saved frames
and data rows equal the per-update states of the same simulation run without
the node, bit for bit, in the reference's files (agents_{k}.npy, data.csv,
metadata.csv, geometry.json)."""
import csv
import json
import os

import numpy as np
import pytest

from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.io import load_npy
from crowddynamics_gb300.simulation import logic as L
from crowddynamics_gb300.simulation.agents import Agents
from crowddynamics_gb300.simulation.field import Field
from crowddynamics_gb300.simulation.multiagent import MultiAgentSimulation

pytestmark = pytest.mark.gpu


def make_sim(scen, seed):
    sim = MultiAgentSimulation(agents=Agents(array=scen.agents.copy()),
                               field=Field(domain=scen.bounds, obstacles=scen.walls),
                               rng=np.random.default_rng(seed), name='room')
    sim.logic = L.Reset(sim) << (L.Integrator(sim, dt_min=0.001, dt_max=0.01) << (
        L.Fluctuation(sim), L.Adjusting(sim) << L.Orientation(sim),
        L.AgentAgentInteractions(sim, max_agent_radius=0.35), L.AgentObstacleInteractions(sim)))
    return sim


@pytest.mark.parametrize('slots', [1, 4])
def test_saved_frames_equal_states(native, tmp_path, slots):
    scen = S.room(n=250, size=12.0, seed=3)
    steps, every = 11, 4
    sim = make_sim(scen, 5)
    node = L.SaveSimulationData(sim, base_directory=str(tmp_path), save_directory='run',
                                save_condition=lambda s: (s.data['iterations'] + 1) % every == 0,
                                slots=slots)
    node.add_to_simulation_logic()
    sim.exit_condition = lambda s: s.data['iterations'] == steps
    sim.run()
    sim.close()

    twin = make_sim(scen, 5)
    states, rows = [], []
    for _ in range(steps):
        twin.update()
        states.append(twin.agents.array.copy())
        rows.append((twin.data['iterations'] - 1, twin.data['time_tot'], twin.data['dt']))
    twin.close()

    d = str(tmp_path / 'run')
    files = list(load_npy(d, 'agents'))
    assert [len(f) for f in files] == [4, 4]          # frames 0-3, 4-7; 8-10 not yet dumped
    frames = np.concatenate(files)
    for k in range(8):
        for name in ('position', 'velocity', 'force_prev', 'orientation', 'torque_prev'):
            assert np.array_equal(frames[k][name], states[k][name]), (k, name)
    with open(os.path.join(d, 'data.csv')) as fp:
        table = list(csv.reader(fp))
    assert table[0] == ['iterations', 'time_tot', 'dt']
    assert len(table) == 1 + 8
    for k in range(8):
        it, tt, dt = table[1 + k]
        assert int(it) == rows[k][0] and float(tt) == rows[k][1] and float(dt) == rows[k][2]
    with open(os.path.join(d, 'metadata.csv')) as fp:
        meta = list(csv.reader(fp))
    assert meta[0] == ['name', 'timestamp'] and meta[1][0] == 'room'
    geom = json.load(open(os.path.join(d, 'geometry.json')))
    assert geom['domain']['type'] == 'Polygon'
    assert len(geom['obstacles']['coordinates']) == len(scen.walls)
