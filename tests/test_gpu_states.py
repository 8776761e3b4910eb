"""State nodes on the device: LeaderFollowerWithHerding and LeaderFollower
against fixtures made by the reference's own collective_motion code (integer
states exact; directions within 1e-12, the reference's np.hypot / np.cos
rounding against the shared float64 functions), InsideDomain and
TargetReached against the crossings test restated in numpy."""
import math
import os

import numpy as np
import pytest

from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.engine import DeviceBatch, walls_as_rows
from crowddynamics_gb300.simulation import logic as L
from crowddynamics_gb300.simulation.agents import Agents, new_agents
from crowddynamics_gb300.simulation.field import Field
from crowddynamics_gb300.simulation.multiagent import MultiAgentSimulation

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


def herding_case(mode):
    d = np.load(os.path.join(GOLDEN, 'herding.npz'))
    g = d[mode + '_grid']
    grid = (g[0], g[1], g[2], int(g[3]), int(g[4]))
    return d[mode + '_before'], d[mode + '_after'], d[mode + '_walls'], grid


def check_herding(got, want):
    assert np.array_equal(got['target'], want['target'])
    assert np.array_equal(got['index_leader'], want['index_leader'])
    f = want['is_follower']
    assert np.all(np.abs(got['target_direction'][f] - want['target_direction'][f]) <= 1e-12)
    assert np.array_equal(got['target_direction'][~f], want['target_direction'][~f])


@pytest.mark.parametrize('mode', ['herding', 'leader'])
def test_herding_matches_reference(native, mode):
    before, want, walls, grid = herding_case(mode)
    b = DeviceBatch('three_circle', [dict(n_agents=len(before), n_walls=len(walls), grid=grid)])
    b.upload(before)
    b.set_walls(walls)
    if mode == 'herding':
        b.herding(True, sight_follower=10.0, size_nearest_other=5)
    else:
        b.herding(False, sight_follower=1.0, sight_leader=20.0)
    got = before.copy()
    b.download(got)
    b.close()
    check_herding(got, want)


def test_herding_node_in_simulation(native):
    before, want, walls, grid = herding_case('herding')
    x0, y0, cell, nx, ny = grid
    sim = MultiAgentSimulation(agents=Agents(array=before.copy()),
                               field=Field(domain=(x0, y0, x0 + nx * cell, y0 + ny * cell),
                                           obstacles=walls))
    sim.logic = L.LeaderFollowerWithHerding(sim)
    sim._config = lambda: (cell, 0.001, 0.01)            # the fixture's grid
    sim.update()
    check_herding(sim.agents.array, want)
    sim.close()


def crossings(points, poly):
    """matplotlib's Path(poly).contains_points(points), restated by the oracle."""
    from oracle.pip import contains_points
    return contains_points(points, poly)


RINGS = {
    'square_ccw': [(0, 0), (4, 0), (4, 4), (0, 4)],
    'square_cw_closed': [(0, 0), (0, 4), (4, 4), (4, 0), (0, 0)],
    'concave': [(0, 0), (8, 0), (8, 4), (5, 4), (4, 1), (3, 4), (0, 4)],
    'triangle': [(0.5, 0.25), (7.75, 1.5), (2.25, 5.5)],
}


@pytest.mark.parametrize('ring', sorted(RINGS))
def test_inside_domain_boundary_conventions(native, ring):
    """Points on a 0.25 m lattice (every vertex and the edges' lattice points
    among them, on the boundary bit for bit), random points and non-finite
    positions: the device's inside flags equal the oracle's restatement of
    matplotlib's crossings test, with its half-open edge conventions."""
    poly = np.array(RINGS[ring], float)
    g = np.arange(-1.0, 9.01, 0.25)
    gx, gy = np.meshgrid(g, g, indexing='ij')
    rng = np.random.default_rng(4)
    pts = np.vstack([np.column_stack([gx.ravel(), gy.ravel()]), rng.uniform(-1, 9, (2000, 2)),
                     [(np.nan, 1.0), (1.0, np.inf), (-np.inf, 2.0)]])
    a = new_agents(len(pts), 'circular')
    a['position'] = pts
    a['active'] = True
    b = DeviceBatch('circular', [dict(n_agents=len(a), n_walls=0, grid=(-1.0, -1.0, 3.7, 3, 3))])
    b.upload(a)
    b.inside_domain(0, poly)
    got = a.copy()
    b.download(got)
    b.close()
    want = crossings(pts, poly)
    bad = np.flatnonzero(got['active'] != want)
    assert bad.size == 0, pts[bad[:5]]
    assert want.any() and (~want).any()


def test_inside_domain_and_target_reached(native):
    scen = S.hallway(n=500, width=20.0, height=8.0, seed=6)
    a = scen.agents
    rng = np.random.default_rng(9)
    a['position'] = np.column_stack([rng.uniform(-3, 23, len(a)), rng.uniform(-3, 11, len(a))])
    b = DeviceBatch('circular', [dict(n_agents=len(a), n_walls=len(scen.walls),
                                      grid=(-4.0, -4.0, 3.7, 8, 5))])
    b.upload(a)
    b.set_walls(scen.walls)
    domain = np.array([[0, 0], [20, 0], [20, 8], [12, 8], [10, 4], [8, 8], [0, 8], [0, 0]], float)
    changed = b.inside_domain(0, domain)
    want = crossings(a['position'], domain)
    assert changed == int((~want).sum())                 # all started active
    got = a.copy()
    b.download(got)
    assert np.array_equal(got['active'], want)
    assert b.inside_domain(0, domain) == 0
    targets = [np.array([[18, 2], [21, 2], [21, 6], [18, 6]], float),
               np.array([[-1, 3], [1, 3], [0, 5]], float)]
    counts = b.target_reached(0, targets, reset=True)
    assert list(counts) == [int(crossings(a['position'], t).sum()) for t in targets]
    # reached agents stay counted after they leave
    a2 = got.copy()
    a2['position'] += 30.0
    b.upload(a2)
    assert list(b.target_reached(0, targets)) == list(counts)
    assert list(b.target_reached(0, targets, reset=True)) == [0, 0]
    b.close()


def test_state_nodes_in_simulation(native):
    scen = S.hallway(n=300, width=20.0, height=8.0, seed=7)
    a = scen.agents
    a['position'][:40, 0] = -2.0                         # outside the domain
    sim = MultiAgentSimulation(agents=Agents(array=a.copy()),
                               field=Field(domain=(0.0, 0.0, 20.0, 8.0), obstacles=scen.walls,
                                           targets=[(15.0, 0.0, 20.0, 8.0)]))
    sim.logic = L.TargetReached(sim) << L.InsideDomain(sim)
    sim.update()
    assert sim.data['inactive'] == 40
    assert sim.data['target_0'] == int((a['position'][:, 0] >= 15.0).sum())
    assert int((~sim.agents.array['active']).sum()) == 40
    sim.close()


def test_exit_detection_matches_reference(native):
    d = np.load(os.path.join(GOLDEN, 'exit.npz'))
    before, want, walls = d['before'], d['after'], d['walls']
    g = d['grid']
    b = DeviceBatch('three_circle', [dict(n_agents=len(before), n_walls=len(walls),
                                          grid=(g[0], g[1], g[2], int(g[3]), int(g[4])))])
    b.upload(before)
    b.set_walls(walls)
    b.exit_detection(0, d['doors'], 20.0)
    got = before.copy()
    b.download(got)
    b.close()
    assert np.array_equal(got['target'], want['target'])
    assert np.array_equal(got['is_follower'], want['is_follower'])


def test_herding_rejects_leader_and_follower(native):
    """A record flagged both leader and follower is rejected before any state
    changes; the same crowd without that record runs."""
    from crowddynamics_gb300.exceptions import InvalidValue
    scen = S.room(n=200, size=15.0, seed=5)
    a = scen.agents
    rng = np.random.default_rng(2)
    a['is_leader'] = rng.uniform(size=len(a)) < 0.1
    a['is_follower'] = ~a['is_leader'] & (rng.uniform(size=len(a)) < 0.7)
    a['target'] = np.where(a['is_leader'], 0, -1)
    bad = a.copy()
    k = int(np.flatnonzero(bad['is_leader'])[0])
    bad['is_follower'][k] = True
    b = DeviceBatch('three_circle', [dict(n_agents=len(a), n_walls=len(scen.walls),
                                          grid=scen.grid)])
    b.set_walls(scen.walls)
    b.upload(bad)
    with pytest.raises(InvalidValue, match='leader and follower'):
        b.herding(True)
    got = bad.copy()
    b.download(got)
    assert np.array_equal(got['target_direction'], bad['target_direction'])
    assert np.array_equal(got['target'], bad['target'])
    b.upload(a)
    b.herding(True)
    b.close()
