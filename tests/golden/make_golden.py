"""Generate the golden fixtures from the reference's own hot-path code.

Run where the reference source tree is present, its project root named by
the CROWDDYNAMICS_REFERENCE environment variable:

    CROWDDYNAMICS_REFERENCE=<crowddynamics checkout> python tests/golden/make_golden.py [case ...]

It executes the reference's numba-decorated functions as plain Python via
``oracle/ref_loader.py`` (numba, cell_lists and the agents module stubbed)
on seeded inputs and stores inputs and outputs in ``tests/golden/*.npz``.
Each case records the grid of the restated cell list it used.  The
``rollout`` case runs the reference with numba's scalar semantics (the C
library's elementary functions, literal integer powers as products).
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_loader as RL  # noqa: E402
from crowddynamics_gb300 import scenarios as S  # noqa: E402
from crowddynamics_gb300.simulation.agents import new_agents, shoulders  # noqa: E402

NODES_ALL = ('fluctuation', 'orientation', 'adjusting', 'agent_agent', 'agent_obstacle',
             'integrate', 'reset')


def save(name, **arrays):
    path = os.path.join(HERE, name + '.npz')
    np.savez_compressed(path, **arrays)
    print('wrote', path, os.path.getsize(path), 'bytes')


def scenario_case(name, scen, steps, seed):
    """Per-node outputs from the initial state, then `steps` full updates
    with host-drawn noise."""
    RL.configure_grid(*scen.grid)
    init = scen.agents.copy()
    out = dict(init=init, walls=scen.walls, grid=np.array(scen.grid, dtype=np.float64),
               cell_size=np.float64(scen.cell_size), dt_min=np.float64(scen.dt_min),
               dt_max=np.float64(scen.dt_max))
    for node in ('agent_agent', 'agent_obstacle', 'adjusting', 'orientation'):
        a = init.copy()
        nodes = (node, 'orientation') if node == 'adjusting' else (node,)
        RL.step(a, scen.cell_size, scen.walls, nodes=nodes)
        out['node_' + node] = a
    rng = np.random.default_rng(seed)
    a = init.copy()
    nf_all, nm_all, dts, states = [], [], [], []
    for k in range(steps):
        nf, nm = S.draw_noise(a, rng)
        dt = RL.step(a, scen.cell_size, scen.walls, nf, nm, scen.dt_min, scen.dt_max,
                     nodes=NODES_ALL)
        nf_all.append(nf)
        nm_all.append(nm if nm is not None else np.zeros(len(a)))
        dts.append(dt)
        states.append(a.copy())
    out['noise_f'] = np.array(nf_all)
    out['noise_m'] = np.array(nm_all)
    out['dt'] = np.array(dts)
    out['states'] = np.array(states)
    save(name, **out)


def pair_cases():
    """Two-agent configurations covering the branches of the pair kernels:
    co-moving (a == 0), head-on, contact (h < 0), coincident centres (d == 0),
    tangential miss, tau > 30 cut-off, and a truncated (|F| > 2000 N) case."""
    R = RL.load()
    cases = []
    for model in ('circular', 'three_circle'):
        base = new_agents(2, model)
        base['radius'] = 0.255
        base['mass'] = 73.5
        base['target_velocity'] = 1.0
        if model == 'three_circle':
            base['r_t'] = 0.5882 * 0.255
            base['r_s'] = 0.3725 * 0.255
            base['r_ts'] = 0.6275 * 0.255
            base['inertia_rot'] = 4.0
            base['target_angular_velocity'] = 4 * np.pi
        configs = [
            ((0, 0), (2, 0), (1, 0), (1, 0), 0.0, 0.0),          # co-moving
            ((0, 0), (2, 0), (1, 0), (-1, 0), 0.0, np.pi),       # head-on
            ((0, 0), (0.4, 0.05), (0.3, 0), (-0.2, 0.1), 0.3, 2.0),  # contact
            ((1, 1), (1, 1), (0.5, 0), (0, 0.5), 0.0, 1.0),      # coincident
            ((0, 0), (2, 2), (1, 0), (0, 0), 0.0, 0.0),          # miss
            ((0, 0), (2.9, 0), (0.01, 0), (0, 0), 0.0, 0.0),     # slow approach, tau > 30
            ((0, 0), (0.56, 0), (2, 0), (-2, 0), 0.0, np.pi),    # near contact, large force
            ((0, 0), (1.1, 0.3), (0.2, -0.4), (-0.7, 0.1), -2.5, 0.7),
            ((3, 3), (3.3, 3.6), (-0.4, 0.2), (0.9, -1.0), 3.0, -1.2),
        ]
        for xi, xj, vi, vj, phi_i, phi_j in configs:
            a = base.copy()
            a['position'] = [xi, xj]
            a['velocity'] = [vi, vj]
            if model == 'three_circle':
                a['orientation'] = [phi_i, phi_j]
                shoulders(a)
            cases.append(a)
    out = {}
    for k, a in enumerate(cases):
        out['in_%d' % k] = a
        b = a.copy()
        if 'position_ls' in a.dtype.fields:
            R.interactions.interaction_agent_agent_three_circle(0, 1, b)
            fi, fj = R.power_law.force_social_three_circle(a, 0, 1)
        else:
            R.interactions.interaction_agent_agent_circular(0, 1, b)
            fi, fj = R.power_law.force_social_circular(a, 0, 1)
        out['pair_%d' % k] = b
        out['social_%d' % k] = np.array([fi, fj])
    out['count'] = np.int64(len(cases))
    save('pairs', **out)


def wall_cases():
    """Agent-wall branches: both endpoints, the interior, a zero-length wall,
    an agent centred on the line."""
    R = RL.load()
    walls = S.walls_array([((0, 0), (4, 0)), ((5, -1), (5, 3)), ((2, 2), (2, 2)),
                           ((-1, 2), (1, 4))])
    out = {'walls': walls}
    for model in ('circular', 'three_circle'):
        pos = np.array([(-0.1, 0.1), (2.0, 0.2), (4.1, -0.1), (4.85, 1.0), (2.0, 0.0),
                        (0.1, 2.95), (2.0, 2.1), (5.0, 3.2)])
        a = new_agents(len(pos), model)
        a['position'] = pos
        a['radius'] = 0.27
        a['velocity'] = [(0.3, -0.2)] * len(pos)
        if model == 'three_circle':
            a['r_t'], a['r_s'], a['r_ts'] = 0.16, 0.1, 0.1
            a['orientation'] = np.linspace(-3, 3, len(pos))
            shoulders(a)
        out['in_' + model] = a
        b = a.copy()
        R.interactions.agent_obstacle(b, walls)
        out['out_' + model] = b
    save('walls', **out)


def misc_cases():
    """wrap_to_pi at odd multiples of pi and adaptive_timestep bounds."""
    R = RL.load()
    x = np.array([0.0, np.pi, -np.pi, 3 * np.pi, -3 * np.pi, 7.0, -7.0, 1e-300, -1e-300,
                  100.0, -100.0, 2 * np.pi, -2 * np.pi, 0.5, -0.5])
    w = np.array([R.vector2D.wrap_to_pi(float(v)) for v in x])
    a = new_agents(5, 'circular')
    a['velocity'] = [(0.1, 0), (0, 0.9), (1.3, 0.4), (0, 0), (0.2, 0.2)]
    a['target_velocity'] = [1.0, 1.2, 0.8, 1.5, 0.9]
    dts = np.array([R.integrator.adaptive_timestep(a, lo, hi)
                    for lo, hi in ((0.001, 0.01), (0.01, 0.01), (0.0001, 0.002), (0.02, 0.5))])
    z = new_agents(3, 'circular')
    dt_zero = R.integrator.adaptive_timestep(z, 0.001, 0.01)
    save('misc', wrap_x=x, wrap_y=w, dt_agents=a, dts=dts, dt_zero=np.float64(dt_zero))


def navigation_cases():
    """Navigation.update with the reference's meshgrid indicer and getdefault
    on two seeded direction maps: agents on every target value (none, each
    map, beyond the maps), positions inside, on grid lines, just below the
    origin (truncation toward zero), beyond the far edge and far outside."""
    rng = np.random.default_rng(31)
    step, bounds = 0.25, (-2.0, 1.0, 8.0, 6.0)
    mg = RL.load_navigation().meshgrid(step, *bounds)
    ny, nx = mg.shape
    ang = rng.uniform(0, 2 * np.pi, (2, ny, nx))
    maps = [(np.cos(ang[k]), np.sin(ang[k])) for k in range(2)]
    out = {}
    for body in ('circular', 'three_circle'):
        n = 400
        a = new_agents(n, body)
        p = np.column_stack([rng.uniform(-3.0, 9.0, n), rng.uniform(0.0, 7.0, n)])
        edge = np.array([[-2.0, 1.0], [-2.1, 1.0], [-2.0, 0.9], [-2.24, 0.76], [-2.26, 1.0],
                         [8.0, 6.0], [8.2, 6.2], [8.25, 6.25], [8.3, 6.0], [1e6, 3.0],
                         [-1e6, 3.0], [0.0, 0.0], [3.0, 3.25], [3.125, 3.375]])
        p[:len(edge)] = edge
        a['position'] = p
        a['target'] = rng.integers(-1, 4, n)          # -1 none, 0-1 maps, 2-3 beyond
        a['target'][:len(edge)] = 0
        a['target_direction'] = np.column_stack([np.full(n, 7.0), np.full(n, -7.0)])
        before = a.copy()
        RL.navigation(a, maps, step, bounds)
        out[body + '_before'] = before
        out[body + '_after'] = a
    save('navigation', step=np.float64(step), bounds=np.array(bounds),
         dir_x=np.stack([m[0] for m in maps]), dir_y=np.stack([m[1] for m in maps]), **out)


def herding_cases():
    """LeaderFollowerWithHerding and LeaderFollower (simulation/logic.py:
    168-217) through the reference's own collective_motion code: a walled
    room with interior walls (line of sight), 10% leaders with targets, 70%
    followers, random velocities, some followers remembering a leader; the
    herding cell list (cell = follower sight) on the grid the device uses
    (the scenario's origin, ceil(extent / sight) cells per axis)."""
    import math
    R = RL.load()
    out = {}
    for mode, seed in (('herding', 41), ('leader', 42)):
        rng = np.random.default_rng(seed)
        scen = S.room(n=240, size=24.0, seed=seed)
        walls = S.walls_array([((6.0, 4.0), (6.0, 16.0)), ((12.0, 20.0), (20.0, 12.0)),
                               ((2.0, 10.0), (9.0, 10.5))])
        walls = np.concatenate([scen.walls, walls])
        a = scen.agents
        n = len(a)
        a['velocity'] = rng.normal(0, 1, (n, 2))
        a['velocity'][rng.uniform(size=n) < 0.05] = 0.0
        a['is_leader'] = rng.uniform(size=n) < 0.1
        a['is_follower'] = ~a['is_leader'] & (rng.uniform(size=n) < 0.7)
        a['target'] = np.where(a['is_leader'], rng.integers(0, 3, n), -1)
        a['familiar_exit'] = rng.integers(-1, 3, n)
        leaders = np.flatnonzero(a['is_leader'])
        mem = a['is_follower'] & (rng.uniform(size=n) < 0.3)
        a['index_leader'][mem] = rng.choice(leaders, mem.sum())
        before = a.copy()
        x0, y0, cell, nx, ny = scen.grid
        if mode == 'herding':
            sight = 10.0
            RL.configure_grid(x0, y0, sight, max(1, math.ceil(nx * cell / sight)),
                              max(1, math.ceil(ny * cell / sight)))
            d = R.collective_motion.leader_follower_with_herding_interaction(a, walls, sight, 5)
        else:
            d = R.collective_motion.leader_follower_interaction(a, walls, 20.0)
        f = a['is_follower']
        a['target_direction'][f] = d[f]
        out[mode + '_before'] = before
        out[mode + '_after'] = a.copy()
        out[mode + '_walls'] = walls
        out[mode + '_grid'] = np.array(scen.grid, dtype=np.float64)
    save('herding', **out)


def exit_cases():
    """ExitDetection (simulation/logic.py:220-237) through the reference's own
    exit_detection: a walled room with an interior wall, three door centres,
    followers taking the nearest visible door within 20 m."""
    R = RL.load()
    rng = np.random.default_rng(51)
    scen = S.room(n=300, size=30.0, seed=51)
    walls = np.concatenate([scen.walls, S.walls_array([((10.0, 5.0), (10.0, 25.0)),
                                                       ((18.0, 10.0), (26.0, 12.0))])])
    a = scen.agents
    n = len(a)
    a['is_follower'] = rng.uniform(size=n) < 0.6
    a['target'] = -1
    doors = np.array([[30.0, 15.0], [0.0, 15.0], [15.0, 30.0]])
    before = a.copy()
    targets, detected = R.evacuation.exit_detection(doors, a['position'], walls, 20.0)
    mask = a['is_follower'] & detected
    a['target'][mask] = targets[mask]
    a['is_follower'][mask] = False
    save('exit', before=before, after=a, walls=walls, doors=doors,
         grid=np.array(scen.grid, dtype=np.float64))


def input_digest(*arrays):
    """sha256 of the inputs' bytes (the fixture stores it instead of the
    inputs, which the seeded generators rebuild)."""
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


ROLLOUTS = {'hallway': (lambda: S.hallway(), 50, 7, 10),      # config 0: 400 Circular
            'room': (lambda: S.room(), 3, 8, 3)}              # config 1: 2000 ThreeCircle
ROLLOUT_FIELDS = ('position', 'velocity', 'force_prev', 'orientation', 'angular_velocity',
                  'torque_prev')


def rollout_noise(scen, steps, seed):
    """The host-drawn fluctuation noise of every step (drawn from the state's
    parameters, which do not change over a rollout)."""
    rng = np.random.default_rng(seed)
    out = [S.draw_noise(scen.agents, rng) for _ in range(steps)]
    return [f for f, _ in out], [m for _, m in out]


def rollout_cases():
    """The reference's own update() on config 0 (the 400-agent Circular
    hallway) for 50 steps and on config 1 (the 2000-agent ThreeCircle room)
    for 3 steps, with host-drawn noise, run with numba's scalar semantics;
    states every `every` steps."""
    out = {}
    for name, (make, steps, seed, every) in ROLLOUTS.items():
        scen = make()
        RL.configure_grid(*scen.grid)
        nf, nm = rollout_noise(scen, steps, seed)
        a = scen.agents.copy()
        out[name + '_digest'] = np.array(input_digest(a, scen.walls, *nf,
                                                      *[m for m in nm if m is not None]))
        dts = []
        for k in range(steps):
            dts.append(RL.step(a, scen.cell_size, scen.walls, nf[k], nm[k], scen.dt_min,
                               scen.dt_max, nodes=NODES_ALL, math='libm'))
            if (k + 1) % every == 0:
                for f in ROLLOUT_FIELDS:
                    if f in a.dtype.names:
                        out['%s_%s_%d' % (name, f, k + 1)] = np.ascontiguousarray(a[f])
            print(name, k + 1, flush=True)
        out[name + '_dt'] = np.array(dts)
    save('rollout', **out)


CASES = {'scenarios': lambda: (
             scenario_case('hallway_small', S.hallway(n=120, width=20.0, height=6.0, seed=3), 3,
                           21),
             scenario_case('room_small', S.room(n=150, size=12.0, seed=4), 3, 22)),
         'pairs': pair_cases, 'walls': wall_cases, 'misc': misc_cases,
         'navigation': navigation_cases, 'herding': herding_cases, 'exit': exit_cases,
         'rollout': rollout_cases}


def main():
    """Generate every fixture, or only the cases named on the command line."""
    if not RL.available():
        sys.exit('reference source tree not found; set CROWDDYNAMICS_REFERENCE')
    for name in (sys.argv[1:] or list(CASES)):
        CASES[name]()


if __name__ == '__main__':
    main()
