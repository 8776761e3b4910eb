"""Pin the C oracle against golden fixtures produced by the reference's own
hot-path code (tests/golden/make_golden.py).  CPU only."""
import os

import numpy as np
import pytest

from conftest import assert_vec_close

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
TOL = dict(rtol=1e-13, atol=1e-13)


def load(name):
    return np.load(os.path.join(GOLDEN, name + '.npz'))


FIELDS = ('position', 'velocity', 'force', 'force_prev', 'torque', 'torque_prev',
          'orientation', 'angular_velocity', 'target_orientation', 'position_ls',
          'position_rs')


def compare(got, ref, tol=TOL, what=''):
    for f in FIELDS:
        if f in ref.dtype.fields:
            assert_vec_close(got[f], ref[f], what='%s %s' % (what, f), **tol)


@pytest.mark.parametrize('case', ['hallway_small', 'room_small'])
def test_nodes(oracle, case, math_mode):
    g = load(case)
    grid = oracle.make_grid(*g['grid'])
    init = g['init']
    for node, flags in (('agent_agent', oracle.ORC_AGENT_AGENT),
                        ('agent_obstacle', oracle.ORC_AGENT_OBSTACLE),
                        ('adjusting', oracle.ORC_ADJUSTING | oracle.ORC_ORIENTATION),
                        ('orientation', oracle.ORC_ORIENTATION)):
        a = init.copy()
        oracle.step(a, grid, g['walls'], flags=flags)
        compare(a, g['node_' + node], what=node)


@pytest.fixture(params=[False, True], ids=['libm', 'exact_math'])
def math_mode(request, oracle):
    oracle.set_exact_math(request.param)
    yield request.param
    oracle.set_exact_math(False)


@pytest.mark.parametrize('case', ['hallway_small', 'room_small'])
@pytest.mark.parametrize('nthreads', [1, 4])
def test_steps(oracle, case, nthreads, math_mode):
    g = load(case)
    grid = oracle.make_grid(*g['grid'])
    a = g['init'].copy()
    three = 'torque' in a.dtype.fields
    for k in range(len(g['dt'])):
        dt = oracle.step(a, grid, g['walls'], g['noise_f'][k], g['noise_m'][k] if three else None,
                         dt_min=float(g['dt_min']), dt_max=float(g['dt_max']), nthreads=nthreads)
        if math_mode:
            assert abs(dt - g['dt'][k]) <= 1e-15 * g['dt'][k]
        else:
            assert dt == g['dt'][k]
        compare(a, g['states'][k], what='step %d' % k)


def test_pairs(oracle, math_mode):
    g = load('pairs')
    import ctypes
    for k in range(int(g['count'])):
        a = g['in_%d' % k].copy()
        three = 'torque' in a.dtype.fields
        x = (3.0 - 2.0, 3.0 - 2.0)
        grid = oracle.make_grid(-10.0, -10.0, 30.0, 1, 1)
        oracle.agent_agent_block_list(a, grid)
        compare(a, g['pair_%d' % k], what='pair %d' % k)


def test_walls(oracle, math_mode):
    g = load('walls')
    for model in ('circular', 'three_circle'):
        a = g['in_' + model].copy()
        oracle.agent_obstacle(a, g['walls'])
        compare(a, g['out_' + model], what='walls ' + model)


def test_misc(oracle):
    g = load('misc')
    for x, y in zip(g['wrap_x'], g['wrap_y']):
        assert oracle.wrap_to_pi(x) == y or (np.isnan(y) and np.isnan(oracle.wrap_to_pi(x)))
    a = g['dt_agents']
    for (lo, hi), dt in zip(((0.001, 0.01), (0.01, 0.01), (0.0001, 0.002), (0.02, 0.5)), g['dts']):
        assert oracle.adaptive_timestep(a, lo, hi) == dt
    from crowddynamics_gb300.simulation.agents import new_agents
    assert oracle.adaptive_timestep(new_agents(3, 'circular'), 0.001, 0.01) == g['dt_zero']


def test_oracle_navigation_matches_golden(oracle):
    """Navigation.update: the oracle's lookup reproduces the reference's
    meshgrid indicer + getdefault output bit for bit (fixture from the
    reference's own code)."""
    d = np.load(os.path.join(GOLDEN, 'navigation.npz'))
    b = d['bounds']
    for body in ('circular', 'three_circle'):
        a = d[body + '_before'].copy()
        oracle.navigation(a, d['dir_x'], d['dir_y'], b[0], b[1], float(d['step']))
        want = d[body + '_after']
        assert np.array_equal(a['target_direction'], want['target_direction']), body


def test_oracle_navigation_live_against_reference(oracle):
    """Fresh seeds: the oracle and the reference's own navigation code agree."""
    from oracle import ref_loader as RL
    if not RL.available():
        pytest.skip('reference source tree not present')
    from crowddynamics_gb300.simulation.agents import new_agents
    rng = np.random.default_rng(77)
    for step, bounds in ((0.1, (0.0, 0.0, 5.0, 3.0)), (0.05, (-1.5, 2.0, 2.5, 4.0))):
        mg = RL.load_navigation().meshgrid(step, *bounds)
        ny, nx = mg.shape
        maps = [(rng.normal(size=(ny, nx)), rng.normal(size=(ny, nx))) for _ in range(3)]
        a = new_agents(300, 'circular')
        a['position'] = np.column_stack([rng.uniform(bounds[0] - 1, bounds[2] + 1, 300),
                                         rng.uniform(bounds[1] - 1, bounds[3] + 1, 300)])
        a['target'] = rng.integers(-1, 4, 300)
        a['target_direction'] = rng.normal(size=(300, 2))
        ref = a.copy()
        RL.navigation(ref, maps, step, bounds)
        oracle.navigation(a, np.stack([m[0] for m in maps]), np.stack([m[1] for m in maps]),
                          bounds[0], bounds[1], step)
        assert np.array_equal(a['target_direction'], ref['target_direction'])


def test_herding_fixture_reproduces_reference():
    """The herding fixture is the reference's own collective_motion output
    (re-run live when the reference source is present)."""
    import math
    from oracle import ref_loader as RL
    if not RL.available():
        pytest.skip('reference source tree not present')
    R = RL.load()
    d = np.load(os.path.join(GOLDEN, 'herding.npz'))
    for mode in ('herding', 'leader'):
        a = d[mode + '_before'].copy()
        walls = d[mode + '_walls']
        x0, y0, cell, nx, ny = d[mode + '_grid']
        if mode == 'herding':
            RL.configure_grid(x0, y0, 10.0, max(1, math.ceil(nx * cell / 10.0)),
                              max(1, math.ceil(ny * cell / 10.0)))
            e = R.collective_motion.leader_follower_with_herding_interaction(a, walls, 10.0, 5)
        else:
            e = R.collective_motion.leader_follower_interaction(a, walls, 20.0)
        f = a['is_follower']
        a['target_direction'][f] = e[f]
        want = d[mode + '_after']
        for name in ('target_direction', 'target', 'index_leader'):
            assert np.array_equal(a[name], want[name]), (mode, name)


def test_exit_fixture_reproduces_reference():
    from oracle import ref_loader as RL
    if not RL.available():
        pytest.skip('reference source tree not present')
    R = RL.load()
    d = np.load(os.path.join(GOLDEN, 'exit.npz'))
    a = d['before'].copy()
    targets, detected = R.evacuation.exit_detection(d['doors'], a['position'], d['walls'], 20.0)
    mask = a['is_follower'] & detected
    a['target'][mask] = targets[mask]
    a['is_follower'][mask] = False
    assert np.array_equal(a, d['after'])


# ---- the reference's own update() at scale (tests/golden/rollout.npz) -------

def _rollout_inputs(name):
    """The seeded inputs of the rollout fixture, rebuilt and checked against
    the digest it stores."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        'make_golden', os.path.join(GOLDEN, 'make_golden.py'))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    make, steps, seed, every = mg.ROLLOUTS[name]
    scen = make()
    nf, nm = mg.rollout_noise(scen, steps, seed)
    digest = mg.input_digest(scen.agents, scen.walls, *nf, *[m for m in nm if m is not None])
    return scen, nf, nm, steps, every, digest, mg.ROLLOUT_FIELDS


@pytest.mark.parametrize('name', ['hallway', 'room'])
def test_oracle_reproduces_reference_rollouts(oracle, name):
    """The C oracle with the C library's elementary functions reproduces the
    reference's own update(), run with numba's scalar semantics, bit for bit:
    config 0 (400 Circular agents, two walls) over 50 steps and config 1
    (2000 ThreeCircle agents in the 30 m room) over 3 steps, with host noise."""
    g = load('rollout')
    scen, nf, nm, steps, every, digest, fields = _rollout_inputs(name)
    assert str(g[name + '_digest']) == digest, 'the seeded inputs changed'
    grid = oracle.make_grid(*scen.grid)
    a = scen.agents.copy()
    for k in range(steps):
        dt = oracle.step(a, grid, scen.walls, nf[k], nm[k], dt_min=scen.dt_min,
                         dt_max=scen.dt_max)
        assert dt == g[name + '_dt'][k], k
        if (k + 1) % every == 0:
            for f in fields:
                if f in a.dtype.names:
                    ref = g['%s_%s_%d' % (name, f, k + 1)]
                    got = np.ascontiguousarray(a[f])
                    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), \
                        (k + 1, f, float(np.abs(got - ref).max()))
