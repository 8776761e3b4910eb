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
