"""The reference's own known-answer tests, restated, run on the oracle (CPU),
plus live oracle-vs-reference checks on fresh seeds when the reference source
tree is present.

Known answers (paths inside the crowddynamics project):
* core/motion/tests/test_power_law_benchmark.py:13-35 -- agents at (0,0) and
  (2,0) both moving +x at 1 m/s feel zero social force;
* :38-63 -- a head-on approach gives a non-zero force on both;
* core/tests/test_integrator.py:8-53 -- dt_min <= dt <= dt_max;
* examples/tests/test_validation.py:32-57 -- a free walker covers >= 10 m in
  1000 steps; in a head-on encounter agent 0 still covers >= 8 m.
"""
import math

import numpy as np
import pytest

from conftest import assert_vec_close
from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.simulation.agents import new_agents, shoulders


def validation_agents(model, orientations, positions):
    """Attributes of examples/validation.py:26-39 (radius 0.255 with the
    adult ratios, v0 = 1, mass 73.5, velocity along the orientation)."""
    a = new_agents(len(positions), model)
    a['radius'] = 0.255
    a['r_t'], a['r_s'], a['r_ts'] = 0.5882 * 0.255, 0.3725 * 0.255, 0.6275 * 0.255
    a['target_velocity'] = 1.0
    a['mass'] = 73.5
    a['inertia_rot'] = 4.0 * np.pi * (73.5 / 80.0) * (0.255 / 0.27) ** 2
    for k, (phi, p) in enumerate(zip(orientations, positions)):
        e = (math.cos(phi), math.sin(phi))
        a[k]['velocity'] = e
        a[k]['target_direction'] = e
        a[k]['position'] = p
        if model == 'three_circle':
            a[k]['orientation'] = phi
            a[k]['target_orientation'] = phi
    if model == 'three_circle':
        shoulders(a)
    return a


@pytest.mark.parametrize('model', ['circular', 'three_circle'])
def test_social_force_known_answers(oracle, model):
    grid = oracle.make_grid(-10, -10, 30.0, 1, 1)
    a = validation_agents(model, [0.0, 0.0], [(0.0, 0.0), (2.0, 0.0)])
    oracle.agent_agent_block_list(a, grid)
    assert np.all(a['force'] == 0)
    b = validation_agents(model, [0.0, math.pi], [(0.0, 0.0), (2.0, 0.0)])
    oracle.agent_agent_block_list(b, grid)
    assert np.all(np.hypot(*b['force'].T) > 0)


@pytest.mark.parametrize('model', ['circular', 'three_circle'])
def test_adaptive_timestep_bounds(oracle, model):
    scen = S.hallway(n=50, width=15.0, height=6.0, seed=1) if model == 'circular' \
        else S.room(n=60, size=10.0, seed=2)
    rng = np.random.default_rng(0)
    scen.agents['velocity'] = rng.uniform(0, 3, (len(scen.agents), 2))
    for dt_min, dt_max in ((1e-3, 1e-2), (0.1, 0.2), (1e-5, 5.0), (0.01, 0.01)):
        dt = oracle.adaptive_timestep(scen.agents, dt_min, dt_max)
        assert dt_min <= dt <= dt_max


def run_validation(oracle, model, positions, orientations, noise, steps=1000):
    a = validation_agents(model, orientations, positions)
    grid = oracle.make_grid(-20, -20, 3.6, 12, 12)
    start = a['position'].copy()
    rng = np.random.default_rng(0)
    flags = oracle.ORC_ORIENTATION | oracle.ORC_ADJUSTING | oracle.ORC_INTEGRATE | oracle.ORC_RESET
    if noise:
        flags |= oracle.ORC_FLUCTUATION | oracle.ORC_AGENT_AGENT
    for _ in range(steps):
        nf, nm = S.draw_noise(a, rng) if noise else (None, None)
        oracle.step(a, grid, None, nf, nm, flags=flags, dt_min=0.01, dt_max=0.01)
    return np.hypot(*(a['position'] - start).T)


@pytest.mark.parametrize('model', ['circular', 'three_circle'])
def test_validation_movement(oracle, model):
    d = run_validation(oracle, model, [(0.0, 0.0)], [0.0], noise=False)
    assert d[0] >= 10.0 or np.isclose(d[0], 10.0)


@pytest.mark.parametrize('model', ['circular', 'three_circle'])
def test_validation_agent_interaction(oracle, model):
    d = run_validation(oracle, model, [(0.0, 0.0), (5.0, 0.0)], [0.0, math.pi], noise=True)
    assert d[0] >= 8.0 or np.isclose(d[0], 8.0)


# ---- live comparison with the reference's own code -------------------------

@pytest.fixture(scope='module')
def reference():
    from oracle import ref_loader as RL
    if not RL.available():
        pytest.skip('reference source tree not present')
    RL.load()
    return RL


@pytest.mark.parametrize('seed', [101, 102, 103])
def test_oracle_matches_reference_code(oracle, reference, seed):
    rng = np.random.default_rng(seed)
    for scen in (S.hallway(n=int(rng.integers(20, 80)), width=12.0, height=5.0, seed=seed),
                 S.room(n=int(rng.integers(20, 80)), size=9.0, seed=seed)):
        # random velocities make contacts, near-misses and both tau branches likely
        scen.agents['velocity'] = rng.normal(0, 1.0, (len(scen.agents), 2))
        reference.configure_grid(*scen.grid)
        a_ref = scen.agents.copy()
        a_orc = scen.agents.copy()
        grid = oracle.make_grid(*scen.grid)
        noise_rng = np.random.default_rng(seed)
        for _ in range(2):
            nf, nm = S.draw_noise(a_ref, noise_rng)
            dt_r = reference.step(a_ref, scen.cell_size, scen.walls, nf, nm)
            dt_o = oracle.step(a_orc, grid, scen.walls, nf, nm)
            assert dt_r == dt_o
        for f in ('position', 'velocity', 'force_prev'):
            assert_vec_close(a_orc[f], a_ref[f], 1e-13, 1e-13, f)
        if scen.body == 'three_circle':
            for f in ('orientation', 'torque_prev', 'position_ls'):
                assert_vec_close(a_orc[f], a_ref[f], 1e-13, 1e-13, f)


def test_oracle_matches_reference_rollout_50_steps(oracle, reference):
    """Config 0 (400 Circular agents) over 50 steps with host noise: the
    reference's own update() with numba's scalar semantics and the C oracle
    with the C library's functions stay bit-identical."""
    scen = S.hallway()
    reference.configure_grid(*scen.grid)
    grid = oracle.make_grid(*scen.grid)
    a_ref, a_orc = scen.agents.copy(), scen.agents.copy()
    rng = np.random.default_rng(7)
    for k in range(50):
        nf, nm = S.draw_noise(a_ref, rng)
        dt_r = reference.step(a_ref, scen.cell_size, scen.walls, nf, nm, math='libm')
        dt_o = oracle.step(a_orc, grid, scen.walls, nf, nm)
        assert dt_r == dt_o, k
    for f in ('position', 'velocity', 'force_prev'):
        assert np.array_equal(a_ref[f], a_orc[f]), f
