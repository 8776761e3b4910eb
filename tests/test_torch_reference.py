"""The pure-PyTorch float64 step used to check the adjoint agrees with the C
oracle (CPU)."""
import numpy as np
import pytest

torch = pytest.importorskip('torch')

from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.engine import walls_as_rows
from conftest import assert_vec_close


def test_torch_step_matches_oracle(oracle):
    from oracle import torch_circular as TC
    scen = S.hallway(n=80, width=16.0, height=6.0, seed=7)
    a = scen.agents
    a['velocity'] = np.random.default_rng(2).normal(0, 1.0, (len(a), 2))
    ref = a.copy()
    grid = oracle.make_grid(*scen.grid)
    T = lambda name: torch.tensor(np.ascontiguousarray(a[name]), dtype=torch.float64)
    x, v, fp = T('position'), T('velocity'), T('force_prev')
    walls = [torch.tensor(w) for w in walls_as_rows(scen.walls)]
    for _ in range(5):
        oracle.step(ref, grid, scen.walls, flags=4 | 8 | 16 | 32 | 64, dt_min=0.001, dt_max=0.01)
        x, v, fp = TC.step(x, v, fp, T('mass'), T('radius'), T('tau_adj'), T('target_velocity'),
                           T('target_direction'), T('tau_0'), T('k_soc'), T('mu'), T('kappa'),
                           T('damping'), walls, 0.001, 0.01)
    assert_vec_close(x.numpy(), ref['position'], 1e-11, 1e-11, 'position')
    assert_vec_close(fp.numpy(), ref['force_prev'], 1e-9, 1e-9, 'force_prev')


def test_torch_gradient_finite(oracle):
    from oracle import torch_circular as TC
    scen = S.hallway(n=40, width=10.0, height=5.0, seed=8)
    a = scen.agents
    p = [torch.tensor(np.ascontiguousarray(a[k]), dtype=torch.float64, requires_grad=True)
         for k in ('tau_adj', 'target_velocity', 'tau_0', 'k_soc')]
    target = np.repeat(a['position'][None], 5, axis=0) + 0.1
    loss = TC.rollout_loss(a, walls_as_rows(scen.walls), target, 5, *p)
    loss.backward()
    for t in p:
        assert torch.isfinite(t.grad).all()
