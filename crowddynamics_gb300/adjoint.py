"""Differentiable rollouts of Circular crowds through the hand-written adjoint.

``RolloutLoss`` is a ``torch.autograd.Function`` over per-agent parameters
(tau_adj, target_velocity, tau_0, k_soc): its forward runs the device
rollout (``cd_rollout_loss``) and, when any input needs a gradient, the
hand-written adjoint of the whole rollout in the same call (checkpoint every
``checkpoint_every`` steps, recomputation in between); backward returns the
stored gradients scaled by the incoming one.  PyTorch is only the autograd
wrapper: every number comes from the CUDA kernels.

Loss: mean over steps t and agents i of |x_i(t) - target[t][i]|^2, with x(t)
the positions after step t of the standard node tree (adjusting, agent-agent,
agent-wall, integrate, reset) without fluctuation.
"""
import numpy as np
import torch

from crowddynamics_gb300.engine import DeviceBatch, batch_from_scenarios
from crowddynamics_gb300.exceptions import InvalidType

PARAMS = ('tau_adj', 'target_velocity', 'tau_0', 'k_soc')


class RolloutLoss(torch.autograd.Function):
    """loss = RolloutLoss.apply(tau_adj, target_velocity, tau_0, k_soc, batch,
    agents0, target, steps, checkpoint_every)"""

    @staticmethod
    def forward(ctx, tau_adj, target_velocity, tau_0, k_soc, batch, agents0, target, steps,
                checkpoint_every):
        a = agents0.copy()
        for name, t in zip(PARAMS, (tau_adj, target_velocity, tau_0, k_soc)):
            a[name] = t.detach().to('cpu', torch.float64).numpy()
        batch.upload(a)
        need = any(ctx.needs_input_grad[:4])
        loss, g, fms, ams = batch.rollout_loss(steps, target, checkpoint_every, grads=need)
        ctx.times = (fms, ams)
        if need:
            ctx.save_for_backward(torch.from_numpy(g).to(tau_adj.device))
        return torch.tensor(loss, dtype=torch.float64, device=tau_adj.device)

    @staticmethod
    def backward(ctx, gout):
        (g,) = ctx.saved_tensors
        return (gout * g[:, 0], gout * g[:, 1], gout * g[:, 2], gout * g[:, 3],
                None, None, None, None, None)


def rollout_loss(batch, agents0, target, steps, params=None, checkpoint_every=20):
    """Convenience: torch tensors of the four parameters (taken from
    ``agents0`` unless given), loss through ``RolloutLoss``."""
    if 'position_ls' in agents0.dtype.fields:
        raise InvalidType('the adjoint covers Circular agents only')
    if params is None:
        params = [torch.tensor(np.ascontiguousarray(agents0[n]), dtype=torch.float64, requires_grad=True)
                  for n in PARAMS]
    loss = RolloutLoss.apply(*params, batch, agents0, target, steps, checkpoint_every)
    return loss, params


def make_target(scenario, hidden, steps):
    """Target trajectory: the scenario rolled out on the device with the
    hidden parameters ``hidden`` (dict name -> array); returns (steps, n, 2)."""
    b, agents, _ = batch_from_scenarios([scenario])
    a = scenario.agents.copy()
    for k, v in hidden.items():
        a[k] = v
    b.upload(a)
    out = np.zeros((steps, len(a), 2))
    nodes = 4 | 8 | 16 | 32 | 64
    rec = a.copy()
    for t in range(steps):
        b.step(nodes)
        b.download(rec)
        out[t] = rec['position']
    b.close()
    return out
