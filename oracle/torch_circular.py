"""Pure-PyTorch float64 restatement of the Circular step (test infrastructure).

Checker for the hand-written adjoint: the same step as the oracle
(core/interactions.py:51-70,107-120; core/motion/power_law.py:213-259;
core/motion/contact.py:12-48; core/motion/adjusting.py:16-51;
core/integrator.py:29-97,164-176), written with dense all-pairs tensors and
torch.where branches so that torch.autograd differentiates it.  All pairs
are evaluated (pairs with skin distance h >= 3 contribute nothing, as in the
reference), so no cell list is needed; sums run in a different order than the
reference's, so values agree to rounding, not bit for bit.
"""
import numpy as np
import torch

SIGTH_SOC = 3.0
F_SOC_MAX = 2e3
TAU_MAX = 30.0


def _safe(cond, x, fill=1.0):
    return torch.where(cond, x, torch.full_like(x, fill))


def forces(x, v, m, r, tau_adj, v0, e0, tau0, k, mu, kappa, damp, walls):
    n = x.shape[0]
    F = (m / tau_adj)[:, None] * (v0[:, None] * e0 - v)
    xr = x[:, None, :] - x[None, :, :]
    vr = v[:, None, :] - v[None, :, :]
    eye = torch.eye(n, dtype=torch.bool)
    d = torch.sqrt(_safe(~eye, (xr * xr).sum(-1)))      # diagonal unused (sqrt(0) has no gradient)
    rt = r[:, None] + r[None, :]
    h = d - rt
    act = (h < SIGTH_SOC) & ~eye
    a = (vr * vr).sum(-1)
    b = -(xr * vr).sum(-1)
    c = (xr * xr).sum(-1) - rt * rt
    disc = b * b - a * c
    ok = act & (disc > 0) & (a != 0)
    dd = torch.sqrt(_safe(ok, disc))
    a_s = _safe(ok, a)
    tau = (b - dd) / a_s
    ok = ok & (tau > 0) & (tau <= TAU_MAX)
    tau_s = _safe(ok, tau)
    dd_s = _safe(ok, dd)
    a_s = _safe(ok, a_s)
    g = (vr - (vr * b[..., None] + xr * a_s[..., None]) / dd_s[..., None]) / a_s[..., None]
    cm = (-m * k)[:, None]
    t0 = tau0[:, None]
    mag = (2.0 / tau_s + 1.0 / t0) * torch.exp(-tau_s / t0) / (tau_s * tau_s)
    Fs = (cm * mag)[..., None] * g
    L = torch.sqrt(_safe(ok, (Fs * Fs).sum(-1)))
    trunc = ok & (L > F_SOC_MAX)
    Fs = torch.where(trunc[..., None], Fs * (F_SOC_MAX / _safe(trunc, L))[..., None], Fs)
    Fs = torch.where(ok[..., None], Fs, torch.zeros_like(Fs))
    con = act & (h < 0) & (d != 0)
    d_s = _safe(con, d)
    nrm = xr / d_s[..., None]
    tng = torch.stack((nrm[..., 1], -nrm[..., 0]), -1)
    vt = (vr * tng).sum(-1)
    vn = (vr * nrm).sum(-1)
    Fc = (-h)[..., None] * (mu[:, None, None] * nrm - (kappa[:, None] * vt)[..., None] * tng) + \
        (damp[:, None] * vn)[..., None] * nrm
    Fc = torch.where(con[..., None], Fc, torch.zeros_like(Fc))
    F = F + (Fs + Fc).sum(1)
    for w in walls:
        p0, p1 = w[0:2], w[2:4]
        dv = p1 - p0
        lw = torch.sqrt((dv * dv).sum())
        tw = dv / lw
        nw = torch.stack((-tw[1], tw[0]))
        q0, q1 = x - p0, x - p1
        lt = -(q1 @ tw) - (q0 @ tw)
        end0, end1 = lt > lw, lt < -lw
        qe = torch.where(end0[:, None], q0, q1)
        de = torch.sqrt((qe * qe).sum(-1))
        ln = q0 @ nw
        perp = ~(end0 | end1)
        dist = torch.where(perp, ln.abs(), de)
        nrm = torch.where(perp[:, None], torch.sign(ln)[:, None] * nw, qe / _safe(~perp, de)[:, None])
        hw = dist - r
        con = hw < 0
        tng = torch.stack((nrm[:, 1], -nrm[:, 0]), -1)
        vt = (v * tng).sum(-1)
        vn = (v * nrm).sum(-1)
        Fw = (-hw)[:, None] * (mu[:, None] * nrm - (kappa * vt)[:, None] * tng) + \
            (damp * vn)[:, None] * nrm
        F = F + torch.where(con[:, None], Fw, torch.zeros_like(Fw))
    return F


def step(x, v, fp, m, r, tau_adj, v0, e0, tau0, k, mu, kappa, damp, walls, dt_min, dt_max,
         f_start=None):
    """One update; ``f_start`` is the force array's value before the force
    nodes add to it (zero after a reset)."""
    F = forces(x, v, m, r, tau_adj, v0, e0, tau0, k, mu, kappa, damp, walls)
    if f_start is not None:
        F = f_start + F
    vmax = torch.sqrt((v * v).sum(-1).max())
    if float(vmax.detach()) == 0.0:
        dt = torch.tensor(dt_max, dtype=torch.float64)
    else:
        dt = 1.1 * v0.max() * dt_max / vmax
        dt = torch.clamp(dt, dt_min, dt_max)
    vn = v + (fp / m[:, None] + F / m[:, None]) / 2 * dt
    xn = x + (vn * dt + F / m[:, None] / 2 * dt * dt)
    return xn, vn, F


def rollout_loss(agents, walls_rows, target, steps, tau_adj, v0, tau0, k, dt_min=0.001,
                 dt_max=0.01):
    """Differentiable loss of the same rollout as cd_rollout_loss."""
    T = lambda name: torch.tensor(np.ascontiguousarray(agents[name]), dtype=torch.float64)
    x, v, fp = T('position'), T('velocity'), T('force_prev')
    m, r, e0 = T('mass'), T('radius'), T('target_direction')
    mu, kappa, damp = T('mu'), T('kappa'), T('damping')
    walls = [torch.tensor(w, dtype=torch.float64) for w in walls_rows]
    tgt = torch.tensor(target, dtype=torch.float64)
    f_start = T('force')                       # the array's force before step 0
    loss = torch.zeros((), dtype=torch.float64)
    for t in range(steps):
        x, v, fp = step(x, v, fp, m, r, tau_adj, v0, e0, tau0, k, mu, kappa, damp, walls,
                        dt_min, dt_max, f_start if t == 0 else None)
        loss = loss + ((x - tgt[t]) ** 2).sum()
    return loss / (steps * len(agents))
