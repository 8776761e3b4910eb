"""Hand-written adjoint of the Circular rollout (cd_rollout_loss) on the GPU,
checked against the float64 autograd of the pure-torch step, against central
finite differences (h = 1e-6) of the device loss, and for invariance under
the checkpoint interval."""
import numpy as np
import pytest

torch = pytest.importorskip('torch')

from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.engine import batch_from_scenarios
from crowddynamics_gb300.exceptions import InvalidType, InvalidValue

pytestmark = pytest.mark.gpu

NODES = 4 | 8 | 16 | 32 | 64           # adjusting, agent-agent, agent-wall, integrate, reset
STEPS = 12
CKPT = 5                                # 12 = 5 + 5 + 2: a partial last segment


def _case(kind, seed=3):
    """(scenario, initial agents, target trajectory).  'sparse': 60 agents with
    fast random velocities (max|v| > 1.1 max v0, so dt is not clamped and its
    own gradient is exercised).  'dense': 130 lattice-placed agents in contact
    with a non-zero initial force array."""
    from crowddynamics_gb300.adjoint import make_target
    rng = np.random.default_rng(seed)
    if kind == 'sparse':
        scen = S.hallway(n=60, width=14.0, height=5.0, seed=seed)
        a = scen.agents
        a['velocity'] = rng.normal(0.0, 1.5, (len(a), 2))
    else:
        scen = S.hallway(n=130, width=14.0, height=5.0, seed=seed)
        a = scen.agents
        a['force'] = rng.normal(0.0, 50.0, (len(a), 2))
    n = len(a)
    a['tau_adj'] = rng.uniform(0.3, 0.7, n)
    a['target_velocity'] = rng.normal(1.2, 0.2, n)
    hidden = {'tau_adj': rng.uniform(0.3, 0.7, n),
              'target_velocity': rng.normal(1.2, 0.2, n)}
    target = make_target(scen, hidden, STEPS)
    return scen, a.copy(), target


def _device(scen, agents, variant=None):
    """A context for the scenario; `variant` 14 (the pair pipeline with the
    force pass) instead of the small-scenario default makes the rollout's
    recomputation context keep each step's cell list and near lists for the
    reverse pass."""
    b, _, walls = batch_from_scenarios([scen])
    if variant is not None:
        b.set_variant(variant)
    b.upload(agents)
    return b, walls


def _loss(scen, agents, target, ckpt=CKPT, grads=True, variant=None):
    b, _ = _device(scen, agents, variant)
    try:
        return b.rollout_loss(STEPS, target, ckpt, grads=grads)
    finally:
        b.close()


@pytest.mark.parametrize('variant', [None, 14])
@pytest.mark.parametrize('kind', ['sparse', 'dense'])
def test_adjoint_matches_torch_autograd(native, kind, variant):
    from oracle import torch_circular as TC
    from crowddynamics_gb300.adjoint import PARAMS
    scen, a, target = _case(kind)
    b, walls = _device(scen, a, variant)
    loss, g, fms, ams = b.rollout_loss(STEPS, target, CKPT)
    b.close()
    p = [torch.tensor(np.ascontiguousarray(a[k]), dtype=torch.float64, requires_grad=True)
         for k in PARAMS]
    lt = TC.rollout_loss(a, walls, target, STEPS, *p, dt_min=scen.dt_min, dt_max=scen.dt_max)
    lt.backward()
    assert abs(loss - lt.item()) <= 1e-10 * abs(lt.item()), (loss, lt.item())
    gt = np.stack([t.grad.numpy() for t in p], 1)
    assert np.isfinite(g).all()
    for col, name in enumerate(PARAMS):
        scale = np.abs(gt[:, col]).max()
        err = np.abs(g[:, col] - gt[:, col]).max()
        assert scale > 0, name
        # float64 gradients of the same function, summed in different orders
        assert err <= 1e-8 * scale, (name, err, scale)
    assert fms > 0 and ams > 0


@pytest.mark.parametrize('kind', ['sparse', 'dense'])
def test_adjoint_matches_central_differences(native, kind):
    """Central differences of the device loss with h = 1e-6 (relative to
    each parameter), falling back to h = 1e-7.  The reference's social force
    is cut off at skin distance 3 m and at time-to-collision 30 s with a
    non-zero value just inside, so the loss is piecewise smooth with small
    jumps; a difference whose +-h points straddle one sees jump / (2h) on top
    of the derivative (the 'sparse' case loses 2.5e-4 relative at h = 1e-6
    and 9e-7 at 1e-7; the pure-torch loss gives the same differences)."""
    from crowddynamics_gb300.adjoint import PARAMS
    scen, a, target = _case(kind)
    loss, g, _, _ = _loss(scen, a, target)
    rng = np.random.default_rng(11)

    def fd(direction, h):
        lo, hi = a.copy(), a.copy()
        for col, name in enumerate(PARAMS):
            hi[name] = a[name] + h * direction[:, col]
            lo[name] = a[name] - h * direction[:, col]
        return (_loss(scen, hi, target, grads=False)[0] -
                _loss(scen, lo, target, grads=False)[0]) / (2 * h)

    def check(direction, what):
        got = float((g * direction).sum())
        errs = []
        for h in (1e-6, 1e-7):
            want = fd(direction, h)
            errs.append((h, want, abs(got - want) / abs(want)))
            if errs[-1][2] <= 1e-5:
                return
        raise AssertionError('%s: adjoint %r, central differences %r' % (what, got, errs))

    # directional derivative along a random direction scaled by each parameter
    base = np.stack([np.ascontiguousarray(a[k]) for k in PARAMS], 1)
    check(rng.normal(size=base.shape) * np.abs(base), 'random direction')
    # single parameters: the agent with the largest gradient in each column
    for col, name in enumerate(PARAMS):
        i = int(np.argmax(np.abs(g[:, col])))
        e = np.zeros_like(base)
        e[i, col] = abs(base[i, col])
        check(e, '%s of agent %d' % (name, i))


@pytest.mark.parametrize('variant', [None, 14])
def test_checkpoint_interval_does_not_change_result(native, variant):
    scen, a, target = _case('sparse')
    ref = _loss(scen, a, target, ckpt=CKPT, variant=variant)
    for ckpt in (1, 4, STEPS, 100):
        got = _loss(scen, a, target, ckpt=ckpt, variant=variant)
        assert got[0] == ref[0], ckpt
        assert np.array_equal(got[1], ref[1]), ckpt
    again = _loss(scen, a, target, ckpt=CKPT, variant=variant)
    assert np.array_equal(again[1], ref[1])                 # deterministic
    if variant is not None:
        # the same gradient as the small-scenario default's (lane groups in
        # the forward, the reverse building its own near lists)
        other = _loss(scen, a, target, ckpt=CKPT)
        assert other[0] == ref[0]
        assert np.array_equal(other[1], ref[1])


@pytest.mark.parametrize('kind', ['sparse', 'dense'])
def test_rollout_leaves_the_forward_state(native, kind):
    """After cd_rollout_loss the context holds the state (and clock) of
    STEPS plain steps, bit for bit, and the loss equals the oracle's
    trajectory loss."""
    scen, a, target = _case(kind)
    b1, _ = _device(scen, a)
    loss, _, _, _ = b1.rollout_loss(STEPS, target, CKPT)
    r1 = a.copy()
    b1.download(r1)
    t1 = b1.time()
    b1.close()
    b2, _ = _device(scen, a)
    r2 = a.copy()
    pos = []
    for _ in range(STEPS):
        b2.step(NODES)
        b2.download(r2)
        pos.append(r2['position'].copy())
    t2 = b2.time()
    b2.close()
    for name in ('position', 'velocity', 'force', 'force_prev'):
        assert np.array_equal(r1[name], r2[name]), name
    assert np.array_equal(t1[0], t2[0]) and np.array_equal(t1[1], t2[1])
    want = sum(((p - target[t]) ** 2).sum() for t, p in enumerate(pos)) / (STEPS * len(a))
    assert abs(loss - want) <= 1e-13 * want


def test_autograd_function(native):
    from crowddynamics_gb300.adjoint import PARAMS, rollout_loss
    scen, a, target = _case('sparse')
    b, _ = _device(scen, a)
    ref_loss, ref_g, _, _ = b.rollout_loss(STEPS, target, CKPT)
    loss, params = rollout_loss(b, a, target, STEPS, checkpoint_every=CKPT)
    (3.0 * loss).backward()
    b.close()
    assert loss.item() == ref_loss
    for col, t in enumerate(params):
        assert np.array_equal(t.grad.numpy(), 3.0 * ref_g[:, col]), PARAMS[col]
    # no gradient requested: forward only, same loss
    b, _ = _device(scen, a)
    with torch.no_grad():
        l2, _ = rollout_loss(b, a, target, STEPS, checkpoint_every=CKPT)
    b.close()
    assert l2.item() == ref_loss


def test_rollout_rejects_bad_input(native):
    scen, a, target = _case('sparse')
    b, _ = _device(scen, a)
    with pytest.raises(InvalidValue):
        b.rollout_loss(STEPS, target[:-1], CKPT)
    with pytest.raises(InvalidValue):
        b.rollout_loss(STEPS, target, 0)
    b.close()
    tc = S.room(n=20, size=8.0, seed=1)                    # ThreeCircle
    bt, _, _ = batch_from_scenarios([tc])
    with pytest.raises(InvalidType):
        bt.rollout_loss(STEPS, np.zeros((STEPS, len(tc.agents), 2)), CKPT)
    bt.close()


def test_adjoint_over_capacity_fallback(native):
    """With the near-list capacity fixed below what the reverse pass needs,
    each reverse step runs the lane-group adjoint instead of the pair form:
    the same gradient up to summation order."""
    scen, a, target = _case('dense')
    ref = _loss(scen, a, target)
    b, _ = _device(scen, a)
    b.set_near_list_capacity(0)
    got = b.rollout_loss(STEPS, target, CKPT)
    b.close()
    assert got[0] == ref[0]                      # the forward is unchanged
    scale = np.abs(ref[1]).max(0)
    assert np.all(np.abs(got[1] - ref[1]) <= 1e-10 * scale)


def test_second_rollout_after_new_agents(native):
    """The rollout's recomputation context takes the agents of each call: a
    second rollout on the same context after a new upload (other tau_adj and
    target speeds) gives the loss and gradients of a fresh context, bit for
    bit."""
    scen, a, target = _case('dense')
    b, _ = _device(scen, a)
    b.rollout_loss(STEPS, target, CKPT)                 # makes the recomputation context
    a2 = a.copy()
    rng = np.random.default_rng(11)
    a2['tau_adj'] = rng.uniform(0.3, 0.7, len(a2))
    a2['target_velocity'] = rng.normal(1.2, 0.2, len(a2))
    b.upload(a2)
    got = b.rollout_loss(STEPS, target, CKPT)
    b.close()
    ref = _loss(scen, a2, target)
    assert got[0] == ref[0]
    assert np.array_equal(got[1], ref[1])
