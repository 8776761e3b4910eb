"""Device path vs the C oracle on seeded inputs, through the C ABI.

Two levels:
* against the oracle in exact-math mode (the device's elementary functions,
  no fused multiply-add on either side) every float64 result must be
  bit-identical, for single nodes, full steps and 50-step rollouts;
* against the plain oracle (C library functions) per-step forces and
  torques must agree within 1e-9 relative with a 1e-12 N (N m) floor.
Integer work (cell keys, cell order, candidate counts) must match bit for
bit.
"""
import numpy as np
import pytest

from conftest import assert_vec_close
from crowddynamics_gb300 import _native as N
from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.engine import DeviceBatch, batch_from_scenarios

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-9, 1e-12


def oracle_grid(O, scen):
    return O.make_grid(*scen.grid)


def device_step(scen, nodes, noise=None, variant=None):
    b, agents, _ = batch_from_scenarios([scen])
    if variant is not None:
        b.set_variant(variant)
    if noise is not None:
        b.set_noise(*noise)
    dt = b.step(nodes, want_dt=True)
    out = agents.copy()
    b.download(out)
    b.close()
    return out, dt[0]


ORC = {N.NODE_FLUCTUATION: 1, N.NODE_ORIENTATION: 2, N.NODE_ADJUSTING: 4,
       N.NODE_AGENT_AGENT: 8, N.NODE_AGENT_OBSTACLE: 16, N.NODE_INTEGRATE: 32,
       N.NODE_RESET: 64}


def orc_flags(nodes):
    return sum(v for k, v in ORC.items() if nodes & k)


def oracle_step(O, scen, nodes, noise=None, nthreads=1, exact=False):
    a = scen.agents.copy()
    nf, nm = noise if noise is not None else (None, None)
    O.set_exact_math(exact)
    try:
        dt = O.step(a, oracle_grid(O, scen), scen.walls, nf, nm, flags=orc_flags(nodes),
                    dt_min=scen.dt_min, dt_max=scen.dt_max, nthreads=nthreads)
    finally:
        O.set_exact_math(False)
    return a, dt


STATE = ('position', 'velocity', 'force', 'force_prev', 'torque', 'torque_prev',
         'orientation', 'angular_velocity', 'target_orientation', 'position_ls',
         'position_rs')


def assert_identical(got, ref, what=''):
    """Every state field bit for bit (signed zeros included; any NaN matches
    any NaN)."""
    for f in STATE:
        if f in ref.dtype.fields:
            g, r = np.ascontiguousarray(got[f]), np.ascontiguousarray(ref[f])
            same = (g.view(np.uint64) == r.view(np.uint64)) | (np.isnan(g) & np.isnan(r))
            if not same.all():
                k = np.argwhere(~same)[0]
                raise AssertionError('%s %s differs at %s: %r vs %r (%d values)' % (
                    what, f, k, g[tuple(k)], r[tuple(k)], int((~same).sum())))


def moving(scen, seed=3):
    """Random velocities, so that every branch of the social force (defined
    and undefined roots, both tau signs, the tau cut-off) is exercised."""
    scen.agents['velocity'] = np.random.default_rng(seed).normal(0, 1.0, (len(scen.agents), 2))
    return scen


SCENARIOS = {
    'hallway': lambda: S.hallway(),
    'room': lambda: S.room(),
    'room_moving': lambda: moving(S.room()),
    'hallway_moving': lambda: moving(S.hallway()),
}


@pytest.mark.parametrize('name', sorted(SCENARIOS))
@pytest.mark.parametrize('nodes', [N.NODE_AGENT_AGENT, N.NODE_AGENT_OBSTACLE,
                                   N.NODE_ADJUSTING | N.NODE_ORIENTATION])
def test_node_forces(oracle, native, name, nodes):
    scen = SCENARIOS[name]()
    got, _ = device_step(scen, nodes)
    assert_identical(got, oracle_step(oracle, scen, nodes, exact=True)[0], 'exact')
    ref, _ = oracle_step(oracle, scen, nodes)
    assert_vec_close(got['force'], ref['force'], RTOL, ATOL, 'force')
    if scen.body == 'three_circle':
        assert_vec_close(got['torque'], ref['torque'], RTOL, ATOL, 'torque')
        assert_vec_close(got['target_orientation'], ref['target_orientation'], 1e-15, 1e-15,
                         'target_orientation')


@pytest.mark.parametrize('name', sorted(SCENARIOS))
def test_full_step(oracle, native, name):
    scen = SCENARIOS[name]()
    rng = np.random.default_rng(11)
    noise = S.draw_noise(scen.agents, rng)
    got, dt_g = device_step(scen, N.NODE_ALL, noise)
    exact, dt_e = oracle_step(oracle, scen, N.NODE_ALL, noise, exact=True)
    assert dt_g == dt_e
    assert_identical(got, exact, 'exact')
    ref, dt_r = oracle_step(oracle, scen, N.NODE_ALL, noise)
    assert abs(dt_g - dt_r) <= 1e-15 * dt_r
    for f in ('force_prev', 'velocity', 'position'):
        assert_vec_close(got[f], ref[f], RTOL, ATOL, f)
    assert np.all(got['force'] == 0)
    if scen.body == 'three_circle':
        for f in ('torque_prev', 'angular_velocity', 'orientation'):
            assert_vec_close(got[f], ref[f], RTOL, ATOL, f)
        assert_vec_close(got['position_ls'], ref['position_ls'], RTOL, ATOL, 'position_ls')


@pytest.mark.parametrize('name', sorted(SCENARIOS))
@pytest.mark.parametrize('variant', range(15))
def test_full_step_every_variant(oracle, native, name, variant):
    """Each force-kernel launch variant (one lane per agent, 4 to 32 lanes
    sharing an agent, or the compute-once pair pipeline with its forces in
    the pair kernel or in a separate force pass) reproduces the oracle's step
    bit for bit."""
    assert len(N.variants()) == 15
    scen = SCENARIOS[name]()
    noise = S.draw_noise(scen.agents, np.random.default_rng(12))
    got, dt_g = device_step(scen, N.NODE_ALL, noise, variant=variant)
    exact, dt_e = oracle_step(oracle, scen, N.NODE_ALL, noise, exact=True)
    assert dt_g == dt_e
    assert_identical(got, exact, 'variant %d' % variant)


@pytest.mark.parametrize('name', sorted(SCENARIOS))
@pytest.mark.parametrize('capacity', [0, 10])
@pytest.mark.parametrize('variant', [10, 13])
def test_pair_pipeline_over_capacity(oracle, native, name, capacity, variant):
    """A pair-pipeline step whose near lists exceed the (fixed) capacity runs
    the lane-group kernel instead, with the same bit-exact results (with the
    forces in the pair kernel and with the force pass)."""
    scen = SCENARIOS[name]()
    noise = S.draw_noise(scen.agents, np.random.default_rng(13))
    b, agents, _ = batch_from_scenarios([scen])
    b.set_variant(variant)
    b.set_near_list_capacity(capacity)
    b.set_noise(*noise)
    dt = b.step(N.NODE_ALL, want_dt=True)
    got = agents.copy()
    b.download(got)
    b.close()
    exact, dt_e = oracle_step(oracle, scen, N.NODE_ALL, noise, exact=True)
    assert dt[0] == dt_e
    assert_identical(got, exact, 'capacity %d' % capacity)


def test_pair_pipeline_grows_capacity(native):
    """Automatic sizing from a too-small capacity: the first step runs the
    fallback, the capacity grows after it, the later steps run the pair
    pipeline; results stay identical to the one-lane kernel."""
    scen = S.hallway(n=2000, width=30.0, height=10.0, seed=9)
    outs = []
    for variant, cap in ((0, None), (10, 1000)):
        b, agents, _ = batch_from_scenarios([scen])
        b.set_variant(variant)
        if cap is not None:
            b.set_near_list_capacity(cap)
            b.run(2, N.NODE_ALL & ~N.NODE_FLUCTUATION)       # fixed: fallback steps
            b.set_near_list_capacity(-1)                     # grows after the next run
        else:
            b.run(2, N.NODE_ALL & ~N.NODE_FLUCTUATION)
        b.run(1, N.NODE_ALL & ~N.NODE_FLUCTUATION)
        b.run(5, N.NODE_ALL & ~N.NODE_FLUCTUATION)
        o = agents.copy()
        b.download(o)
        b.close()
        outs.append(o)
    assert_identical(outs[1], outs[0], 'pair pipeline vs one-lane kernel')


@pytest.mark.parametrize('name', sorted(SCENARIOS))
def test_rollout_50_steps(oracle, native, name):
    scen = SCENARIOS[name]()
    rng = np.random.default_rng(5)
    b, agents, _ = batch_from_scenarios([scen])
    ref = scen.agents.copy()
    grid = oracle_grid(oracle, scen)
    t_ref = 0.0
    with oracle.exact_math():
        for k in range(50):
            nf, nm = S.draw_noise(ref, rng)
            b.set_noise(nf, nm)
            b.step(N.NODE_ALL)
            t_ref += oracle.step(ref, grid, scen.walls, nf, nm, dt_min=scen.dt_min,
                                 dt_max=scen.dt_max)
    got = agents.copy()
    b.download(got)
    dt, tt = b.time()
    b.close()
    assert_identical(got, ref, 'rollout')
    assert tt[0] == t_ref
    d = np.hypot(*(got['position'] - ref['position']).T)
    assert d.max() <= 1e-6, d.max()


@pytest.mark.parametrize('grow', [0.0, 0.2])
def test_wall_bins_after_extent_growth(oracle, native, grow):
    """An upload whose agents outgrew the extent the wall bins were built
    for: the step right after it runs on the old bins (the grown agents scan
    every wall of the scenario), the bins are rebuilt at that step's
    synchronisation, and the second step runs on the new ones.  Both match
    the oracle bit for bit."""
    scen = S.hallway(n=300, seed=4, max_agent_radius=0.6)
    nodes = N.NODE_ALL & ~N.NODE_FLUCTUATION
    b, agents, _ = batch_from_scenarios([scen])
    b.step(nodes)
    rec = agents.copy()
    b.download(rec)
    y = rec['position'][:, 1]
    near = np.argsort(np.minimum(y, 10.0 - y))[:20]
    rec['radius'][near] += grow + 0.05
    ref = rec.copy()
    b.upload(rec)
    grid = oracle_grid(oracle, scen)
    with oracle.exact_math():
        for k in range(2):
            b.step(nodes)
            oracle.step(ref, grid, scen.walls, None, None, flags=orc_flags(nodes),
                        dt_min=scen.dt_min, dt_max=scen.dt_max)
            got = rec.copy()
            b.download(got)
            assert_identical(got, ref, 'step %d after the upload' % k)
    b.close()


def test_cell_list_bit_exact(oracle, native):
    for scen in (S.hallway(), S.room(), S.large_field(n=20000, size=140.0, n_walls=100, seed=9)):
        b, agents, _ = batch_from_scenarios([scen])
        b.step(N.NODE_AGENT_AGENT)
        keys, order, cnt, off = b.cell_list()
        b.close()
        x = np.ascontiguousarray(scen.agents['position'][:, 0])
        y = np.ascontiguousarray(scen.agents['position'][:, 1])
        k_ref, p_ref, c_ref, o_ref = oracle.cell_list(x, y, oracle_grid(oracle, scen))
        assert np.array_equal(keys, k_ref)
        assert np.array_equal(order, p_ref)
        assert np.array_equal(cnt, c_ref)
        assert np.array_equal(off, o_ref)


def test_candidate_pairs_bit_exact(oracle, native):
    """Per-agent number of candidate partners equals the restated cell_lists
    pair set, and every partner the pre-check keeps is a candidate."""
    for scen in (S.hallway(), S.room()):
        b, agents, _ = batch_from_scenarios([scen])
        counts = b.pair_counts()
        cand, near = counts[:, 0], counts[:, 1]
        b.close()
        x = np.ascontiguousarray(scen.agents['position'][:, 0])
        y = np.ascontiguousarray(scen.agents['position'][:, 1])
        pairs = oracle.candidate_pairs(x, y, oracle_grid(oracle, scen))
        ref = np.bincount(pairs.ravel(), minlength=len(x))
        assert np.array_equal(cand, ref)
        assert np.all(near <= cand)
        # every pair within the social range must survive the pre-check
        d = np.hypot(*(scen.agents['position'][pairs[:, 0]] - scen.agents['position'][pairs[:, 1]]).T)
        close = pairs[d < 3.0]
        need = np.bincount(close.ravel(), minlength=len(x))
        assert np.all(near >= need)


def social_branches_np(a, first, second):
    """(sub-pair loop run, defined roots, valid time-to-collision) per pair
    (first, second), restated from core/motion/power_law.py:213-363."""
    v = a['velocity'][first] - a['velocity'][second]
    av = (v * v).sum(1)
    if 'position_ls' not in a.dtype.names:
        x = a['position'][first] - a['position'][second]
        r = a['radius'][first] + a['radius'][second]
        b = -(x[:, 0] * v[:, 0] + x[:, 1] * v[:, 1])
        c = (x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) - r * r
        with np.errstate(invalid='ignore', divide='ignore'):
            d = np.sqrt(b * b - av * c)
            defined = ~(np.isnan(d) | (d == 0) | (av == 0))
            tau = (b - d) / av
        return np.ones(len(first), int), defined.astype(int), (defined & ~((tau <= 0) | (tau > 30))).astype(int)
    parts = ('position', 'position_ls', 'position_rs')
    radii = ('r_t', 'r_s', 'r_s')
    soc = av != 0
    tau = np.full(len(first), np.nan)
    ndef = np.zeros(len(first), int)
    for i in range(3):
        for j in range(3):
            x = a[parts[i]][first] - a[parts[j]][second]
            r = a[radii[i]][first] + a[radii[j]][second]
            b = -(x[:, 0] * v[:, 0] + x[:, 1] * v[:, 1])
            c = (x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) - r * r
            with np.errstate(invalid='ignore', divide='ignore'):
                d = np.sqrt(b * b - av * c)
                ok = soc & ~(np.isnan(d) | (d == 0))
                tn = (b - d) / av
            ndef += ok
            take = ok & (np.isnan(tau) | ((0 < tn) & (tn < tau)))
            tau = np.where(take, tn, tau)
    valid = soc & ~(np.isnan(tau) | (tau <= 0))
    return soc.astype(int), ndef, valid.astype(int)


def skin_distance_np(a, i, j):
    if 'position_ls' not in a.dtype.names:
        x = a['position'][i] - a['position'][j]
        return np.sqrt(x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) - (a['radius'][i] + a['radius'][j])
    parts = ('position', 'position_ls', 'position_rs')
    radii = ('r_t', 'r_s', 'r_s')
    h = np.full(len(i), np.inf)
    for p in range(3):
        for q in range(3):
            x = a[parts[p]][i] - a[parts[q]][j]
            h = np.minimum(h, np.sqrt(x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) -
                           (a[radii[p]][i] + a[radii[q]][j]))
    return h


def test_social_branch_counts(oracle, native):
    """The social-force branch counts used for work accounting equal a numpy
    restatement over the interacting pairs, each attributed to the pair's
    first agent (the lower cell-sorted slot)."""
    for scen in (S.hallway(), S.room()):
        b, agents, _ = batch_from_scenarios([scen])
        b.run(15, N.NODE_ALL & ~N.NODE_FLUCTUATION)      # agents under way
        a = agents.copy()
        b.download(a)
        counts = b.pair_counts()
        _, order, _, _ = b.cell_list()
        b.close()
        slot = np.empty(len(order), np.int64)
        slot[order] = np.arange(len(order))
        x = np.ascontiguousarray(a['position'][:, 0])
        y = np.ascontiguousarray(a['position'][:, 1])
        pairs = oracle.candidate_pairs(x, y, oracle_grid(oracle, scen))
        lo = np.where(slot[pairs[:, 0]] < slot[pairs[:, 1]], pairs[:, 0], pairs[:, 1])
        hi = np.where(slot[pairs[:, 0]] < slot[pairs[:, 1]], pairs[:, 1], pairs[:, 0])
        inter = skin_distance_np(a, lo, hi) < 3.0
        lo, hi = lo[inter], hi[inter]
        soc, ndef, valid = social_branches_np(a, lo, hi)
        n = len(a)
        assert np.array_equal(counts[:, 6], np.bincount(lo, soc, n).astype(int)), scen.name
        assert np.array_equal(counts[:, 7], np.bincount(lo, ndef, n).astype(int)), scen.name
        assert np.array_equal(counts[:, 8], np.bincount(lo, valid, n).astype(int)), scen.name
        assert counts[:, 8].sum() > 0


@pytest.mark.parametrize('move', [False, True])
def test_zero_force_torque_signs(oracle, native, move):
    """A ThreeCircle pair that exerts no force adds r x (+0, +0), a signed
    zero, to each agent's torque.  The pair kernel leaves its sign to the
    gather, which resolves it only when the agent's running torque is -0.
    Records whose torque starts at -0 (no adjusting, no reset), in a sparse
    room (a few partners per agent), make these terms decide the result:
    the torques must match the oracle bit for bit, and some agents with
    interacting partners must end at -0 (so adding +0 would be wrong)."""
    scen = S.room(n=60, seed=12)
    if move:
        scen = moving(scen, seed=5)
    scen.agents['torque'] = -0.0
    nodes = N.NODE_AGENT_AGENT | N.NODE_AGENT_OBSTACLE
    b, agents, _ = batch_from_scenarios([scen])
    inter = b.pair_counts()[:, 2]
    b.close()
    got, _ = device_step(scen, nodes)
    ref, _ = oracle_step(oracle, scen, nodes, exact=True)
    assert_identical(got, ref, 'zero-force torque')
    neg = np.signbit(ref['torque']) & (ref['torque'] == 0)
    assert (neg & (inter > 0)).any() and (~neg & (inter > 0)).any()


def edge_pairs(seed=17):
    """Isolated ThreeCircle pairs (15 m apart) placed at the edges of the
    pair kernel's float32 certificates: torso skin distance within 1e-7 ..
    1e-3 m of 3 (interaction) and of 0 (contact), exactly at them, and
    coincident centres; moving head-on, grazing (miss distance within 1e-9 m
    of the torsos' radii sum), receding, together (a = 0), with a relative
    speed of 1e-150 (a tiny) and of 1e-170 (a underflows to 0), or at random."""
    from crowddynamics_gb300.simulation.agents import new_agents, shoulders
    rng = np.random.default_rng(seed)
    cases = []
    for target in (3.0, 0.0):
        for dh in (-1e-3, -1e-5, -1e-7, 0.0, 1e-7, 1e-5, 1e-3):
            for motion in ('head_on', 'graze', 'receding', 'together', 'tiny', 'underflow',
                           'random'):
                cases.append((target + dh, motion))
    cases += [(None, 'random'), (None, 'head_on')]
    n = 2 * len(cases)
    a = new_agents(n, 'three_circle')
    S._three_circle_bodies(a, rng, n)
    side = int(np.ceil(np.sqrt(len(cases))))
    spacing = 15.0
    for k, (h, motion) in enumerate(cases):
        A, B = 2 * k, 2 * k + 1
        th = rng.uniform(0, 2 * np.pi)
        u = np.array([np.cos(th), np.sin(th)])
        nrm = np.array([-u[1], u[0]])
        a['orientation'][A], a['orientation'][B] = th, th + np.pi
        rsum = a['r_t'][A] + a['r_t'][B]
        d = 0.0 if h is None else h + rsum
        pa = np.array([10.0 + spacing * (k % side), 10.0 + spacing * (k // side)])
        a['position'][A] = pa
        a['position'][B] = pa + d * u
        v = rng.normal(0.0, 1.0, 2)
        if motion == 'head_on':
            va, vb = 0.8 * u, -0.8 * u
        elif motion == 'graze':
            s = min(1.0, (rsum + rng.choice([-1e-9, 1e-9])) / max(d, 1e-9))
            rel = 1.3 * (np.sqrt(1 - s * s) * u + s * nrm)      # from A towards B, missing by ~rsum
            va, vb = rel / 2, -rel / 2
        elif motion == 'receding':
            va, vb = -0.8 * u, 0.8 * u
        elif motion == 'together':
            va, vb = v, v
        elif motion == 'tiny':
            va, vb = v, v + 1e-150
        elif motion == 'underflow':
            va, vb = v, v + 1e-170
        else:
            va, vb = v, rng.normal(0.0, 1.0, 2)
        a['velocity'][A], a['velocity'][B] = va, vb
    e0 = rng.normal(0.0, 1.0, (n, 2))
    a['target_direction'] = e0 / np.hypot(*e0.T)[:, None]
    a['target_orientation'] = np.arctan2(a['target_direction'][:, 1], a['target_direction'][:, 0])
    shoulders(a)
    rows = int(np.ceil(len(cases) / side))
    bounds = (0.0, 0.0, 20.0 + spacing * side, 20.0 + spacing * rows)
    return S.Scenario('edge_pairs', a, S.walls_array([]), bounds, 3.6)


@pytest.mark.parametrize('variant', [9, 10, 11, 12, 14])
def test_certificate_edges(oracle, native, variant):
    """The pair kernel's float32 certificates (distance bounds, pre-selection,
    no time to collision) at their edges: one full step bit for bit."""
    scen = edge_pairs()
    nodes = N.NODE_ALL & ~N.NODE_FLUCTUATION
    got, _ = device_step(scen, nodes, variant=variant)
    ref, _ = oracle_step(oracle, scen, nodes, exact=True)
    assert_identical(got, ref, 'edge pairs')


def test_certificate_edges_rollout(oracle, native):
    """The same pairs over 30 steps (they approach, touch, graze and part)."""
    scen = edge_pairs(seed=23)
    nodes = N.NODE_ALL & ~N.NODE_FLUCTUATION
    b, agents, _ = batch_from_scenarios([scen])
    b.set_variant(10)
    ref = scen.agents.copy()
    grid = oracle_grid(oracle, scen)
    with oracle.exact_math():
        for _ in range(30):
            b.step(nodes)
            oracle.step(ref, grid, scen.walls, flags=orc_flags(nodes), dt_min=scen.dt_min,
                        dt_max=scen.dt_max)
    got = agents.copy()
    b.download(got)
    b.close()
    assert_identical(got, ref, 'edge pairs rollout')


def crowded(seed, speed=1.0):
    """A dense ThreeCircle field (2.5 agents/m^2) with positions jittered
    into overlaps (contacts) and random velocities."""
    from crowddynamics_gb300.simulation.agents import shoulders
    scen = S.large_field(n=4000, size=40.0, n_walls=10, seed=seed)
    rng = np.random.default_rng(seed)
    a = scen.agents
    a['position'] += rng.normal(0.0, 0.25, (len(a), 2))
    a['velocity'] = rng.normal(0.0, speed, (len(a), 2))
    shoulders(a)
    return scen


@pytest.mark.parametrize('variant', [10, 13])
@pytest.mark.parametrize('case', [('room', 1, 0.1), ('room', 2, 1.0), ('room', 3, 3.0),
                                  ('crowded', 4, 0.3), ('crowded', 5, 1.0), ('crowded', 6, 2.5)])
def test_pair_pipeline_random_sweep(oracle, native, case, variant):
    """Random states for the pair pipeline's float32 decisions: moving rooms at
    several speed scales and dense, overlapping fields (contacts: the force
    pass's jobs with contact apart from the others); three steps bit for bit,
    with the forces in the pair kernel and in the separate force pass."""
    kind, seed, speed = case
    if kind == 'room':
        scen = S.room(n=1500, size=25.0, seed=seed)
        scen.agents['velocity'] = np.random.default_rng(seed).normal(0.0, speed,
                                                                      (len(scen.agents), 2))
    else:
        scen = crowded(seed, speed)
    nodes = N.NODE_ALL & ~N.NODE_FLUCTUATION
    b, agents, _ = batch_from_scenarios([scen])
    b.set_variant(variant)
    b.run(3, nodes)
    got = agents.copy()
    b.download(got)
    counts = b.pair_counts()
    b.close()
    ref = scen.agents.copy()
    grid = oracle_grid(oracle, scen)
    with oracle.exact_math():
        for _ in range(3):
            oracle.step(ref, grid, scen.walls, flags=orc_flags(nodes), dt_min=scen.dt_min,
                        dt_max=scen.dt_max)
    assert_identical(got, ref, '%s seed %d' % (kind, seed))
    if kind == 'crowded':
        assert counts[:, 3].sum() > 0                  # contacts occur


def test_large_field_forces(oracle, native):
    """Full-size 100k ThreeCircle step: agent-agent + walls + adjusting vs the
    oracle's agent-parallel restatement."""
    scen = S.large_field()
    nodes = N.NODE_ORIENTATION | N.NODE_ADJUSTING | N.NODE_AGENT_AGENT | N.NODE_AGENT_OBSTACLE
    got, _ = device_step(scen, nodes)
    assert_identical(got, oracle_step(oracle, scen, nodes, nthreads=16, exact=True)[0], 'exact')
    ref, _ = oracle_step(oracle, scen, nodes, nthreads=16)
    assert_vec_close(got['force'], ref['force'], RTOL, ATOL, 'force')
    assert_vec_close(got['torque'], ref['torque'], RTOL, ATOL, 'torque')


@pytest.mark.parametrize('speed', [0.0, 1.0, 3.0])
def test_pair_split(oracle, native, speed):
    """The flat pair list's split after a ThreeCircle pair-pipeline step: the
    first part and the pairs the float32 pass deferred are within the list
    (with all agents at rest no pair is guessed, and every interacting pair
    has zero relative speed, which the float32 pass defers), and the step
    matches the oracle bit for bit."""
    scen = crowded(21, speed)
    b, agents, _ = batch_from_scenarios([scen])
    b.set_variant(10)
    nodes = N.NODE_ALL & ~N.NODE_FLUCTUATION
    b.step(nodes)
    sp = b.pair_split()
    got = agents.copy()
    b.download(got)
    b.close()
    assert sp['pairs'] > 0
    assert 0 <= sp['first_part'] <= sp['pairs']
    assert 0 <= sp['deferred'] <= sp['pairs'] - sp['first_part']
    if speed == 0.0:
        assert sp['first_part'] == 0 and sp['deferred'] > 0
    assert_identical(got, oracle_step(oracle, scen, nodes, exact=True)[0], 'split')


def test_deterministic(native):
    scen = S.room()
    outs = []
    for _ in range(2):
        b, agents, _ = batch_from_scenarios([scen])
        b.run(20)
        o = agents.copy()
        b.download(o)
        b.close()
        outs.append(o)
    assert outs[0].tobytes() == outs[1].tobytes()


def test_graph_run_matches_steps(native):
    scen = S.hallway()
    b1, a1, _ = batch_from_scenarios([scen])
    b2, a2, _ = batch_from_scenarios([scen])
    nodes = N.NODE_ALL & ~N.NODE_FLUCTUATION
    b1.run(10, nodes)
    for _ in range(10):
        b2.step(nodes)
    o1, o2 = a1.copy(), a2.copy()
    b1.download(o1)
    b2.download(o2)
    assert o1.tobytes() == o2.tobytes()
    assert np.array_equal(b1.time()[1], b2.time()[1])
    b1.close()
    b2.close()


def test_non_finite_position_raises(native):
    from crowddynamics_gb300.exceptions import InvalidValue
    scen = S.hallway()
    scen.agents['position'][3] = (np.nan, 1.0)
    b, agents, _ = batch_from_scenarios([scen])
    with pytest.raises(InvalidValue):
        b.step(N.NODE_AGENT_AGENT, want_dt=True)
    b.close()


def circular_edge_pairs(seed=31, n_pairs=1500, center=(0.0, 0.0)):
    """Isolated Circular pairs from the float32 certificates' edge population
    (tests/test_cpu_certificates.py): skin distances at 3 and 0, grazing,
    roots near 0 and near the 30 s cut-off, parallel and tiny relative
    speeds; each pair 15 m from the next."""
    from crowddynamics_gb300.simulation.agents import new_agents
    from test_cpu_certificates import circ_edge_population
    x, v, r, p, q = circ_edge_population(n_pairs, seed)
    side = int(np.ceil(np.sqrt(n_pairs)))
    spacing = 15.0
    k = np.arange(n_pairs)
    slot = np.stack((10.0 + spacing * (k % side), 10.0 + spacing * (k // side)), 1) + \
        np.asarray(center)
    x = x - np.repeat(x[p], 2, axis=0) + np.repeat(slot, 2, axis=0)
    a = new_agents(2 * n_pairs, 'circular')
    S._circular_bodies(a, np.random.default_rng(seed), 2 * n_pairs)
    a['radius'] = r
    a['position'] = x
    a['velocity'] = v
    rows = int(np.ceil(n_pairs / side))
    bounds = (center[0], center[1], center[0] + 20.0 + spacing * side,
              center[1] + 20.0 + spacing * rows)
    return S.Scenario('circular_edge_pairs', a, S.walls_array([]), bounds, 3.7)


@pytest.mark.parametrize('variant', [9, 10, 11, 12, 14])
@pytest.mark.parametrize('where', ['origin', 'utm'])
def test_circular_certificate_edges(oracle, native, variant, where):
    """circ_pair_light's certificates at their edges, near the origin and at
    (5e5, 7e6) m: one full step of the pair pipeline bit for bit."""
    scen = circular_edge_pairs(center=(0.0, 0.0) if where == 'origin' else (5e5, 7e6))
    nodes = N.NODE_ALL & ~N.NODE_FLUCTUATION
    got, _ = device_step(scen, nodes, variant=variant)
    ref, _ = oracle_step(oracle, scen, nodes, exact=True)
    assert_identical(got, ref, 'circular edge pairs')


@pytest.mark.parametrize('case', ['ties', 'spread', 'tiny', 'huge'])
def test_timestep_speed_maximum(oracle, native, case):
    """The per-scenario maximum speed behind the adaptive timestep
    (core/integrator.py:29-97): k_prepare evaluates hypot only where it can
    hold a block's maximum.  Speeds equal up to their last bits in every
    direction, a wide spread, squares that underflow and squares that
    overflow: the timestep equals the oracle's bit for bit."""
    scen = S.hallway(n=3000, width=60.0, height=40.0, seed=12)
    n = len(scen.agents)
    rng = np.random.default_rng(13)
    th = rng.uniform(0, 2 * np.pi, n)
    mag = {'ties': np.full(n, 5.0), 'spread': rng.uniform(0.0, 12.0, n),
           'tiny': 10.0 ** rng.uniform(-170, -150, n), 'huge': 10.0 ** rng.uniform(150, 156, n)}[case]
    scen.agents['velocity'] = np.stack((mag * np.cos(th), mag * np.sin(th)), 1)
    dts = []
    for variant in (7, 10):
        b, agents, _ = batch_from_scenarios([scen])
        b.set_variant(variant)
        dts.append(b.step(N.NODE_INTEGRATE, want_dt=True)[0])
        b.close()
    want = oracle.adaptive_timestep(scen.agents.copy(), scen.dt_min, scen.dt_max)
    assert dts[0] == want and dts[1] == want, (dts, want)
