"""The float32 certificates of the ThreeCircle pair pass, checked on the CPU.

`tc_pair_light` (csrc/cd_kernels.cu) decides a pair in float32 alone where
its certificates allow: "no interaction" (skin distance >= 3 m) or "an
interaction without a force" (no contact and no positive time to
collision); every other pair is deferred to float64.  This test restates,
operation by operation in numpy float32 (IEEE rounding per operation, no
fused multiply-add, as the kernel is compiled), the pre-check records the
cell list writes (`k_gather`) and the pass's decisions, and checks them
against the reference's float64 classification (skin distance, contact and
the time-to-collision selection of core/motion/power_law.py:213-363,
restated below) on two million seeded pairs placed at the certificates'
edges: minimum skin distances within 1e-9 .. 1e-2 m of 3 and of 0, head-on,
receding, grazing (discriminants near 0), parallel and nearly parallel
motion, positions far from the origin.  A decided pair must never disagree
with the reference.  The population is sharp enough to matter: with every
margin of the certificates set to zero it yields about 25,000 wrong
decisions in 500,000 pairs.

The pre-check records hold positions relative to the scenario's grid origin,
with every extent raised by 2^-21 of the position's magnitude
(csrc/cd_cull.cuh); walls likewise, with 2^-20 of their endpoints'
magnitudes.  The same checks run on crowds at UTM-like coordinates
(5e5, 7e6) m, with the grid origin beside the crowd and with it at (0, 0)
(relative coordinates near the 1e7 m bound the step enforces), and the cull
of the earlier absolute records without the slack is shown to drop
interacting pairs and wall contacts there.
"""
import numpy as np

from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.simulation.agents import new_agents, shoulders

F = np.float32
SIGHT = F(3.0)
PRESEL_MARGIN = F(1e-4)
CULL_MARGIN = F(0.01)
CULL_MAG = F(2.0 ** -21)
WALL_MAG = F(2.0 ** -20)
NONE, ZERO, DEFER = 0, 1, 3
UTM = (5e5, 7e6)


def cull_slack(xh, yh):
    """cull_slack (csrc/cd_cull.cuh)."""
    m = np.abs(xh) + np.abs(yh)
    return np.where(m <= F(3.0e38), m * CULL_MAG, F(0.0)).astype(F)


def precheck_records(a, origin=(0.0, 0.0), relative=True):
    """k_gather's float32 records: hi and lo parts of the torso position
    relative to the grid origin, shoulder offsets from the torso, radii, and
    the extent bound raised by the position's slack.  relative=False gives
    the earlier records (absolute positions, no slack)."""
    x, y = a['position'][:, 0], a['position'][:, 1]
    if relative:
        xr, yr = x - origin[0], y - origin[1]
    else:
        xr, yr = x, y
    xh, yh = xr.astype(F), yr.astype(F)
    rec = dict(xh=xh, yh=yh,
               xl=(xr - xh.astype(np.float64)).astype(F), yl=(yr - yh.astype(np.float64)).astype(F),
               rt=a['r_t'].astype(F), rs=a['r_s'].astype(F),
               oxl=(a['position_ls'][:, 0] - x).astype(F), oyl=(a['position_ls'][:, 1] - y).astype(F),
               oxr=(a['position_rs'][:, 0] - x).astype(F), oyr=(a['position_rs'][:, 1] - y).astype(F))
    el = np.sqrt(rec['oxl'] * rec['oxl'] + rec['oyl'] * rec['oyl']) + rec['rs']
    er = np.sqrt(rec['oxr'] * rec['oxr'] + rec['oyr'] * rec['oyr']) + rec['rs']
    ef = np.fmax(rec['rt'], np.fmax(el, er))
    rec['ext'] = (ef + ef * F(1e-5)) + F(1e-5)
    if relative:
        rec['ext'] = rec['ext'] + cull_slack(xh, yh)
    return rec


def light_decisions(a, p, q, origin=(0.0, 0.0)):
    """tc_pair_light for the pairs (p[k], q[k])."""
    R = precheck_records(a, origin)
    g = lambda name, idx: R[name][idx]
    dxt = (g('xh', p) - g('xh', q)) + (g('xl', p) - g('xl', q))
    dyt = (g('yh', p) - g('yh', q)) + (g('yl', p) - g('yl', q))
    zero = np.zeros_like(dxt)
    mox = [zero, g('oxl', p), g('oxr', p)]
    moy = [zero, g('oyl', p), g('oyr', p)]
    oox = [zero, g('oxl', q), g('oxr', q)]
    ooy = [zero, g('oyl', q), g('oyr', q)]
    mr = [g('rt', p), g('rs', p), g('rs', p)]
    orr = [g('rt', q), g('rs', q), g('rs', q)]
    out = np.full(len(p), -1, int)

    def decide(mask, value):
        sel = mask & (out < 0)
        out[sel] = value

    xe2 = dxt * dxt + dyt * dyt
    xe = np.sqrt(xe2)
    re = g('ext', p) + g('ext', q)
    scale = np.abs(dxt) + np.abs(dyt)
    for t in (np.abs(mox[1]), np.abs(moy[1]), np.abs(mox[2]), np.abs(moy[2]), np.abs(oox[1]),
              np.abs(ooy[1]), np.abs(oox[2]), np.abs(ooy[2]), mr[0], mr[1], orr[0], orr[1]):
        scale = scale + t
    dmarg = PRESEL_MARGIN + F(1e-6) * scale
    h_lo, h_hi = xe - re, xe - (mr[0] + orr[0])
    decide(h_lo - dmarg >= SIGHT, NONE)
    fast = (h_hi + dmarg < SIGHT) & (h_lo - dmarg > F(0))
    # pre-selection (tc_presel)
    hf = []
    hfmin = np.full(len(p), np.inf, F)
    anynan = np.zeros(len(p), bool)
    for i in range(3):
        for j in range(3):
            dx = (dxt + mox[i]) - oox[j]
            dy = (dyt + moy[i]) - ooy[j]
            h = np.sqrt(dx * dx + dy * dy) - (mr[i] + orr[j])
            hf.append(h)
            anynan |= np.isnan(h)
            hfmin = np.fmin(hfmin, h)
    margin = PRESEL_MARGIN + F(1e-6) * scale
    nsel = sum((h <= hfmin + margin).astype(int) for h in hf)
    unique = (nsel == 1) & ~anynan
    far_cert = hfmin - margin >= SIGHT
    near_cert = (hfmin + margin < SIGHT) & (hfmin - margin > F(0))
    decide(~fast & ~(unique & (far_cert | near_cert)), DEFER)
    decide(~fast & ~near_cert, NONE)
    # interacting without contact: the time to collision
    vp, vq = a['velocity'][p], a['velocity'][q]
    vxf, vyf = (vp[:, 0] - vq[:, 0]).astype(F), (vp[:, 1] - vq[:, 1]).astype(F)
    decide(~((np.abs(vxf) > F(1e-20)) | (np.abs(vyf) > F(1e-20))), DEFER)
    af = vxf * vxf + vyf * vyf
    e0s = F(1.0) + np.abs(dxt)
    for t in (np.abs(dyt), np.abs(mox[1]), np.abs(moy[1]), np.abs(mox[2]), np.abs(moy[2]),
              np.abs(oox[1]), np.abs(ooy[1]), np.abs(oox[2]), np.abs(ooy[2])):
        e0s = e0s + t
    e0 = F(1e-6) * e0s
    be = -(dxt * vxf + dyt * vyf)
    ce = xe2 - re * re
    mbe = (F(4.0) * e0) * (np.abs(vxf) + np.abs(vyf)) + \
        F(1e-6) * (np.abs(dxt * vxf) + np.abs(dyt * vyf))
    mce = (F(8.0) * e0) * ((np.abs(dxt) + np.abs(dyt)) + re) + F(1e-6) * (xe2 + re * re)
    bbe = np.abs(be) + mbe
    decide((ce - mce > F(0)) & ((be + mbe <= F(0)) | (bbe * bbe < (F(0.99) * af) * (ce - mce))),
           ZERO)
    for k in range(9):
        i, j = k // 3, k % 3
        dx = (dxt + mox[i]) - oox[j]
        dy = (dyt + moy[i]) - ooy[j]
        rt = mr[i] + orr[j]
        bf = -(dx * vxf + dy * vyf)
        x2 = dx * dx + dy * dy
        cf = x2 - rt * rt
        acf = af * cf
        discf = bf * bf - acf
        m = (F(1e-5) * af) * ((F(1.0) + x2) + rt * rt) + F(1e-6) * (bf * bf + np.abs(acf))
        cand = ~(discf < -m) & (out < 0)            # the first sub-pair that may have a root
        decide(cand & ~(discf > m), DEFER)
        mb = (F(4.0) * e0) * (np.abs(vxf) + np.abs(vyf)) + \
            F(1e-6) * (np.abs(dx * vxf) + np.abs(dy * vyf))
        mc = (F(8.0) * e0) * ((np.abs(dx) + np.abs(dy)) + rt) + F(1e-6) * (x2 + rt * rt)
        bb = (np.abs(bf) + mb) * (np.abs(bf) + mb)
        neg = (bf < -mb) | ((cf < -mc) & ((F(0.99) * af) * (-cf - mc) > F(1e-9) * bb))
        decide(cand & neg, ZERO)
        decide(cand, DEFER)
    decide(np.ones(len(p), bool), ZERO)                 # no sub-pair has a root
    return out


def reference_classes(a, p, q):
    """(interacting, force) per pair in float64 as the reference decides:
    skin distance below 3 m; contact (skin distance below 0) or a positive
    selected time to collision (the first defined root in visiting order,
    replaced only by a smaller positive one)."""
    parts, radii = ('position', 'position_ls', 'position_rs'), ('r_t', 'r_s', 'r_s')
    v = a['velocity'][p] - a['velocity'][q]
    av = v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]
    h = np.full(len(p), np.inf)
    tau = np.full(len(p), np.nan)
    for i in range(3):
        for j in range(3):
            x = a[parts[i]][p] - a[parts[j]][q]
            r = a[radii[i]][p] + a[radii[j]][q]
            h = np.minimum(h, np.sqrt(x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) - r)
            b = -(x[:, 0] * v[:, 0] + x[:, 1] * v[:, 1])
            c = (x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) - r * r
            with np.errstate(invalid='ignore', divide='ignore'):
                d = np.sqrt(b * b - av * c)
                ok = (av != 0) & ~(np.isnan(d) | (d == 0))
                tn = (b - d) / av
            tau = np.where(ok & (np.isnan(tau) | ((0 < tn) & (tn < tau))), tn, tau)
    inter = h < 3.0
    social = (av != 0) & ~(np.isnan(tau) | (tau <= 0))
    return inter, inter & ((h < 0) | social)


PARTS, RADII = ('position', 'position_ls', 'position_rs'), ('r_t', 'r_s', 'r_s')


def min_subpair(a, p, q):
    """Per pair: the minimum float64 skin distance over the sub-pairs and the
    centre difference (q's part minus p's part) of the sub-pair attaining it."""
    h = np.full(len(p), np.inf)
    w = np.zeros((len(p), 2))
    for i in range(3):
        for j in range(3):
            x = a[PARTS[j]][q] - a[PARTS[i]][p]
            hk = np.sqrt(x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) - (a[RADII[i]][p] + a[RADII[j]][q])
            take = hk < h
            h = np.where(take, hk, h)
            w = np.where(take[:, None], x, w)
    return h, w


def move(a, idx, d):
    for part in PARTS:
        a[part][idx] += d


def edge_population(n_pairs, seed, center=(0.0, 0.0)):
    """Pairs (2k, 2k + 1) of ThreeCircle agents at the certificates' edges:
    the exact minimum skin distance set to within 1e-9 .. 1e-2 m of 3 or of
    0 (or anywhere in [-0.4, 3.6]); relative velocities random, head-on,
    receding, grazing the closest sub-pair within 1e-9 .. 1e-3 of its radii
    sum, zero, or tiny; torsos up to 300 m from `center`."""
    rng = np.random.default_rng(seed)
    n = 2 * n_pairs
    a = new_agents(n, 'three_circle')
    S._three_circle_bodies(a, rng, n)
    a['orientation'] = rng.uniform(-np.pi, np.pi, n)
    p, q = np.arange(0, n, 2), np.arange(1, n, 2)
    th = rng.uniform(0, 2 * np.pi, n_pairs)
    u = np.stack((np.cos(th), np.sin(th)), 1)
    origin = np.asarray(center) + rng.uniform(0, 300.0, (n_pairs, 2))
    a['position'][p] = origin
    a['position'][q] = origin + (rng.uniform(-0.4, 3.6, n_pairs) + a['r_t'][p] +
                                 a['r_t'][q])[:, None] * u
    shoulders(a)
    # move q along the closest sub-pair's centre line until the minimum
    # skin distance sits at the edge (a few passes: the closest sub-pair can
    # change)
    kind = rng.integers(0, 3, n_pairs)
    dh = rng.choice([-1.0, 1.0], n_pairs) * 10.0 ** rng.uniform(-9, -2, n_pairs)
    target = np.where(kind == 0, 3.0 + dh, dh)
    edge = kind < 2
    for _ in range(4):
        h, w = min_subpair(a, p, q)
        lw = np.sqrt((w * w).sum(1))
        step = np.where(edge & (lw > 0), (target - h) / np.where(lw > 0, lw, 1.0), 0.0)
        move(a, q, w * step[:, None])
    # relative motion of p against q
    h, w = min_subpair(a, p, q)
    lw = np.sqrt((w * w).sum(1))
    wn = w / np.where(lw > 0, lw, 1.0)[:, None]                # from p's part towards q's
    motion = rng.integers(0, 6, n_pairs)
    speed = rng.uniform(0.2, 2.0, n_pairs)[:, None]
    rel = rng.normal(0, 1.0, (n_pairs, 2))
    rel = np.where((motion == 1)[:, None], speed * wn, rel)    # head-on
    rel = np.where((motion == 2)[:, None], -speed * wn, rel)   # receding
    # grazing: the closest sub-pair's line of approach misses by its radii
    # sum times (1 +- eps), so its discriminant sits near 0
    rsum = lw - h
    s_ang = np.clip(rsum * (1 + rng.choice([-1.0, 1.0], n_pairs) *
                            10.0 ** rng.uniform(-9, -3, n_pairs)) / np.where(lw > 0, lw, 1.0),
                    -1.0, 1.0)
    c_ang = np.sqrt(1 - s_ang * s_ang)
    sign = rng.choice([-1.0, 1.0], n_pairs)
    gx = wn[:, 0] * c_ang - sign * wn[:, 1] * s_ang
    gy = wn[:, 1] * c_ang + sign * wn[:, 0] * s_ang
    rel = np.where((motion == 3)[:, None], speed * np.stack((gx, gy), 1), rel)
    rel = np.where((motion == 4)[:, None], 0.0, rel)          # parallel
    tiny = rng.normal(0, 1.0, (n_pairs, 2)) * (10.0 ** rng.uniform(-12, -3, n_pairs))[:, None]
    rel = np.where((motion == 5)[:, None], tiny, rel)
    base = rng.normal(0, 1.0, (n_pairs, 2))
    a['velocity'][q] = base
    a['velocity'][p] = base + rel
    return a, p, q


def near_list_far(a, p, q, origin=(0.0, 0.0), relative=True):
    """pair_far: the near lists' float32 cull (torso centres' hi parts, the
    raised extent bounds, 1 cm of margin)."""
    R = precheck_records(a, origin, relative)
    dx = R['xh'][p] - R['xh'][q]
    dy = R['yh'][p] - R['yh'][q]
    lim = (R['ext'][p] + R['ext'][q]) + (SIGHT + CULL_MARGIN)
    return dx * dx + dy * dy > lim * lim


def test_near_list_cull_is_sound():
    """A pair the near lists leave out never interacts."""
    for seed in range(2):
        a, p, q = edge_population(500_000, 10 + seed)
        far = near_list_far(a, p, q)
        inter, _ = reference_classes(a, p, q)
        assert not (far & inter).any()
        assert far.any() and (~far).any()


def test_near_list_cull_is_sound_at_utm_coordinates():
    """Crowds at (5e5, 7e6) m: the cull stays sound with the grid origin
    beside the crowd and with it at (0, 0), where the relative coordinates
    reach 7e6 m (near the 1e7 m bound) and only the extent slack keeps the
    float32 rounding (0.25 m per coordinate there) on the safe side: there
    the slack (3.6 m per agent) keeps every pair of this population, which
    costs time, not results.  The earlier absolute records without slack
    drop interacting pairs here."""
    a, p, q = edge_population(300_000, 30, center=UTM)
    inter, _ = reference_classes(a, p, q)
    far = near_list_far(a, p, q, (UTM[0] - 20.0, UTM[1] - 20.0))
    assert not (far & inter).any()
    assert far.sum() > 1000 and (~far).any()
    for origin in ((0.0, 0.0), (-2e6, 9.9e6)):
        far = near_list_far(a, p, q, origin)
        assert not (far & inter).any(), origin
    old = near_list_far(a, p, q, relative=False)
    assert (old & inter).sum() > 1000


def test_float32_pair_certificates_are_sound():
    total = decided = 0
    for seed in range(4):
        a, p, q = edge_population(500_000, seed)
        got = light_decisions(a, p, q)
        assert np.all((got == NONE) | (got == ZERO) | (got == DEFER))
        inter, force = reference_classes(a, p, q)
        wrong_none = (got == NONE) & inter
        wrong_zero = (got == ZERO) & (~inter | force)
        assert not wrong_none.any(), np.flatnonzero(wrong_none)[:5]
        assert not wrong_zero.any(), np.flatnonzero(wrong_zero)[:5]
        total += len(p)
        decided += int(np.sum(got != DEFER))
    # not vacuous: at these edges the certificates still decide about a
    # quarter of the pairs (most pairs of a real crowd are far from every
    # edge: the float32 pass defers 436 of 1.83M on the 100k field)
    assert decided > 0.15 * total, decided / total


def test_float32_pair_certificates_are_sound_at_utm_coordinates():
    """The certificates on hi + lo positions relative to a grid origin beside
    the crowd and 7e6 m away from it."""
    a, p, q = edge_population(300_000, 31, center=UTM)
    inter, force = reference_classes(a, p, q)
    for origin in ((UTM[0] - 20.0, UTM[1] - 20.0), (0.0, 0.0)):
        got = light_decisions(a, p, q, origin)
        assert not ((got == NONE) & inter).any(), origin
        assert not ((got == ZERO) & (~inter | force)).any(), origin
        assert np.sum(got != DEFER) > 0.15 * len(p)


def wall_far(xh, yh, reach, w):
    """wall_far (csrc/cd_cull.cuh) in float32, w = (p0x, p0y, p1x, p1y)."""
    dx, dy = w[:, 2] - w[:, 0], w[:, 3] - w[:, 1]
    qx, qy = xh - w[:, 0], yh - w[:, 1]
    dd = dx * dx + dy * dy
    with np.errstate(invalid='ignore', divide='ignore'):
        t = np.where(dd > F(0), np.fmin(np.fmax((qx * dx + qy * dy) / dd, F(0)), F(1)), F(0))
    rx, ry = qx - t * dx, qy - t * dy
    wm = (np.abs(w[:, 0]) + np.abs(w[:, 1])) + (np.abs(w[:, 2]) + np.abs(w[:, 3]))
    lim = (reach + CULL_MARGIN) + wm * WALL_MAG
    return rx * rx + ry * ry > lim * lim


def wall_population(n, seed, center):
    """ThreeCircle agents and one wall segment each (length 1-15 m, any
    angle, up to 300 m from `center`), the torso centre's distance to the
    segment set within 1e-7 .. 1e-1 m of the agent's extent (either side),
    or anywhere in [0, 4] m; about a third of the closest points are the
    segment's end points."""
    rng = np.random.default_rng(seed)
    a = new_agents(n, 'three_circle')
    S._three_circle_bodies(a, rng, n)
    a['orientation'] = rng.uniform(-np.pi, np.pi, n)
    a['position'] = np.asarray(center) + rng.uniform(0, 300.0, (n, 2))
    shoulders(a)
    x = a['position']
    ext = np.maximum(a['r_t'], np.maximum(
        np.hypot(*(a['position_ls'] - x).T) + a['r_s'],
        np.hypot(*(a['position_rs'] - x).T) + a['r_s']))
    dh = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-7, -1, n)
    dist = np.where(rng.uniform(size=n) < 0.8, ext + dh, rng.uniform(0, 4.0, n))
    th = rng.uniform(0, 2 * np.pi, n)
    t = np.stack((np.cos(th), np.sin(th)), 1)
    nrm = np.stack((-t[:, 1], t[:, 0]), 1)
    length = rng.uniform(1.0, 15.0, n)
    # the closest point: inside the segment, or an end point (then the
    # agent sits beyond that end, along a direction in the end's half-plane)
    along = rng.uniform(0, 1.0, n) * length
    end = rng.integers(0, 3, n)
    ang = rng.uniform(-np.pi / 2, np.pi / 2, n)
    out_dir = np.where((end == 1)[:, None], -t, t)
    off = np.where((end == 0)[:, None], nrm * dist[:, None],
                   (out_dir * np.cos(ang)[:, None] + nrm * np.sin(ang)[:, None]) * dist[:, None])
    foot = np.where((end == 0)[:, None], x - off, x - off)
    start = np.where((end == 1)[:, None], foot,
                     np.where((end == 2)[:, None], foot - t * length[:, None],
                              foot - t * along[:, None]))
    walls = np.concatenate((start, start + t * length[:, None]), 1)
    return a, walls, ext


def segment_distance(x, w):
    """The torso centre's distance to the segment in float64, as
    distance_circle_line (core/distance.py:108-146) computes it with r = 0."""
    p0, p1 = w[:, :2], w[:, 2:]
    d = p1 - p0
    lw = np.hypot(d[:, 0], d[:, 1])
    t = d / lw[:, None]
    q0, q1 = x - p0, x - p1
    l_t = -(t * q1).sum(1) - (t * q0).sum(1)
    nrm = np.stack((-t[:, 1], t[:, 0]), 1)
    perp = np.abs((nrm * q0).sum(1))
    return np.where(l_t > lw, np.hypot(*q0.T), np.where(l_t < -lw, np.hypot(*q1.T), perp))


def test_wall_cull_is_sound():
    """A wall segment the float32 wall cull skips is farther from the torso
    centre than the agent's extent, so the reference finds no contact with
    it; near the origin, at (5e5, 7e6) m with the grid origin beside the crowd
    and at (0, 0).  The earlier absolute records without the magnitude terms
    skip walls in contact there."""
    for center, origins in (((0.0, 0.0), ((0.0, 0.0),)),
                            (UTM, ((UTM[0] - 20.0, UTM[1] - 20.0), (0.0, 0.0)))):
        a, walls, ext = wall_population(300_000, 40, center)
        dist = segment_distance(a['position'], walls)
        touching = dist <= ext
        for k, origin in enumerate(origins):
            o = np.array([origin[0], origin[1], origin[0], origin[1]])
            R = precheck_records(a, origin)
            far = wall_far(R['xh'], R['yh'], R['ext'], (walls - o).astype(F))
            assert not (far & touching).any(), (center, origin)
            if k == 0:                      # the grid origin beside the crowd
                assert far.sum() > 1000 and (~far).any()
    R = precheck_records(a, relative=False)
    wf = walls.astype(F)
    dx, dy = wf[:, 2] - wf[:, 0], wf[:, 3] - wf[:, 1]
    qx, qy = R['xh'] - wf[:, 0], R['yh'] - wf[:, 1]
    t = np.fmin(np.fmax((qx * dx + qy * dy) / (dx * dx + dy * dy), F(0)), F(1))
    rx, ry = qx - t * dx, qy - t * dy
    lim = R['ext'] + CULL_MARGIN
    assert ((rx * rx + ry * ry > lim * lim) & touching).sum() > 1000


def root_certificates(a, p, q):
    """The float32 time-to-collision part of tc_pair_both for the pairs
    (p[k], q[k]): the class of the first sub-pair that may have a root
    (0 float64 decides, 1 certainly negative, 2 certainly positive), the
    sub-pairs queued for float64 roots before and after the pruning of roots
    that cannot be the least positive one (bit k: sub-pair k)."""
    R = precheck_records(a)
    g = lambda name, idx: R[name][idx]
    dxt = (g('xh', p) - g('xh', q)) + (g('xl', p) - g('xl', q))
    dyt = (g('yh', p) - g('yh', q)) + (g('yl', p) - g('yl', q))
    zero = np.zeros_like(dxt)
    mox = [zero, g('oxl', p), g('oxr', p)]
    moy = [zero, g('oyl', p), g('oyr', p)]
    oox = [zero, g('oxl', q), g('oxr', q)]
    ooy = [zero, g('oyl', q), g('oyr', q)]
    mr = [g('rt', p), g('rs', p), g('rs', p)]
    orr = [g('rt', q), g('rs', q), g('rs', q)]
    vp, vq = a['velocity'][p], a['velocity'][q]
    vxf, vyf = (vp[:, 0] - vq[:, 0]).astype(F), (vp[:, 1] - vq[:, 1]).astype(F)
    af = vxf * vxf + vyf * vyf
    e0s = F(1.0) + np.abs(dxt)
    for t in (np.abs(dyt), np.abs(mox[1]), np.abs(moy[1]), np.abs(mox[2]), np.abs(moy[2]),
              np.abs(oox[1]), np.abs(ooy[1]), np.abs(oox[2]), np.abs(ooy[2])):
        e0s = e0s + t
    e0 = F(1e-6) * e0s
    re = g('ext', p) + g('ext', q)
    xe2 = dxt * dxt + dyt * dyt
    be = -(dxt * vxf + dyt * vyf)
    ce = xe2 - re * re
    mbe = (F(4.0) * e0) * (np.abs(vxf) + np.abs(vyf)) + \
        F(1e-6) * (np.abs(dxt * vxf) + np.abs(dyt * vyf))
    mce = (F(8.0) * e0) * ((np.abs(dxt) + np.abs(dyt)) + re) + F(1e-6) * (xe2 + re * re)
    bbe = np.abs(be) + mbe
    apart = (ce - mce > F(0)) & ((be + mbe <= F(0)) | (bbe * bbe < (F(0.99) * af) * (ce - mce)))
    first = np.where(apart, 1, -1)
    cand = np.zeros(len(p), np.int64)
    min_hi = np.full(len(p), np.inf, F)
    terms = []
    for k in range(9):
        i, j = k // 3, k % 3
        dx = (dxt + mox[i]) - oox[j]
        dy = (dyt + moy[i]) - ooy[j]
        rt = mr[i] + orr[j]
        bf = -(dx * vxf + dy * vyf)
        x2 = dx * dx + dy * dy
        cf = x2 - rt * rt
        acf = af * cf
        discf = bf * bf - acf
        m = (F(1e-5) * af) * ((F(1.0) + x2) + rt * rt) + F(1e-6) * (bf * bf + np.abs(acf))
        mb = (F(4.0) * e0) * (np.abs(vxf) + np.abs(vyf)) + \
            F(1e-6) * (np.abs(dx * vxf) + np.abs(dy * vyf))
        mc = (F(8.0) * e0) * ((np.abs(dx) + np.abs(dy)) + rt) + F(1e-6) * (x2 + rt * rt)
        bb = (np.abs(bf) + mb) * (np.abs(bf) + mb)
        terms.append((bf, cf, discf, m, mb, mc, bb))
        c_k = ~apart & ~(discf < -m)
        cand |= np.where(c_k, 1 << k, 0)
        pos = (discf > m) & (bf > mb) & (cf > mc) & ((F(0.99) * af) * (cf - mc) > F(1e-9) * bb)
        neg = (bf < -mb) | ((cf < -mc) & ((F(0.99) * af) * (-cf - mc) > F(1e-9) * bb))
        cls = np.where(discf > m, np.where(neg, 1, np.where(pos, 2, 0)), 0)
        first = np.where(c_k & (first < 0), cls, first)
        with np.errstate(invalid='ignore', divide='ignore'):
            hi = (cf + mc) / ((bf - mb) + np.sqrt(discf - m)) * F(1.00001)
        min_hi = np.where(c_k & pos, np.fmin(min_hi, hi), min_hi)
    queued = np.where(first == 1, 0, cand)
    pruned = queued.copy()
    several = np.array([bin(int(x)).count('1') > 1 for x in queued])
    for k in range(9):
        bf, cf, discf, m, mb, mc, bb = terms[k]
        inq = ((queued >> k) & 1).astype(bool) & (first == 2) & several & (discf > m)
        drop = (bf < -mb) | ((cf < -mc) & ((F(0.99) * af) * (-cf - mc) > F(1e-9) * bb))
        ok = ~drop & (bf > mb) & (cf > mc) & ((F(0.99) * af) * (cf - mc) > F(1e-9) * bb)
        with np.errstate(invalid='ignore', divide='ignore'):
            lo = (cf - mc) / ((bf + mb) + np.sqrt(discf + m)) * F(0.99999)
        drop = drop | (ok & (lo > min_hi))
        pruned = np.where(inq & drop, pruned & ~(1 << k), pruned)
    return first, queued, pruned, vxf, vyf


def reference_roots(a, p, q):
    """Per pair and sub-pair in visiting order: the reference's root (NaN
    where undefined), and the index of the selected one (-1 for none)."""
    v = a['velocity'][p] - a['velocity'][q]
    av = v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]
    roots = np.full((len(p), 9), np.nan)
    tau = np.full(len(p), np.nan)
    sel = np.full(len(p), -1)
    for k in range(9):
        i, j = k // 3, k % 3
        x = a[PARTS[i]][p] - a[PARTS[j]][q]
        r = a[RADII[i]][p] + a[RADII[j]][q]
        b = -(x[:, 0] * v[:, 0] + x[:, 1] * v[:, 1])
        c = (x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) - r * r
        with np.errstate(invalid='ignore', divide='ignore'):
            d = np.sqrt(b * b - av * c)
            ok = (av != 0) & ~(np.isnan(d) | (d == 0))
            tn = (b - d) / av
        roots[:, k] = np.where(ok, tn, np.nan)
        take = ok & (np.isnan(tau) | ((0 < tn) & (tn < tau)))
        tau = np.where(take, tn, tau)
        sel = np.where(take, k, sel)
    return roots, sel, tau


def test_float32_root_certificates_are_sound():
    """tc_pair_both's float32 time-to-collision certificates: every defined
    root is queued unless the first root is certainly negative; a first root
    classed negative or positive has that sign; and the pruning keeps the
    root the reference selects.  With the margins and the 1e-5 bound factors
    removed, 400,000 of these pairs give thousands of misses, wrong signs and
    lost roots."""
    checked = pruned_any = 0
    for seed in range(3):
        a, p, q = edge_population(400_000, 20 + seed)
        inter, _ = reference_classes(a, p, q)
        first, queued, pruned, vxf, vyf = root_certificates(a, p, q)
        roots, sel, tau = reference_roots(a, p, q)
        live = inter & ((np.abs(vxf) > F(1e-20)) | (np.abs(vyf) > F(1e-20)))
        defined = ~np.isnan(roots)
        first_root = np.array([r[np.flatnonzero(~np.isnan(r))[0]] if (~np.isnan(r)).any()
                               else np.nan for r in roots])
        bits = (queued[:, None] >> np.arange(9)) & 1
        # every defined root queued, unless the first one is certainly negative
        missed = live & (first != 1) & (defined & (bits == 0)).any(1)
        assert not missed.any(), np.flatnonzero(missed)[:5]
        neg_wrong = live & (first == 1) & ~(np.isnan(tau) | (tau <= 0))
        assert not neg_wrong.any(), np.flatnonzero(neg_wrong)[:5]
        pos_wrong = live & (first == 2) & ~(first_root > 0)
        assert not pos_wrong.any(), np.flatnonzero(pos_wrong)[:5]
        lost = live & (first == 2) & (sel >= 0) & (((pruned >> np.maximum(sel, 0)) & 1) == 0)
        assert not lost.any(), np.flatnonzero(lost)[:5]
        checked += int(live.sum())
        pruned_any += int((live & (pruned != queued)).sum())
    assert checked > 100_000 and pruned_any > 1000, (checked, pruned_any)


# ---- Circular bodies: circ_pair_light ---------------------------------------

def circ_records(x, r, origin=(0.0, 0.0)):
    """k_gather's Circular pre-check records: position hi (cull) and lo
    (stage_f) relative to the grid origin, the radius as float32."""
    xr, yr = x[:, 0] - origin[0], x[:, 1] - origin[1]
    xh, yh = xr.astype(F), yr.astype(F)
    return dict(xh=xh, yh=yh, xl=(xr - xh.astype(np.float64)).astype(F),
                yl=(yr - yh.astype(np.float64)).astype(F), r=r.astype(F))


def circ_light(x, v, r, p, q, origin=(0.0, 0.0), margins=True):
    """circ_pair_light (csrc/cd_kernels.cu) in numpy float32 for the pairs
    (p[k], q[k]); margins=False drops every margin."""
    R = circ_records(x, r, origin)
    k = F(1.0) if margins else F(0.0)
    dx = (R['xh'][p] - R['xh'][q]) + (R['xl'][p] - R['xl'][q])
    dy = (R['yh'][p] - R['yh'][q]) + (R['yl'][p] - R['yl'][q])
    rt = R['r'][p] + R['r'][q]
    x2 = dx * dx + dy * dy
    h = np.sqrt(x2) - rt
    dmarg = k * (PRESEL_MARGIN + F(1e-6) * ((np.abs(dx) + np.abs(dy)) + rt))
    out = np.full(len(p), -1, int)

    def decide(mask, value):
        out[mask & (out < 0)] = value

    decide(h - dmarg >= SIGHT, NONE)
    decide(~((h + dmarg < SIGHT) & (h - dmarg > F(0))), DEFER)
    vxf = (v[p, 0] - v[q, 0]).astype(F)
    vyf = (v[p, 1] - v[q, 1]).astype(F)
    decide(~((np.abs(vxf) > F(1e-20)) | (np.abs(vyf) > F(1e-20))), DEFER)
    af = vxf * vxf + vyf * vyf
    e0 = F(1e-6) * ((F(1.0) + np.abs(dx)) + np.abs(dy))
    bf = -(dx * vxf + dy * vyf)
    cf = x2 - rt * rt
    acf = af * cf
    discf = bf * bf - acf
    m = k * ((F(1e-5) * af) * ((F(1.0) + x2) + rt * rt) + F(1e-6) * (bf * bf + np.abs(acf)))
    decide(discf < -m, ZERO)
    decide(~(discf > m), DEFER)
    mb = k * ((F(4.0) * e0) * (np.abs(vxf) + np.abs(vyf)) +
              F(1e-6) * (np.abs(dx * vxf) + np.abs(dy * vyf)))
    mc = k * ((F(8.0) * e0) * ((np.abs(dx) + np.abs(dy)) + rt) + F(1e-6) * (x2 + rt * rt))
    decide(bf < -mb, ZERO)
    bb = (np.abs(bf) + mb) * (np.abs(bf) + mb)
    ok = (bf > mb) & (cf > mc) & ((F(0.99) * af) * (cf - mc) > F(1e-9) * bb)
    with np.errstate(invalid='ignore', divide='ignore', over='ignore'):
        lo = (cf - mc) / ((bf + mb) + np.sqrt(discf + m)) * (F(0.99999) if margins else F(1.0))
    decide(ok & (lo > F(30.0) * (F(1.00001) if margins else F(1.0))), ZERO)
    decide(np.ones(len(p), bool), DEFER)
    return out


def circ_reference(x, v, r, p, q):
    """(interacting, force) per pair as pair_circular_both decides in float64
    (core/interactions.py:51-70, core/motion/power_law.py:213-259): h < 3;
    contact, or a time to collision in (0, 30]."""
    xx, xy = x[p, 0] - x[q, 0], x[p, 1] - x[q, 1]
    rt = r[p] + r[q]
    h = np.hypot(xx, xy) - rt
    vx, vy = v[p, 0] - v[q, 0], v[p, 1] - v[q, 1]
    a = vx * vx + vy * vy
    b = -(xx * vx + xy * vy)
    c = (xx * xx + xy * xy) - rt * rt
    disc = b * b - a * c
    with np.errstate(invalid='ignore', divide='ignore'):
        tau = (b - np.sqrt(disc)) / a
    social = (disc > 0) & (a != 0) & (tau > 0) & (tau <= 30.0)
    inter = h < 3.0
    return inter, inter & ((h < 0) | social)


def circ_edge_population(n_pairs, seed, center=(0.0, 0.0)):
    """Circular pairs at the certificates' edges: skin distance within
    1e-9 .. 1e-2 m of 3 or 0 (or anywhere in [-0.3, 3.5]); relative motion
    random, head-on, receding, grazing (discriminant near 0), parallel or
    tiny, or head-on with the time to collision within 1e-7 .. 1e-2 of the
    30 s cut-off (either side); torsos up to 300 m from `center`."""
    rng = np.random.default_rng(seed)
    n = 2 * n_pairs
    r = rng.uniform(0.2, 0.35, n)
    p, q = np.arange(0, n, 2), np.arange(1, n, 2)
    x = np.zeros((n, 2))
    x[p] = np.asarray(center) + rng.uniform(0, 300.0, (n_pairs, 2))
    th = rng.uniform(0, 2 * np.pi, n_pairs)
    u = np.stack((np.cos(th), np.sin(th)), 1)                  # from p towards q
    kind = rng.integers(0, 3, n_pairs)
    dh = rng.choice([-1.0, 1.0], n_pairs) * 10.0 ** rng.uniform(-9, -2, n_pairs)
    h = np.where(kind == 0, 3.0 + dh, np.where(kind == 1, dh, rng.uniform(-0.3, 3.5, n_pairs)))
    rt = r[p] + r[q]
    x[q] = x[p] + ((rt + h)[:, None] * u)
    motion = rng.integers(0, 7, n_pairs)
    speed = rng.uniform(0.05, 2.0, n_pairs)[:, None]
    rel = rng.normal(0, 1.0, (n_pairs, 2))
    rel = np.where((motion == 1)[:, None], speed * u, rel)        # p heads for q
    rel = np.where((motion == 2)[:, None], -speed * u, rel)       # receding
    d = rt + h
    s_ang = np.clip(rt / d * (1 + rng.choice([-1.0, 1.0], n_pairs) *
                              10.0 ** rng.uniform(-9, -3, n_pairs)), -1.0, 1.0)
    c_ang = np.sqrt(1 - s_ang * s_ang)
    sg = rng.choice([-1.0, 1.0], n_pairs)
    g = np.stack((u[:, 0] * c_ang - sg * u[:, 1] * s_ang, u[:, 1] * c_ang + sg * u[:, 0] * s_ang), 1)
    rel = np.where((motion == 3)[:, None], speed * g, rel)        # grazing
    rel = np.where((motion == 4)[:, None], 0.0, rel)
    tiny = rng.normal(0, 1.0, (n_pairs, 2)) * (10.0 ** rng.uniform(-12, -3, n_pairs))[:, None]
    rel = np.where((motion == 5)[:, None], tiny, rel)
    # head-on with tau = (d - rt) / speed near 30 s
    t30 = 30.0 * (1 + rng.choice([-1.0, 1.0], n_pairs) * 10.0 ** rng.uniform(-7, -2, n_pairs))
    sp30 = np.maximum(h, 1e-3) / t30
    rel = np.where((motion == 6)[:, None], sp30[:, None] * u, rel)
    base = rng.normal(0, 1.0, (n_pairs, 2))
    v = np.zeros((n, 2))
    v[q] = base
    v[p] = base + rel
    return x, v, r, p, q


def test_circular_float32_pair_certificates_are_sound():
    """circ_pair_light never disagrees with the reference's float64
    classification, near the origin and at UTM coordinates (grid origin beside
    the crowd and at (0, 0)); without its margins the same population gives
    wrong decisions."""
    total = decided = 0
    for seed, center, origins in ((50, (0.0, 0.0), ((0.0, 0.0),)),
                                  (51, (0.0, 0.0), ((0.0, 0.0),)),
                                  (52, UTM, ((UTM[0] - 20.0, UTM[1] - 20.0), (0.0, 0.0)))):
        x, v, r, p, q = circ_edge_population(400_000, seed, center)
        inter, force = circ_reference(x, v, r, p, q)
        for origin in origins:
            got = circ_light(x, v, r, p, q, origin)
            assert np.all((got == NONE) | (got == ZERO) | (got == DEFER))
            wrong_none = (got == NONE) & inter
            wrong_zero = (got == ZERO) & (~inter | force)
            assert not wrong_none.any(), (origin, np.flatnonzero(wrong_none)[:5])
            assert not wrong_zero.any(), (origin, np.flatnonzero(wrong_zero)[:5])
        total += len(p)
        decided += int(np.sum(got != DEFER))
        if seed == 50:
            bare = circ_light(x, v, r, p, q, margins=False)
            wrong = ((bare == NONE) & inter) | ((bare == ZERO) & (~inter | force))
            assert wrong.sum() > 1000, wrong.sum()
    assert decided > 0.15 * total, decided / total
