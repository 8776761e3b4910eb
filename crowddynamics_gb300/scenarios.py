"""Seeded synthetic scenarios for the per-step agent update.

The reference ships no datasets; these generators build the workloads the
device path is measured and checked on, from a seed:

* ``hallway``      - bidirectional Circular hallway bounded by two walls
                     (40 x 10 m, N=400; also 80 x 20 m, N=5000).
* ``room``         - ThreeCircle square room with one exit and a target
                     direction map toward the exit on a 0.05 m grid.
* ``large_field``  - 300 x 300 m free space with random wall segments and
                     N=100,000 ThreeCircle agents at ~1.1 agents/m^2, target
                     directions from a smooth random unit-vector field.
* ``batch_mix``    - many independent scenarios of uneven size and type.

Placement is setup, not the hot path: small scenarios use seeded rejection
sampling without overlap (as ``Agents.add_non_overlapping_group`` does,
``crowddynamics/simulation/agents.py:633-680``); the large ones use a seeded
jittered lattice whose jitter keeps agents apart.  The fluctuation noise of
``core/motion/fluctuation.py:14-62`` is drawn on the host from the seed by
``draw_noise`` so that the device path and the oracle see the same input.
"""
import math
from dataclasses import dataclass, field

import numpy as np

from crowddynamics_gb300.core.structures import obstacle_type_linear
from crowddynamics_gb300.simulation.agents import new_agents, shoulders, max_extent

SIGHT_SOC = 3.0


@dataclass
class Scenario:
    """One workload: agent array, walls, cell grid and integrator bounds."""
    name: str
    agents: np.ndarray
    walls: np.ndarray
    bounds: tuple            # (xmin, ymin, xmax, ymax) of the cell grid
    cell_size: float
    dt_min: float = 0.001
    dt_max: float = 0.01
    steps: int = 100
    seed: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def grid(self):
        """(x0, y0, cell, nx, ny) of the uniform cell grid over ``bounds``."""
        return grid_for(self.bounds, self.cell_size)

    @property
    def body(self):
        return 'three_circle' if 'position_ls' in self.agents.dtype.fields else 'circular'


def grid_for(bounds, cell_size):
    xmin, ymin, xmax, ymax = bounds
    nx = max(1, int(math.ceil((xmax - xmin) / cell_size)))
    ny = max(1, int(math.ceil((ymax - ymin) / cell_size)))
    return float(xmin), float(ymin), float(cell_size), nx, ny


def truncated_normal(rng, mean, std, lo, hi, size):
    """Normal(mean, std) restricted to [lo, hi] by redrawing."""
    out = rng.normal(mean, std, size)
    bad = (out < lo) | (out > hi)
    while np.any(bad):
        out[bad] = rng.normal(mean, std, int(bad.sum()))
        bad = (out < lo) | (out > hi)
    return out


def walls_array(segments):
    w = np.zeros(len(segments), dtype=obstacle_type_linear)
    for k, (p0, p1) in enumerate(segments):
        w[k]['p0'] = p0
        w[k]['p1'] = p1
    return w


def point_segment_distance(px, py, w):
    """Distance from points (px, py) to every segment of ``w``; shape (P, W)."""
    if len(w) == 0:
        return np.full((len(px), 0), np.inf)
    p0 = w['p0'][None, :, :]
    d = (w['p1'] - w['p0'])[None, :, :]
    q = np.stack((px, py), -1)[:, None, :] - p0
    dd = np.maximum((d * d).sum(-1), 1e-300)
    t = np.clip((q * d).sum(-1) / dd, 0.0, 1.0)
    r = q - t[..., None] * d
    return np.hypot(r[..., 0], r[..., 1])


def place_rejection(rng, n, bounds, extents, walls, margin=0.01, max_tries=None):
    """Seeded rejection sampling of ``n`` non-overlapping discs of radius
    ``extents`` inside ``bounds``, clear of ``walls``.  Returns (n, 2)."""
    xmin, ymin, xmax, ymax = bounds
    rmax = float(np.max(extents)) if n else 0.0
    cs = max(2 * rmax + margin, 1e-3)
    grid = {}
    pos = np.zeros((n, 2))
    tries = 0
    max_tries = max_tries or 200 * max(n, 1)
    k = 0
    while k < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError('placement failed: domain too dense')
        r = extents[k]
        p = rng.uniform((xmin + r, ymin + r), (xmax - r, ymax - r))
        if len(walls) and point_segment_distance(p[None, 0], p[None, 1],
                                                 walls).min() <= r + margin:
            continue
        cx, cy = int(p[0] // cs), int(p[1] // cs)
        ok = True
        for gx in (cx - 1, cx, cx + 1):
            for gy in (cy - 1, cy, cy + 1):
                for j in grid.get((gx, gy), ()):
                    if math.hypot(*(pos[j] - p)) <= r + extents[j] + margin:
                        ok = False
                        break
                if not ok:
                    break
            if not ok:
                break
        if not ok:
            continue
        pos[k] = p
        grid.setdefault((cx, cy), []).append(k)
        k += 1
    return pos


def place_lattice(rng, n, bounds, extent_max, walls, density, margin=0.01):
    """Seeded jittered square lattice: sites at spacing ~1/sqrt(density*1.06),
    each jittered by at most half of (spacing - 2*extent_max), sites closer
    than extent_max + margin to a wall dropped, then ``n`` sites chosen at
    random.  If walls leave too few sites the spacing shrinks by 5% steps.
    Returns (n, 2)."""
    xmin, ymin, xmax, ymax = bounds
    factor = 1.06
    for _ in range(40):
        s = 1.0 / math.sqrt(density * factor)
        xs = np.arange(xmin + s / 2, xmax - extent_max, s)
        ys = np.arange(ymin + s / 2, ymax - extent_max, s)
        gx, gy = np.meshgrid(xs, ys, indexing='ij')
        sites = np.stack((gx.ravel(), gy.ravel()), -1)
        jit = max(0.0, (s - 2 * extent_max - margin) / 2)
        sites = sites + rng.uniform(-jit, jit, sites.shape)
        keep = np.ones(len(sites), bool)
        if len(walls):
            for k0 in range(0, len(sites), 20000):
                d = point_segment_distance(sites[k0:k0 + 20000, 0], sites[k0:k0 + 20000, 1], walls)
                keep[k0:k0 + 20000] = d.min(axis=1) > extent_max + margin
        sites = sites[keep]
        if len(sites) >= n:
            idx = rng.choice(len(sites), n, replace=False)
            return sites[np.sort(idx)]
        factor *= 1.1025
    raise RuntimeError('lattice has %d free sites, need %d' % (len(sites), n))


def draw_noise(agents, rng):
    """Fluctuation force and torque for one step, drawn on the host
    (core/motion/fluctuation.py:14-62 with core/rand.py:8-32):
    force = mass * truncnorm[0, 3](scale=std_rand_force) * (cos phi, sin phi),
    phi ~ U(0, 2 pi); torque = inertia_rot * truncnorm[-3, 3](scale=std_rand_torque).
    Returns (force (N, 2), torque (N,) or None)."""
    from scipy.stats import truncnorm
    n = len(agents)
    phi = rng.uniform(0.0, 2.0 * np.pi, size=n)
    unit = np.array((np.cos(phi), np.sin(phi)))
    mag = truncnorm.rvs(0.0, 3.0, loc=0.0, scale=agents['std_rand_force'], size=n,
                        random_state=rng) if n else np.zeros(0)
    force = np.ascontiguousarray((agents['mass'] * mag * unit).T)
    torque = None
    if 'torque' in agents.dtype.fields:
        torque = agents['inertia_rot'] * truncnorm.rvs(
            -3.0, 3.0, loc=0.0, scale=agents['std_rand_torque'], size=n,
            random_state=rng) if n else np.zeros(0)
    return force, torque


def _circular_bodies(agents, rng, n):
    agents['radius'] = truncated_normal(rng, 0.27, 0.02, 0.2, 0.35, n)
    agents['mass'] = truncated_normal(rng, 80.0, 8.0, 40.0, 120.0, n)
    agents['target_velocity'] = truncated_normal(rng, 1.15, 0.15, 0.5, 1.8, n)


def _three_circle_bodies(agents, rng, n):
    agents['r_t'] = truncated_normal(rng, 0.16, 0.01, 0.13, 0.19, n)
    agents['r_s'] = truncated_normal(rng, 0.10, 0.01, 0.07, 0.13, n)
    agents['r_ts'] = truncated_normal(rng, 0.10, 0.01, 0.07, 0.13, n)
    agents['radius'] = np.maximum(agents['r_t'], agents['r_ts'] + agents['r_s'])
    agents['mass'] = truncated_normal(rng, 80.0, 8.0, 40.0, 120.0, n)
    agents['inertia_rot'] = 4.0
    agents['target_velocity'] = truncated_normal(rng, 1.15, 0.15, 0.5, 1.8, n)
    agents['target_angular_velocity'] = 4.0 * np.pi
    agents['tau_rot'] = 0.2


def hallway(n=400, width=40.0, height=10.0, seed=0, max_agent_radius=0.35,
            steps=100):
    """Bidirectional Circular hallway: walls y=0 and y=height, half the
    agents heading +x and half -x (initial velocity 1 m/s along the target
    direction, as the reference's Hallway attributes set it)."""
    rng = np.random.default_rng(seed)
    a = new_agents(n, 'circular')
    _circular_bodies(a, rng, n)
    walls = walls_array([((0.0, 0.0), (width, 0.0)), ((0.0, height), (width, height))])
    bounds = (0.0, 0.0, width, height)
    if n / (width * height) > 1.2:
        a['position'] = place_lattice(rng, n, bounds, 0.0, walls, n / (width * height))
    else:
        a['position'] = place_rejection(rng, n, bounds, a['radius'], walls)
    e = np.zeros((n, 2))
    e[: n // 2, 0] = 1.0
    e[n // 2:, 0] = -1.0
    a['target_direction'] = e
    a['velocity'] = e
    cell = SIGHT_SOC + 2 * max_agent_radius
    return Scenario('hallway_%dx%d_n%d' % (width, height, n), a, walls, bounds, cell,
                    steps=steps, seed=seed)


def room_exit_direction_map(width, height, exit_y0, exit_y1, step=0.05):
    """Direction map toward an exit on the right wall x=width, y in
    [exit_y0, exit_y1], on a meshgrid with inclusive end points
    (core/steering/quickest_path.py:22-49).  In a convex room without
    interior obstacles the eikonal (fast-marching) solution's gradient is the
    unit vector toward the nearest exit point, which is what this returns.
    Arrays are indexed [j, i] = [y, x] like the reference's maps."""
    x = np.arange(0.0, width + step, step)
    y = np.arange(0.0, height + step, step)
    X, Y = np.meshgrid(x, y, indexing='xy')
    ty = np.clip(Y, exit_y0, exit_y1)
    dx, dy = width - X, ty - Y
    ln = np.hypot(dx, dy)
    ln[ln == 0] = 1.0
    return dx / ln, dy / ln, step


def lookup_direction(positions, dir_map, step, minx=0.0, miny=0.0, defaults=None):
    """Nearest-cell lookup of a direction map (core/steering/navigation.py:69-78
    with the meshgrid indicer of core/steering/quickest_path.py:41-44)."""
    mx, my = dir_map
    idx = ((np.asarray(positions) - np.array((minx, miny))) / step).astype(np.int64)
    i, j = idx[:, 1], idx[:, 0]
    out = np.array(defaults, dtype=np.float64, copy=True) if defaults is not None \
        else np.zeros((len(idx), 2))
    inside = (i >= 0) & (i < mx.shape[0]) & (j >= 0) & (j < mx.shape[1])
    out[inside, 0] = mx[i[inside], j[inside]]
    out[inside, 1] = my[i[inside], j[inside]]
    return out


def room(n=2000, size=30.0, exit_width=1.2, seed=1, steps=500):
    """ThreeCircle square room with one exit on the right wall."""
    from crowddynamics_gb300.simulation.agents import agents_wrap_orientation
    rng = np.random.default_rng(seed)
    a = new_agents(n, 'three_circle')
    _three_circle_bodies(a, rng, n)
    e0, e1 = size / 2 - exit_width / 2, size / 2 + exit_width / 2
    walls = walls_array([
        ((0.0, 0.0), (size, 0.0)), ((0.0, size), (size, size)),
        ((0.0, 0.0), (0.0, size)),
        ((size, 0.0), (size, e0)), ((size, e1), (size, size))])
    bounds = (0.0, 0.0, size, size)
    ext = np.maximum(a['r_t'], a['r_ts'] + a['r_s'])
    a['position'] = place_rejection(rng, n, bounds, ext, walls)
    a['orientation'] = agents_wrap_orientation(rng.uniform(0.0, 2 * np.pi, n))
    mx, my, step = room_exit_direction_map(size, size, e0, e1)
    a['target_direction'] = lookup_direction(a['position'], (mx, my), step)
    a['target_orientation'] = np.arctan2(a['target_direction'][:, 1], a['target_direction'][:, 0])
    a['velocity'] = 0.0
    shoulders(a)
    cell = SIGHT_SOC + 2 * max(0.3, max_extent(a))
    return Scenario('room_%d_n%d' % (size, n), a, walls, bounds, cell, steps=steps,
                    seed=seed, extra={'direction_map': (mx, my), 'map_step': step})


def segment_distance(a0, a1, b0, b1):
    """Distance between segments a0-a1 and b0-b1 (zero if they cross)."""
    def cross(u, v):
        return u[0] * v[1] - u[1] * v[0]
    d1, d2 = a1 - a0, b1 - b0
    den = cross(d1, d2)
    if den != 0.0:
        t = cross(b0 - a0, d2) / den
        u = cross(b0 - a0, d1) / den
        if 0 <= t <= 1 and 0 <= u <= 1:
            return 0.0

    def pt(p, s0, s1):
        d = s1 - s0
        dd = float(d @ d)
        t = 0.0 if dd == 0 else min(1.0, max(0.0, float((p - s0) @ d) / dd))
        return float(np.hypot(*(p - (s0 + t * d))))
    return min(pt(a0, b0, b1), pt(a1, b0, b1), pt(b0, a0, a1), pt(b1, a0, a1))


def _seg_dist_many(a0, a1, B0, B1):
    """Distance from segment a0-a1 to each segment B0[k]-B1[k] (zero when
    they cross); vectorised over k."""
    def cross(u, v):
        return u[..., 0] * v[..., 1] - u[..., 1] * v[..., 0]

    def pt_seg(p, s0, s1):
        d = s1 - s0
        dd = (d * d).sum(-1)
        t = np.where(dd > 0, ((p - s0) * d).sum(-1) / np.where(dd > 0, dd, 1.0), 0.0)
        t = np.clip(t, 0.0, 1.0)
        r = p - (s0 + t[..., None] * d)
        return np.hypot(r[..., 0], r[..., 1])
    d1 = a1 - a0
    d2 = B1 - B0
    den = cross(np.broadcast_to(d1, d2.shape), d2)
    w = B0 - a0
    with np.errstate(divide='ignore', invalid='ignore'):
        t = cross(w, d2) / den
        u = cross(w, np.broadcast_to(d1, d2.shape)) / den
    crossing = (den != 0) & (t >= 0) & (t <= 1) & (u >= 0) & (u <= 1)
    dist = np.minimum(np.minimum(pt_seg(a0, B0, B1), pt_seg(a1, B0, B1)),
                      np.minimum(pt_seg(B0, a0, a1), pt_seg(B1, a0, a1)))
    return np.where(crossing, 0.0, dist)


def random_walls(rng, count, bounds, length=(1.0, 15.0), min_gap=1.0):
    """``count`` random segments inside ``bounds`` with lengths U(length),
    uniform orientation, and no two segments within ``min_gap``."""
    xmin, ymin, xmax, ymax = bounds
    P0 = np.zeros((count, 2))
    P1 = np.zeros((count, 2))
    k = 0
    tries = 0
    while k < count:
        tries += 1
        if tries > 10000 * max(count, 1):
            raise RuntimeError('could not place walls')
        L = rng.uniform(*length)
        th = rng.uniform(0.0, np.pi)
        c = rng.uniform((xmin, ymin), (xmax, ymax))
        d = 0.5 * L * np.array((np.cos(th), np.sin(th)))
        p0, p1 = c - d, c + d
        if min(p0[0], p1[0]) < xmin or max(p0[0], p1[0]) > xmax or \
           min(p0[1], p1[1]) < ymin or max(p0[1], p1[1]) > ymax:
            continue
        if k and _seg_dist_many(p0, p1, P0[:k], P1[:k]).min() < min_gap:
            continue
        P0[k], P1[k] = p0, p1
        k += 1
    return walls_array([(tuple(a), tuple(b)) for a, b in zip(P0, P1)])


def smooth_unit_field(rng, size, step=1.0, modes=6):
    """Seeded smooth random unit-vector field on a grid of ``step`` over
    [0, size]^2: angle = sum of random low-frequency sinusoids."""
    x = np.arange(0.0, size + step, step)
    X, Y = np.meshgrid(x, x, indexing='xy')
    th = np.zeros_like(X)
    for _ in range(modes):
        k = rng.uniform(0.005, 0.03, 2) * 2 * np.pi
        th += rng.uniform(0.5, 1.5) * np.sin(k[0] * X + k[1] * Y + rng.uniform(0, 2 * np.pi))
    th += rng.uniform(0, 2 * np.pi)
    return np.cos(th), np.sin(th), step


def large_field(n=100_000, size=300.0, n_walls=600, seed=2, steps=200,
                cell_size=3.6):
    """300 x 300 m field, 600 random walls, ThreeCircle agents at about
    n / size^2 agents per m^2 (1.1 for the defaults), smooth target field."""
    from crowddynamics_gb300.simulation.agents import agents_wrap_orientation
    rng = np.random.default_rng(seed)
    bounds = (0.0, 0.0, size, size)
    walls = random_walls(rng, n_walls, bounds)
    a = new_agents(n, 'three_circle')
    _three_circle_bodies(a, rng, n)
    ext = float(np.max(np.maximum(a['r_t'], a['r_ts'] + a['r_s'])))
    a['position'] = place_lattice(rng, n, bounds, ext, walls, n / size ** 2)
    a['orientation'] = agents_wrap_orientation(rng.uniform(0.0, 2 * np.pi, n))
    fx, fy, step = smooth_unit_field(rng, size)
    a['target_direction'] = lookup_direction(a['position'], (fx, fy), step)
    a['target_orientation'] = np.arctan2(a['target_direction'][:, 1], a['target_direction'][:, 0])
    a['velocity'] = a['target_direction'] * a['target_velocity'][:, None] * 0.5
    shoulders(a)
    return Scenario('field_%d_n%d_w%d' % (size, n, n_walls), a, walls, bounds, cell_size,
                    steps=steps, seed=seed, extra={'direction_map': (fx, fy), 'map_step': step})


def batch_mix(n_scenarios=512, seed=3, n_min=100, n_max=20000, steps=200):
    """Independent scenarios of uneven size and type: agent count
    log-uniform in [n_min, n_max], Circular or ThreeCircle at random, a
    square room sized for a density uniform in [0.5, 2.5] agents/m^2, 0-200
    random wall segments (fewer in small rooms), and per-scenario tau_0 ~
    U(2, 4) s and k_soc ~ U(1, 2) written into every agent's fields.
    Returns a list of Scenario."""
    from crowddynamics_gb300.simulation.agents import agents_wrap_orientation
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_scenarios):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        body = 'circular' if rng.uniform() < 0.5 else 'three_circle'
        density = rng.uniform(0.5, 2.5)
        size = math.sqrt(n / density)
        n_walls = int(rng.integers(0, 201))
        n_walls = min(n_walls, int(size * size / 40))
        bounds = (0.0, 0.0, size, size)
        walls = random_walls(rng, n_walls, bounds, length=(1.0, min(15.0, size / 3)),
                             min_gap=1.0) if n_walls else walls_array([])
        a = new_agents(n, body)
        if body == 'circular':
            _circular_bodies(a, rng, n)
            ext = float(np.max(a['radius']))
        else:
            _three_circle_bodies(a, rng, n)
            ext = float(np.max(np.maximum(a['r_t'], a['r_ts'] + a['r_s'])))
        # dense rooms leave less clearance than 2 * extent between lattice
        # sites; placement then packs agents tighter than their extent
        a['position'] = place_lattice(rng, n, bounds, min(ext, 0.5 / math.sqrt(density * 1.06)),
                                      walls, density)
        fx, fy, fstep = smooth_unit_field(rng, size, step=1.0, modes=3)
        a['target_direction'] = lookup_direction(a['position'], (fx, fy), fstep)
        a['velocity'] = a['target_direction'] * (0.5 * a['target_velocity'])[:, None]
        a['tau_0'] = rng.uniform(2.0, 4.0)
        a['k_soc'] = rng.uniform(1.0, 2.0)
        if body == 'three_circle':
            a['orientation'] = agents_wrap_orientation(rng.uniform(0.0, 2 * np.pi, n))
            a['target_orientation'] = np.arctan2(a['target_direction'][:, 1],
                                                 a['target_direction'][:, 0])
            shoulders(a)
        cell = SIGHT_SOC + 2 * max(0.35, ext)
        out.append(Scenario('mix%03d_%s_n%d' % (k, body, n), a, walls, bounds, cell, steps=steps,
                            seed=seed, extra={'density': density}))
    return out
