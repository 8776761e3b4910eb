"""ctypes front-end of the C oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this module, as the checker / baseline.  The product path never
imports it.  Every function mirrors the reference function named in its
docstring and works in place on a packed agent structured array, exactly as
the reference's numba kernels do.
"""
import ctypes
import os

import numpy as np

from oracle.build import build, LIB

ORC_FLUCTUATION = 1
ORC_ORIENTATION = 2
ORC_ADJUSTING = 4
ORC_AGENT_AGENT = 8
ORC_AGENT_OBSTACLE = 16
ORC_INTEGRATE = 32
ORC_RESET = 64
ORC_FULL = 127
ORC_NAVIGATION = 128

BODY_CIRCULAR = 0
BODY_THREE_CIRCLE = 1

# Field order of the offset table (must match cd_oracle.c's F_* enum).
FIELD_NAMES = (
    'position', 'velocity', 'target_direction', 'force', 'force_prev',
    'radius', 'r_t', 'r_s', 'r_ts', 'mass', 'inertia_rot', 'target_velocity',
    'target_angular_velocity', 'tau_adj', 'k_soc', 'tau_0', 'mu', 'kappa',
    'damping', 'std_rand_force', 'position_ls', 'position_rs', 'orientation',
    'angular_velocity', 'target_orientation', 'torque', 'torque_prev',
    'tau_rot', 'std_rand_torque', 'target',
)


class Grid(ctypes.Structure):
    """Uniform cell grid: origin (x0, y0), square cell size, nx by ny cells;
    flat cell index is ix * ny + iy."""
    _fields_ = [('x0', ctypes.c_double), ('y0', ctypes.c_double),
                ('cell', ctypes.c_double), ('nx', ctypes.c_int64),
                ('ny', ctypes.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        d = ctypes.c_double
        L.orc_agent_agent.argtypes = [P, i64, i64, P, ctypes.c_int, ctypes.POINTER(Grid), ctypes.c_int]
        L.orc_agent_agent.restype = ctypes.c_int
        L.orc_agent_obstacle.argtypes = [P, i64, i64, P, ctypes.c_int, P, i64, ctypes.c_int]
        L.orc_agent_obstacle.restype = None
        for name in ('orc_force_adjust_agents', 'orc_torque_adjust_agents',
                     'orc_orient_towards_target_direction', 'orc_shoulders'):
            getattr(L, name).argtypes = [P, i64, i64, P]
            getattr(L, name).restype = None
        L.orc_reset.argtypes = [P, i64, i64, P, ctypes.c_int]
        L.orc_add_noise.argtypes = [P, i64, i64, P, ctypes.c_int, P, P]
        L.orc_adaptive_timestep.argtypes = [P, i64, i64, P, d, d]
        L.orc_adaptive_timestep.restype = d
        L.orc_velocity_verlet.argtypes = [P, i64, i64, P, ctypes.c_int, d, d]
        L.orc_velocity_verlet.restype = d
        L.orc_step.argtypes = [P, i64, i64, P, ctypes.c_int, ctypes.c_int,
                               ctypes.POINTER(Grid), P, i64, P, P, d, d, ctypes.c_int]
        L.orc_step.restype = d
        L.orc_cell_list.argtypes = [P, P, i64, ctypes.POINTER(Grid), P, P, P, P]
        L.orc_cell_list.restype = i64
        L.orc_candidate_pairs.argtypes = [P, P, i64, ctypes.POINTER(Grid), P, i64]
        L.orc_candidate_pairs.restype = i64
        L.orc_set_exact_math.argtypes = [ctypes.c_int]
        L.orc_set_exact_math.restype = None
        L.orc_cdm.argtypes = [ctypes.c_int, d, d]
        L.orc_cdm.restype = d
        L.orc_wrap_to_pi.argtypes = [d]
        L.orc_wrap_to_pi.restype = d
        L.orc_philox4x32_10.argtypes = [P, P, P]
        L.orc_philox4x32_10.restype = None
        L.orc_device_noise.argtypes = [P, i64, i64, P, ctypes.c_int, ctypes.c_uint64,
                                       ctypes.c_uint64, P, P]
        L.orc_device_noise.restype = None
        L.orc_set_navigation.argtypes = [i64, P, P, i64, i64, d, d, d]
        L.orc_set_navigation.restype = None
        L.orc_navigation.argtypes = [P, i64, i64, P]
        L.orc_navigation.restype = None
        _lib = L
    return _lib


def set_exact_math(on):
    """Use the device's elementary functions (cd_math.h) instead of the C
    library's, for bit-for-bit comparison with the device path."""
    lib().orc_set_exact_math(1 if on else 0)


class exact_math:
    """Context manager enabling set_exact_math for a block."""

    def __enter__(self):
        set_exact_math(True)

    def __exit__(self, *exc):
        set_exact_math(False)


def _offsets(agents):
    off = np.full(len(FIELD_NAMES), -1, dtype=np.int64)
    for k, name in enumerate(FIELD_NAMES):
        if name in agents.dtype.fields:
            off[k] = agents.dtype.fields[name][1]
    return off


def _body(agents):
    return BODY_THREE_CIRCLE if 'position_ls' in agents.dtype.fields else BODY_CIRCULAR


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(agents):
    if not agents.flags.c_contiguous:
        raise ValueError('agent array must be C-contiguous')


def make_grid(x0, y0, cell, nx, ny):
    return Grid(float(x0), float(y0), float(cell), int(nx), int(ny))


def agent_agent_block_list(agents, grid, nthreads=1):
    """core/interactions.py:191-205 over the restated cell list."""
    _check(agents)
    off = _offsets(agents)
    rc = lib().orc_agent_agent(_ptr(agents), len(agents), agents.dtype.itemsize,
                               _ptr(off), _body(agents), ctypes.byref(grid), nthreads)
    if rc != 0:
        raise ValueError('non-finite agent position')


def agent_obstacle(agents, walls, nthreads=1):
    """core/interactions.py:208-214; ``walls`` is an obstacle_type_linear
    array or a (W, 4) float64 array of (p0x, p0y, p1x, p1y)."""
    _check(agents)
    w = np.ascontiguousarray(np.asarray(walls).view(np.float64).reshape(-1, 4)) \
        if len(walls) else np.zeros((0, 4))
    off = _offsets(agents)
    lib().orc_agent_obstacle(_ptr(agents), len(agents), agents.dtype.itemsize,
                             _ptr(off), _body(agents), _ptr(w), len(w), nthreads)


def force_adjust_agents(agents):
    """core/motion/adjusting.py:98-108"""
    off = _offsets(agents)
    lib().orc_force_adjust_agents(_ptr(agents), len(agents), agents.dtype.itemsize, _ptr(off))


def torque_adjust_agents(agents):
    """core/motion/adjusting.py:111-121"""
    off = _offsets(agents)
    lib().orc_torque_adjust_agents(_ptr(agents), len(agents), agents.dtype.itemsize, _ptr(off))


def orient_towards_target_direction(agents):
    """core/steering/orientation.py:17-21"""
    off = _offsets(agents)
    lib().orc_orient_towards_target_direction(_ptr(agents), len(agents),
                                              agents.dtype.itemsize, _ptr(off))


def adaptive_timestep(agents, dt_min, dt_max):
    """core/integrator.py:29-97"""
    off = _offsets(agents)
    return lib().orc_adaptive_timestep(_ptr(agents), len(agents), agents.dtype.itemsize,
                                       _ptr(off), dt_min, dt_max)


def velocity_verlet_integrator(agents, dt_min, dt_max):
    """core/integrator.py:209-256"""
    off = _offsets(agents)
    return lib().orc_velocity_verlet(_ptr(agents), len(agents), agents.dtype.itemsize,
                                     _ptr(off), _body(agents), dt_min, dt_max)


def reset(agents):
    """simulation/logic.py:59-64"""
    off = _offsets(agents)
    lib().orc_reset(_ptr(agents), len(agents), agents.dtype.itemsize, _ptr(off), _body(agents))


def cdm(name, a, b=0.0):
    """One of the shared elementary functions: hypot, exp, sin, cos, atan2."""
    which = ('hypot', 'exp', 'sin', 'cos', 'atan2', 'log').index(name)
    return lib().orc_cdm(which, float(a), float(b))


def wrap_to_pi(x):
    """core/vector2D.py:8-36"""
    return lib().orc_wrap_to_pi(float(x))


def step(agents, grid, walls=None, noise_f=None, noise_m=None, flags=ORC_FULL,
         dt_min=0.001, dt_max=0.01, nthreads=1, nav=None):
    """One MultiAgentSimulation.update() of the standard node tree
    (simulation/multiagent.py:51-55); returns dt.  ``nav`` = (dir_x, dir_y,
    minx, miny, step) with dir_x, dir_y of shape (targets, ny, nx) for
    ORC_NAVIGATION."""
    _check(agents)
    keep = None
    if nav is not None:
        mx, my, minx, miny, step_ = nav
        mx = np.ascontiguousarray(mx, dtype=np.float64)
        my = np.ascontiguousarray(my, dtype=np.float64)
        keep = (mx, my)
        lib().orc_set_navigation(mx.shape[0], _ptr(mx), _ptr(my), mx.shape[1], mx.shape[2],
                                 float(minx), float(miny), float(step_))
    else:
        lib().orc_set_navigation(0, None, None, 0, 0, 0.0, 0.0, 1.0)
        flags &= ~ORC_NAVIGATION
    off = _offsets(agents)
    w = np.zeros((0, 4)) if walls is None or len(walls) == 0 else \
        np.ascontiguousarray(np.asarray(walls).view(np.float64).reshape(-1, 4))
    nf = None if noise_f is None else np.ascontiguousarray(noise_f, dtype=np.float64)
    nm = None if noise_m is None else np.ascontiguousarray(noise_m, dtype=np.float64)
    if noise_f is None and noise_m is None:
        flags &= ~ORC_FLUCTUATION
    dt = lib().orc_step(_ptr(agents), len(agents), agents.dtype.itemsize, _ptr(off),
                        _body(agents), flags, ctypes.byref(grid), _ptr(w), len(w),
                        None if nf is None else _ptr(nf), None if nm is None else _ptr(nm),
                        dt_min, dt_max, nthreads)
    if dt != dt:
        raise ValueError('non-finite agent position')
    return dt


def navigation(agents, dir_x, dir_y, minx, miny, step):
    """Navigation.update alone: target directions from the maps (targets, ny,
    nx) for the agents whose ``target`` names a map."""
    _check(agents)
    mx = np.ascontiguousarray(dir_x, dtype=np.float64)
    my = np.ascontiguousarray(dir_y, dtype=np.float64)
    lib().orc_set_navigation(mx.shape[0], _ptr(mx), _ptr(my), mx.shape[1], mx.shape[2],
                             float(minx), float(miny), float(step))
    off = _offsets(agents)
    lib().orc_navigation(_ptr(agents), len(agents), agents.dtype.itemsize, _ptr(off))
    lib().orc_set_navigation(0, None, None, 0, 0, 0.0, 0.0, 1.0)


def philox4x32_10(ctr, key):
    """Philox4x32-10 of the shared noise header: 4 output words."""
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return out


def device_noise(agents, seed, step):
    """The fluctuation noise the device draws at step `step` with `seed`:
    (force (n, 2), torque (n,) or None)."""
    _check(agents)
    off = _offsets(agents)
    n = len(agents)
    f = np.zeros((n, 2))
    three = _body(agents) == BODY_THREE_CIRCLE
    m = np.zeros(n) if three else None
    lib().orc_device_noise(_ptr(agents), n, agents.dtype.itemsize, _ptr(off), _body(agents),
                           int(seed), int(step), _ptr(f), None if m is None else _ptr(m))
    return f, m


def cell_list(x, y, grid):
    """Restated cell_lists.add_to_cells: (keys, points_indices, cells_count,
    cells_offset)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    n = len(x)
    ncells = grid.nx * grid.ny
    keys = np.zeros(n, np.int64)
    pidx = np.zeros(n, np.int64)
    cnt = np.zeros(ncells, np.int64)
    off = np.zeros(ncells, np.int64)
    rc = lib().orc_cell_list(_ptr(x), _ptr(y), n, ctypes.byref(grid), _ptr(keys),
                             _ptr(pidx), _ptr(cnt), _ptr(off))
    if rc != 0:
        raise ValueError('non-finite agent position')
    return keys, pidx, cnt, off


def candidate_pairs(x, y, grid):
    """All (i, j) candidate pairs in visiting order, shape (P, 2)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    total = lib().orc_candidate_pairs(_ptr(x), _ptr(y), len(x), ctypes.byref(grid), None, 0)
    if total < 0:
        raise ValueError('non-finite agent position')
    out = np.zeros((max(total, 1), 2), np.int64)
    lib().orc_candidate_pairs(_ptr(x), _ptr(y), len(x), ctypes.byref(grid), _ptr(out), total)
    return out[:total]
