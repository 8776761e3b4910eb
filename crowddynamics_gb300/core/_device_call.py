"""One-shot device execution for the function-level drop-ins.

The reference's numba kernels are stateless functions that update a
structured agent array in place.  Their drop-ins here upload the array, run
the matching node(s) on the device, and copy the result back.  Contexts are
cached by shape so repeated calls do not reallocate device memory.
"""
import collections

import numpy as np

from crowddynamics_gb300 import _native as N
from crowddynamics_gb300.engine import DeviceBatch, grid_for_bounds, walls_as_rows
from crowddynamics_gb300.exceptions import InvalidValue
from crowddynamics_gb300.simulation.agents import body_type_of, BODY_CIRCULAR

_CACHE = collections.OrderedDict()
_CACHE_SIZE = 4
DEFAULT_CELL = 3.6


def _batch(body, n, nw, grid, dt_min, dt_max):
    key = (body, n, nw, grid, dt_min, dt_max)
    b = _CACHE.pop(key, None)
    if b is None:
        b = DeviceBatch(body, [dict(n_agents=n, n_walls=nw, grid=grid, dt_min=dt_min,
                                    dt_max=dt_max)])
    _CACHE[key] = b
    while len(_CACHE) > _CACHE_SIZE:
        _CACHE.popitem(last=False)[1].close()
    return b


def position_grid(agents, cell_size, walls=None):
    """Grid whose origin is the lower-left corner of the agents' (and walls')
    bounding box, cells of ``cell_size``."""
    pos = agents['position']
    pts = [pos.reshape(-1, 2)]
    if walls is not None and len(walls):
        w = walls_as_rows(walls)
        pts += [w[:, 0:2], w[:, 2:4]]
    pts = np.concatenate(pts)
    finite = np.isfinite(pts).all(axis=1)
    if not finite[:len(pos)].all():
        raise InvalidValue('agent positions must be finite')
    pts = pts[finite]
    lo, hi = pts.min(axis=0), pts.max(axis=0)
    return grid_for_bounds((lo[0], lo[1], hi[0], hi[1]), cell_size)


def run_nodes(agents, nodes, cell_size=DEFAULT_CELL, walls=None, dt_min=0.001,
              dt_max=0.01, noise=None, write_back=True):
    """Run ``nodes`` on a copy of ``agents`` on the device.  Returns (result
    array, dt).  With ``write_back`` the whole result is copied into
    ``agents``."""
    if not isinstance(agents, np.ndarray) or agents.ndim != 1:
        raise InvalidValue('agents must be a 1-d structured array')
    body = 'circular' if body_type_of(agents) == BODY_CIRCULAR else 'three_circle'
    src = np.ascontiguousarray(agents)
    nw = 0 if walls is None else len(walls_as_rows(walls))
    if len(src) == 0:
        return src.copy(), dt_max
    grid = position_grid(src, cell_size, walls)
    b = _batch(body, len(src), nw, grid, float(dt_min), float(dt_max))
    b.upload(src)
    if nw:
        b.set_walls(walls)
    if noise is not None:
        b.set_noise(*noise)
    dt = b.step(nodes, want_dt=True)[0]
    out = src.copy()
    b.download(out)
    if write_back:
        agents[...] = out
    return out, dt
