"""Minimal field: domain bounds and line obstacles.

The reference's ``Field`` holds shapely geometries
(``crowddynamics/simulation/field.py:18-163``) and converts obstacles to
``obstacle_type_linear`` segments every step
(``core/geometry.py:63-102``, ``simulation/logic.py:122-130``).  The device
path needs only the segments and a bounding box for the cell grid, so this
field accepts segments directly; a shapely-like geometry (``coords``,
``exterior`` or ``geoms``) is converted with the reference's segment rules.
"""
import numpy as np

from crowddynamics_gb300.core.structures import obstacle_type_linear


def geom_to_linesegment(geom):
    """Segments of a shapely-like geometry (``core/geometry.py:63-96``):
    points give none, line strings consecutive coordinate pairs, polygons
    their exterior ring, multi-part geometries the concatenation."""
    if hasattr(geom, 'geoms'):
        for g in geom.geoms:
            yield from geom_to_linesegment(g)
    elif hasattr(geom, 'exterior'):
        c = list(geom.exterior.coords)
        yield from zip(c[:-1], c[1:])
    elif hasattr(geom, 'coords'):
        c = list(geom.coords)
        yield from zip(c[:-1], c[1:])
    else:
        raise TypeError('unsupported geometry %r' % (geom,))


def geom_to_linear_obstacles(geom):
    """``core/geometry.py:99-102``: geometry -> obstacle_type_linear array."""
    segments = [] if geom is None else list(geom_to_linesegment(geom))
    return np.array(segments, dtype=obstacle_type_linear)


def as_linear_obstacles(obstacles):
    if obstacles is None:
        return np.zeros(0, dtype=obstacle_type_linear)
    if isinstance(obstacles, np.ndarray) and obstacles.dtype == obstacle_type_linear:
        return obstacles
    if hasattr(obstacles, 'coords') or hasattr(obstacles, 'exterior') or hasattr(obstacles, 'geoms'):
        return geom_to_linear_obstacles(obstacles)
    rows = np.asarray(obstacles, dtype=np.float64).reshape(-1, 4)
    out = np.zeros(len(rows), dtype=obstacle_type_linear)
    out['p0'] = rows[:, 0:2]
    out['p1'] = rows[:, 2:4]
    return out


class Field:
    """``domain``: (xmin, ymin, xmax, ymax) of the cell grid (None: fitted to
    agents and obstacles); ``obstacles``: wall segments."""

    def __init__(self, domain=None, obstacles=None, targets=()):
        self.domain = domain
        self.obstacles = as_linear_obstacles(obstacles)
        self.targets = list(targets)
