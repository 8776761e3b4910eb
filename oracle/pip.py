"""Point in polygon as the reference's InsideDomain / TargetReached nodes
compute it (test infrastructure only: the checker of the device kernels in
csrc/cd_states.cu, never called by the product path).

The reference calls matplotlib's ``Path(ring).contains_points(positions)``
(crowddynamics/simulation/logic.py:348-357 and :372-387) on the exterior ring
of a shapely polygon, with no transform and radius 0.  matplotlib is absent
here, so it cannot be run; what it computes for that call is the published
"crossings multiply" test of E. Haines ("Point in Polygon Strategies",
Graphics Gems IV, 1994, the CrossingsMultiplyTest routine), which matplotlib
carries (from the Anti-Grain Geometry 2.3 examples) as its point-in-path test.
This module restates that algorithm with the conventions of matplotlib's
use of it:

* every test point shoots a ray towards +x; an edge from an earlier vertex
  (x0, y0) to the next one (x1, y1) is a candidate when the flags
  ``y0 >= ty`` and ``y1 >= ty`` differ;
* a candidate is crossed when ``((y1 - ty) * (x0 - x1) >= (x1 - tx) * (y0 - y1))``
  equals the later vertex's flag (no division; plain float64 products);
* the vertices come in path order, the path is always closed: after the
  last vertex an edge back to the first one is tested (a ring whose last
  point repeats the first, as shapely writes exteriors, only adds edges of
  length zero, which are never candidates);
* a point with a non-finite coordinate is outside;
* inside = an odd number of crossings.

The flags make the test half-open: on the unit square (counter-clockwise)
the edge y = 1 and both vertical edges count as inside, the edge y = 0 as
outside; the known answers in tests/test_pip.py spell these out.  Parity
with matplotlib itself stays unpinned: it cannot run here.
"""
import numpy as np


def contains_points(points, ring):
    """Inside flags of `points` (n x 2) for the closed path through `ring`
    (m x 2 vertices in order)."""
    pts = np.asarray(points, dtype=np.float64).reshape(-1, 2)
    verts = np.asarray(ring, dtype=np.float64).reshape(-1, 2)
    tx, ty = pts[:, 0], pts[:, 1]
    finite = np.isfinite(tx) & np.isfinite(ty)
    crossed = np.zeros(len(pts), dtype=bool)
    m = len(verts)
    if m == 0:
        return crossed
    # the edges in path order, then the closing edge back to the first vertex
    for k in range(m):
        x0, y0 = verts[k]
        x1, y1 = verts[(k + 1) % m]
        f0, f1 = y0 >= ty, y1 >= ty
        with np.errstate(invalid='ignore'):
            hit = (f0 != f1) & (((y1 - ty) * (x0 - x1) >= (x1 - tx) * (y0 - y1)) == f1)
        crossed ^= hit
    return crossed & finite
