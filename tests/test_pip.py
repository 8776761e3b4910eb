"""The point-in-polygon oracle (oracle/pip.py): the crossings multiply test
that matplotlib's Path.contains_points runs for the reference's InsideDomain
and TargetReached nodes, checked on known answers at the boundary (worked
out from the published test by hand) and against an independent even-odd
count on points off the boundary.  CPU only."""
import numpy as np
import pytest

from oracle.pip import contains_points

SQUARE = [(0, 0), (1, 0), (1, 1), (0, 1)]


# (point, inside) for the counter-clockwise unit square, from the test's flags
# (vertex.y >= ty) and its crossing product, edge by edge
SQUARE_KNOWN = [
    ((0.5, 0.5), True),
    ((0.5, 0.0), False),     # bottom edge: every flag true, no candidate edge
    ((0.5, 1.0), True),      # top edge: the right edge is crossed (0 >= -0.5)
    ((0.0, 0.5), True),      # left edge: the right edge is crossed, the left not
    ((1.0, 0.5), True),      # right edge: 0 >= -0 holds, equal to the later flag
    ((0.0, 0.0), False), ((1.0, 0.0), False),
    ((1.0, 1.0), True), ((0.0, 1.0), True),
    ((1.0 + 1e-12, 0.5), False), ((-1e-12, 0.5), False),
    ((0.5, 1.0 + 1e-12), False), ((0.5, -1e-12), False),
    ((np.nan, 0.5), False), ((0.5, np.inf), False), ((-np.inf, 0.5), False),
]


@pytest.mark.parametrize('ring', [SQUARE, SQUARE + [SQUARE[0]]], ids=['open', 'closed'])
def test_square_known_answers(ring):
    pts = np.array([p for p, _ in SQUARE_KNOWN], float)
    want = np.array([v for _, v in SQUARE_KNOWN])
    assert np.array_equal(contains_points(pts, ring), want)


def test_orientation_and_start_vertex_off_the_boundary():
    """Off the boundary the result is the even-odd rule: independent of the
    ring's orientation and starting vertex, and equal to a plain count of
    ray crossings computed with the intersection abscissa."""
    rng = np.random.default_rng(3)
    ring = np.array([(0, 0), (20, 0), (20, 8), (12, 8), (10, 4), (8, 8), (0, 8)], float)
    pts = rng.uniform(-3, 23, (20000, 2))
    base = contains_points(pts, ring)
    for r in (ring[::-1], np.roll(ring, 3, 0), np.vstack([ring, ring[:1]])):
        assert np.array_equal(contains_points(pts, r), base)
    count = np.zeros(len(pts), int)
    for k in range(len(ring)):
        (x0, y0), (x1, y1) = ring[k], ring[(k + 1) % len(ring)]
        straddle = (y0 > pts[:, 1]) != (y1 > pts[:, 1])
        with np.errstate(divide='ignore', invalid='ignore'):
            xc = x0 + (pts[:, 1] - y0) * (x1 - x0) / (y1 - y0)
        count += straddle & (xc > pts[:, 0])
    assert np.array_equal(base, count % 2 == 1)
    assert base.any() and (~base).any()
