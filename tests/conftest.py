import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA device (GB300) and libcdgpu.so')


@pytest.fixture(scope='session')
def oracle():
    """The C oracle (built on first use)."""
    from oracle import build as ob
    ob.build()
    from oracle import oracle as O
    return O


@pytest.fixture(scope='session')
def native():
    """libcdgpu.so, built in-tree for sm_103a on first use."""
    from crowddynamics_gb300 import build as b
    b.build()
    from crowddynamics_gb300 import _native as N
    N.load()
    return N


def assert_vec_close(got, ref, rtol=1e-9, atol=1e-12, what=''):
    """Per-agent vector check: |got - ref| <= atol + rtol * |ref| (Euclidean
    norm over the trailing axis for vectors, absolute value for scalars)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    if got.ndim == 2:
        d = np.hypot(*(got - ref).T)
        s = np.hypot(*ref.T)
    else:
        d = np.abs(got - ref)
        s = np.abs(ref)
    bad = ~(d <= atol + rtol * s)
    if bad.any():
        k = int(np.argmax(np.where(bad, d / np.maximum(s, 1e-300), -1)))
        raise AssertionError('%s: %d/%d outside tolerance; worst index %d got %r ref %r '
                             '(abs %.3e rel %.3e)' % (what, int(bad.sum()), len(d), k, got[k],
                                                      ref[k], d[k], d[k] / max(s[k], 1e-300)))
