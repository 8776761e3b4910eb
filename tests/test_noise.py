"""Device fluctuation noise (cd_noise.h), CPU side: the Philox4x32-10
generator against the published known-answer vectors, the shared logarithm
against the C library, and the drawn force / torque distributions against
scipy's truncated normals (core/motion/fluctuation.py:14-62)."""
import math

import numpy as np
import pytest


def test_philox_known_answers(oracle):
    # Salmon et al. (SC11) Philox4x32-10 known-answer vectors
    cases = [
        ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
        ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
        ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
         [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
    ]
    for ctr, key, want in cases:
        assert list(oracle.philox4x32_10(ctr, key)) == want


def test_shared_log_accuracy(oracle):
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(0, 1, 20000), 10 ** rng.uniform(-300, 300, 20000),
                         rng.uniform(0.7, 1.4, 20000),
                         [1.0, 2.0, 0.5, 1e-308, 5e-324, 1.7e308, np.nextafter(1, 0)]])
    for x in xs:
        got, want = oracle.cdm('log', float(x)), math.log(x)
        assert abs(got - want) <= 2 * math.ulp(want) or got == want, x
    assert oracle.cdm('log', 0.0) == -math.inf
    assert math.isnan(oracle.cdm('log', -1.0)) and math.isnan(oracle.cdm('log', math.nan))
    assert oracle.cdm('log', math.inf) == math.inf


def test_noise_distribution(oracle):
    stats = pytest.importorskip('scipy.stats')
    from crowddynamics_gb300 import scenarios as S
    a = S.room(n=2000, size=30.0, seed=1).agents
    a['mass'] = 2.0
    a['std_rand_force'] = 0.5
    a['inertia_rot'] = 3.0
    a['std_rand_torque'] = 0.25
    f, m = zip(*[oracle.device_noise(a, 12345, k) for k in range(1, 41)])
    f, m = np.concatenate(f), np.concatenate(m)
    mag = np.hypot(*f.T) / (2.0 * 0.5)
    ang = np.mod(np.arctan2(f[:, 1], f[:, 0]), 2 * np.pi) / (2 * np.pi)
    tq = m / (3.0 * 0.25)
    assert mag.max() <= 3.0 + 1e-12 and np.abs(tq).max() <= 3.0 + 1e-12
    assert stats.kstest(mag, stats.truncnorm(0, 3).cdf).pvalue > 1e-3
    assert stats.kstest(tq, stats.truncnorm(-3, 3).cdf).pvalue > 1e-3
    assert stats.kstest(ang, 'uniform').pvalue > 1e-3
    assert abs(mag.mean() - stats.truncnorm.mean(0, 3)) < 0.01


def test_noise_counter_streams(oracle):
    """Same (seed, step) -> same noise; other steps, seeds or agents differ;
    Circular agents get no torque."""
    from crowddynamics_gb300 import scenarios as S
    a = S.hallway(n=200, seed=2).agents
    f1, m1 = oracle.device_noise(a, 7, 3)
    f2, _ = oracle.device_noise(a, 7, 3)
    f3, _ = oracle.device_noise(a, 7, 4)
    f4, _ = oracle.device_noise(a, 8, 3)
    assert m1 is None
    assert np.array_equal(f1, f2)
    assert not np.any(np.all(f1 == f3, axis=1)) and not np.any(np.all(f1 == f4, axis=1))
    assert len({tuple(x) for x in f1}) == len(f1)
