"""Batched form: many independent scenarios of both body types advanced in
one context per body type.  Every scenario must evolve bit-identically to
the same scenario advanced alone, every force-kernel launch variant must give
identical forces, and the autotuner must pick and cache a variant."""
import json
import os

import numpy as np
import pytest

from crowddynamics_gb300 import _native as N
from crowddynamics_gb300 import autotune
from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.engine import batch_from_scenarios
from test_gpu_parity import assert_identical

pytestmark = pytest.mark.gpu

NODES = N.NODE_ALL & ~N.NODE_FLUCTUATION


@pytest.fixture(scope='module')
def mix():
    return S.batch_mix(n_scenarios=14, seed=21, n_min=60, n_max=3000)


def test_batch_equals_scenarios_alone(native, mix):
    for body in ('circular', 'three_circle'):
        group = [s for s in mix if s.body == body]
        assert group, body
        b, agents, _ = batch_from_scenarios(group)
        b.run(8, NODES)
        got = agents.copy()
        b.download(got)
        dt_b, tt_b = b.time()
        b.close()
        off = 0
        for k, s in enumerate(group):
            one, a1, _ = batch_from_scenarios([s])
            one.run(8, NODES)
            ref = a1.copy()
            one.download(ref)
            dt1, tt1 = one.time()
            one.close()
            assert_identical(got[off:off + len(s.agents)], ref, s.name)
            assert dt_b[k] == dt1[0] and tt_b[k] == tt1[0]
            off += len(s.agents)


def test_variants_identical(native, mix):
    for body in ('circular', 'three_circle'):
        s = max((x for x in mix if x.body == body), key=lambda x: len(x.agents))
        outs = []
        for v in range(len(N.variants())):
            b, agents, _ = batch_from_scenarios([s])
            b.set_variant(v)
            b.run(3, NODES)
            o = agents.copy()
            b.download(o)
            b.close()
            outs.append(o)
        for o in outs[1:]:
            assert_identical(o, outs[0], body)


def test_autotune_picks_and_caches(native, mix, tmp_path, monkeypatch):
    monkeypatch.setenv('CROWDDYNAMICS_GB300_TUNE_CACHE', str(tmp_path / 'tune.json'))
    group = [s for s in mix if s.body == 'three_circle']
    b, agents, _ = batch_from_scenarios(group)
    before = agents.copy()
    b.download(before)
    v, times = autotune.tune(b, agents, steps=2)
    assert times is not None and set(times) == set(range(len(N.variants())))
    assert v == min(times, key=times.get)
    after = agents.copy()
    b.download(after)
    assert_identical(after, before, 'state restored after tuning')
    v2, times2 = autotune.tune(b, agents)
    assert v2 == v and times2 is None
    data = json.load(open(tmp_path / 'tune.json'))
    assert len(data) == 1
    b.close()


@pytest.mark.parametrize('per_launch', [1, 4])
def test_group_launch_equals_contexts_alone(native, mix, per_launch):
    """Both body types' contexts advanced by one graph launch (cd_group_*),
    `per_launch` steps per launch: bit-identical to each context run alone,
    also after a member changes its variant (the group recaptures)."""
    from crowddynamics_gb300.engine import DeviceGroup
    bodies = ('circular', 'three_circle')
    groups = [[s for s in mix if s.body == body] for body in bodies]
    alone = []
    for g in groups:
        b, agents, _ = batch_from_scenarios(g)
        b.run(8, NODES)
        o = agents.copy()
        b.download(o)
        alone.append((o, b.time()))
        b.close()
    members = [batch_from_scenarios(g) for g in groups]
    grp = DeviceGroup([m[0] for m in members], NODES, steps_per_launch=per_launch)
    grp.launch(4 // per_launch)
    members[1][0].set_variant(7)                   # recaptured at the next launch
    grp.launch(4 // per_launch)
    grp.synchronize()
    for (b, agents, _), (ref, (dt, tt)) in zip(members, alone):
        got = agents.copy()
        b.download(got)
        assert_identical(got, ref, 'group member')
        dt_g, tt_g = b.time()
        assert np.array_equal(dt_g, dt) and np.array_equal(tt_g, tt)
    grp.close()
    for b, _, _ in members:
        b.close()
