"""Autotuner for the agent-force kernel's launch variant.

Every variant (threads per block x candidates staged per thread per pass,
``_native.variants()``) gives bit-identical forces; which one is fastest
depends on the agent count, density, body type and device.  ``tune()`` times
each variant on a context's own data with CUDA events around the force
kernel (agent-agent node only, state restored afterwards), keeps the fastest
and caches the choice in a JSON file keyed by device, body type, agent-count
bucket and density bucket, so later runs with a similar workload skip the
timing.

Cache file: ``$CROWDDYNAMICS_GB300_TUNE_CACHE`` if set, else
``~/.cache/crowddynamics_gb300/autotune.json``.
"""
import json
import math
import os

import numpy as np

from crowddynamics_gb300 import _native as N


def cache_path():
    p = os.environ.get('CROWDDYNAMICS_GB300_TUNE_CACHE')
    if p:
        return p
    return os.path.join(os.path.expanduser('~'), '.cache', 'crowddynamics_gb300', 'autotune.json')


def device_name():
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name()
    except Exception:
        pass
    return 'cuda-device'


def workload_key(batch, agents):
    """Cache key: device | body | log2 bucket of mean agents per scenario |
    density bucket (agents per m^2 of the grids, halves)."""
    n = max(batch.n_agents, 1)
    per = n / max(batch.n_scenarios, 1)
    area = sum(sp['grid'][3] * sp['grid'][4] * sp['grid'][2] ** 2 for sp in batch.specs)
    dens = n / max(area, 1e-9)
    return '%s|%s|n2^%d|rho%.1f' % (device_name(), batch.body, int(math.log2(per)),
                                    round(dens * 2) / 2)


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, data):
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = path + '.tmp'
    with open(tmp, 'w') as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def time_variants(batch, agents, steps=3):
    """Milliseconds per force-kernel launch for every variant on this
    batch's current state ({variant: ms}).  The agent array is re-uploaded
    afterwards, so the context state is unchanged."""
    saved = agents.copy()
    batch.download(saved)
    out = {}
    for v in range(len(N.variants())):
        batch.set_variant(v)
        batch.step(N.NODE_AGENT_AGENT)               # warm-up
        batch.set_timing(True)
        for _ in range(steps):
            batch.step(N.NODE_AGENT_AGENT)
        kt = batch.kernel_time()
        batch.set_timing(False)
        out[v] = kt['force_ms'] / max(kt['force_launches'], 1)
    batch.upload(saved)
    return out


def tune(batch, agents, steps=3, use_cache=True):
    """Pick and apply the fastest variant for ``batch``; returns
    (variant, {variant: ms} or None when taken from the cache)."""
    path = cache_path()
    key = workload_key(batch, agents)
    data = _load(path) if use_cache else {}
    if key in data:
        v = int(data[key]['variant'])
        if 0 <= v < len(N.variants()):
            batch.set_variant(v)
            return v, None
    times = time_variants(batch, agents, steps)
    best = min(times, key=times.get)
    batch.set_variant(best)
    if use_cache:
        data = _load(path)
        data[key] = {'variant': best, 'shape': N.variants()[best],
                     'ms': {str(k): round(t, 4) for k, t in times.items()}}
        try:
            _store(path, data)
        except OSError:
            pass
    return best, times
