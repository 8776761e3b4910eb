"""Host record transfers: pinned host records are read and written by the
device directly (copy and transpose in one kernel pass), other host memory
through a staged copy.  Both must move exactly the same bytes, for both body
types, agent counts that do not fill the last block of records, and records
that carry fields of their own beyond the reference's."""
import numpy as np
import pytest
import torch

from crowddynamics_gb300 import _native as N
from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.engine import batch_from_scenarios, field_offsets

pytestmark = pytest.mark.gpu

NODES = N.NODE_ALL & ~N.NODE_FLUCTUATION


def pinned_like(a):
    """A copy of structured array ``a`` in page-locked host memory."""
    buf = torch.empty(max(a.nbytes, 1), dtype=torch.uint8, pin_memory=True)
    out = buf.numpy()[:a.nbytes].view(a.dtype)
    out[:] = a
    return out, buf


def with_extra_field(a):
    """``a`` with an extra float32 field after the reference's fields."""
    dt = np.dtype(a.dtype.descr + [('user_tag', '<f4')])
    out = np.zeros(len(a), dt)
    for name in a.dtype.names:
        out[name] = a[name]
    out['user_tag'] = np.arange(len(a), dtype=np.float32) * 0.5 + 3.0
    return out


def c_upload(b, records):
    """cd_upload_agents on any record layout (the Python layer accepts only
    the reference's exact dtypes; the C ABI takes any field offsets)."""
    off = field_offsets(records.dtype)
    assert b._lib.cd_upload_agents(b._ctx, N.ptr(records), len(records), records.dtype.itemsize,
                                   N.i64ptr(off)) == 0


def c_download(b, records):
    off = field_offsets(records.dtype)
    assert b._lib.cd_download_agents(b._ctx, N.ptr(records), len(records),
                                     records.dtype.itemsize, N.i64ptr(off)) == 0


def advance(scen, records, direct, steps=3):
    b, agents, _ = batch_from_scenarios([scen])
    b.set_direct_host_access(direct)
    c_upload(b, records)
    b.run(steps, NODES)
    return b


@pytest.mark.parametrize('make', [
    lambda: S.hallway(n=130, seed=5),
    lambda: S.room(n=197, seed=6),
    lambda: S.hallway(n=1, seed=7),
])
@pytest.mark.parametrize('extra', [False, True])
def test_direct_and_staged_transfers_identical(native, make, extra):
    scen = make()
    recs = with_extra_field(scen.agents) if extra else scen.agents.copy()
    pinned, keep_in = pinned_like(recs)
    # direct upload from pinned memory, staged upload from pageable memory
    bd = advance(scen, pinned, True)
    bs = advance(scen, recs.copy(), False)
    outs = {}
    for name, b in (('direct', bd), ('staged', bs)):
        o_pin, keep = pinned_like(np.zeros_like(recs))
        c_download(b, o_pin)                                   # direct when enabled
        o_page = np.zeros_like(recs)
        c_download(b, o_page)                                  # staged
        assert o_pin.tobytes() == o_page.tobytes(), name
        outs[name] = o_pin.copy()
        b.close()
        del keep
    assert outs['direct'].tobytes() == outs['staged'].tobytes()
    if extra:
        assert np.array_equal(outs['direct']['user_tag'], recs['user_tag'])
    else:
        ref, _, _ = batch_from_scenarios([scen])
        ref.run(3, NODES)
        r = np.zeros_like(recs)
        ref.download(r)
        ref.close()
        assert r.tobytes() == outs['direct'].tobytes()
    del keep_in


def test_direct_upload_round_trip(native):
    """Upload from pinned memory and download at once: the records come back
    byte for byte (no step in between)."""
    scen = S.room(n=300, seed=9)
    recs, keep = pinned_like(scen.agents)
    b, _, _ = batch_from_scenarios([scen])
    b.upload(recs)
    back, keep2 = pinned_like(np.zeros_like(recs))
    b.download(back)
    b.close()
    assert back.tobytes() == scen.agents.tobytes()
    del keep, keep2


@pytest.mark.parametrize('pinned', [True, False])
def test_step_records_matches_upload_run_download(native, pinned):
    """cd_step_records (upload, graph steps and download in one call, the
    host not waiting in between) gives the records of cd_upload_agents,
    cd_run and cd_download_agents, byte for byte, over three calls."""
    scen = S.room(n=1500, seed=12)
    recs = scen.agents.copy()
    if pinned:
        recs, keep = pinned_like(recs)
    b1, _, _ = batch_from_scenarios([scen])
    b2, _, _ = batch_from_scenarios([scen])
    ref = scen.agents.copy()
    for _ in range(3):
        b1.step_records(recs, 2, NODES)
        b2.upload(ref)
        b2.run(2, NODES)
        b2.download(ref)
        assert recs.tobytes() == ref.tobytes()
    b1.close()
    b2.close()


def test_step_records_without_steps_round_trips(native):
    """cd_step_records with no steps uploads and downloads the records:
    they come back byte for byte."""
    scen = S.hallway(n=700, seed=21)
    recs, keep = pinned_like(scen.agents)
    before = recs.tobytes()
    b, _, _ = batch_from_scenarios([scen])
    b.step_records(recs, 0, NODES)
    assert recs.tobytes() == before
    b.close()


def test_direct_upload_maxima_across_scenarios(native):
    """The direct upload reduces each scenario's largest target speed and
    extent in its own pass (per block of records, blocks that straddle
    scenarios included); the steps after it match those after a staged
    upload byte for byte, dt and time included."""
    sizes = [37, 64, 5, 129, 200, 1, 77, 300, 63, 65]
    scens = [S.hallway(n=n, seed=30 + k) for k, n in enumerate(sizes)]
    for k, sc in enumerate(scens):                 # distinct maxima per scenario
        sc.agents['target_velocity'] *= 1.0 + 0.1 * k
    bd, agents, _ = batch_from_scenarios(scens)
    bs, _, _ = batch_from_scenarios(scens)
    pinned, keep = pinned_like(agents)
    bd.set_direct_host_access(True)
    bs.set_direct_host_access(False)
    for _ in range(2):                             # the second upload reuses the keys
        c_upload(bd, pinned)
        c_upload(bs, agents.copy())
        bd.run(3, NODES)
        bs.run(3, NODES)
        od, os_ = np.zeros_like(agents), np.zeros_like(agents)
        bd.download(od)
        bs.download(os_)
        assert od.tobytes() == os_.tobytes()
        for x, y in zip(bd.time(), bs.time()):
            assert x.tobytes() == y.tobytes()
        pinned[:] = od
        agents = od.copy()
    bd.close()
    bs.close()
    del keep
