"""On-disk formats of SaveSimulationData (crowddynamics/io.py): the
reference's own save_npy / save_csv coroutines and ours write identical
files; the frame writer the device path uses gives the same .npy files as
np.save of the stacked frames; geometry mappings."""
import csv
import json
import os
import types

import numpy as np
import pytest

from crowddynamics_gb300 import io as IO
from crowddynamics_gb300 import scenarios as S


def reference_io():
    from oracle import ref_loader as RL
    if not RL.available():
        pytest.skip('reference source tree not present')
    from io import StringIO
    ns = {'np': np, 'os': os, 'csv': csv, 'json': json, 'StringIO': StringIO}
    RL._extract('crowddynamics/io.py', ('save_npy', 'save_csv'), ns)
    return types.SimpleNamespace(**ns)


def run_coroutine(factory, directory, items):
    co = factory(directory, 'x')
    co.send(None)
    for value, dump in items:
        co.send(value)
        co.send(dump)


def test_save_npy_matches_reference(tmp_path):
    ref = reference_io()
    a = S.hallway(n=50, seed=1).agents
    frames = []
    for k in range(7):
        f = a.copy()
        f['position'] += k
        frames.append((f, k in (2, 6)))
    os.makedirs(tmp_path / 'ref')
    os.makedirs(tmp_path / 'ours')
    run_coroutine(ref.save_npy, str(tmp_path / 'ref'), frames)
    run_coroutine(IO.save_npy, str(tmp_path / 'ours'), frames)
    for k in (0, 1):
        r = open(tmp_path / 'ref' / ('x_%d.npy' % k), 'rb').read()
        o = open(tmp_path / 'ours' / ('x_%d.npy' % k), 'rb').read()
        assert r == o
    got = IO.load_npy_concatenated(str(tmp_path / 'ours'), 'x')
    assert got.shape == (7, 50) and np.array_equal(got[3]['position'], frames[3][0]['position'])


def test_save_csv_matches_reference(tmp_path):
    ref = reference_io()
    rows = [({'iterations': k, 'time_tot': 0.01 * k + 1e-17, 'dt': 0.01 / (k + 1)}, k % 3 == 2)
            for k in range(8)]
    for name, factory in (('ref', ref.save_csv), ('ours', IO.save_csv)):
        os.makedirs(tmp_path / name)
        run_coroutine(factory, str(tmp_path / name), rows)
    assert open(tmp_path / 'ref' / 'x.csv').read() == open(tmp_path / 'ours' / 'x.csv').read()


@pytest.mark.parametrize('spill', [256 << 20, 3 * 316 * 30])
def test_frame_writer_equals_np_save(tmp_path, spill):
    """In memory and spilled to the side file: the same .npy bytes."""
    a = S.room(n=30, size=8.0, seed=2).agents
    w = IO.AgentFrameWriter(str(tmp_path), 'agents', a.dtype, len(a), spill_bytes=spill)
    frames = []
    for k in range(5):
        f = a.copy()
        f['velocity'] = k
        w.append(f)
        frames.append(f)
        if k == 2:
            w.dump()
    w.dump()
    w.close()
    np.save(tmp_path / 'want_0.npy', np.vstack(frames[:3]))
    np.save(tmp_path / 'want_1.npy', np.vstack(frames[3:]))
    for k in (0, 1):
        assert open(tmp_path / ('agents_%d.npy' % k), 'rb').read() == \
            open(tmp_path / ('want_%d.npy' % k), 'rb').read()
    assert not os.path.exists(tmp_path / '.agents.frames')


def test_geometry_mapping(tmp_path):
    scen = S.hallway(n=10, seed=1)
    g = {'domain': (0.0, 0.0, 40.0, 10.0), 'obstacles': scen.walls, 'targets': None,
         'spawns': [(0.0, 0.0, 1.0, 1.0)]}
    IO.save_geometry_json(str(tmp_path / 'geometry.json'), g)
    got = IO.load_geometry_json(str(tmp_path / 'geometry.json'))
    assert got['domain']['type'] == 'Polygon' and got['domain']['coordinates'][0][2] == [40.0, 10.0]
    assert got['obstacles']['type'] == 'MultiLineString'
    assert got['obstacles']['coordinates'][1] == [[0.0, 10.0], [40.0, 10.0]]
    assert got['targets'] is None and got['spawns'][0]['type'] == 'Polygon'
