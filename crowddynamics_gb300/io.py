"""Simulation data on disk in the reference's formats (``crowddynamics/io.py``).

* ``{basename}_{index}.npy``: agent records, one numpy file per dump, shape
  (frames, agents) of the agent dtype (``save_npy``, io.py:19-44);
* ``{basename}.csv``: a header row of the data keys, then one row of values
  per frame, appended at each dump (``save_csv``, io.py:97-136);
* ``geometry.json``: the field's geometries as GeoJSON-like mappings
  (``save_geometry_json``, io.py:159-172).

``save_npy`` and ``save_csv`` keep the reference's coroutine protocol: send
``None`` to start, then alternately a value and a bool (True dumps).
``AgentFrameWriter`` is the form the device path uses: frames are appended as
they arrive (kept in memory, or in a raw side file beyond a size limit) and
written as the ``.npy`` file at a dump.
"""
import csv
import json
import os
from io import StringIO

import numpy as np


# -- npy: agent records ----------------------------------------------------

def save_npy(directory, basename):
    """Coroutine writing ``{basename}_{index}.npy`` files of stacked arrays."""
    filepath = os.path.join(directory, basename + '_{index}.npy')
    frames = []
    index = 0
    while True:
        data = yield
        frames.append(np.array(data, copy=True))
        dump = yield
        if dump:
            np.save(filepath.format(index=index), np.vstack(frames))
            frames.clear()
            index += 1


def find_npy_files(directory, basename):
    """(index, path) of every ``{basename}_{index}.npy`` under ``directory``."""
    prefix = basename + '_'
    for root, _, files in os.walk(directory):
        for name in files:
            if name.startswith(prefix) and name.endswith('.npy'):
                stem = name[len(prefix):-len('.npy')]
                if stem.isdigit():
                    yield int(stem), os.path.join(root, name)


def load_npy(directory, basename):
    """The ``.npy`` files of ``basename`` in index order."""
    for _, path in sorted(find_npy_files(directory, basename)):
        yield np.load(path)


def load_npy_concatenated(directory, basename):
    return np.vstack(list(load_npy(directory, basename)))


class AgentFrameWriter:
    """``{basename}_{index}.npy`` files built from frames appended one at a
    time.  Frames are kept in memory until ``dump()`` writes them with
    ``np.save`` (the reference's format: the stacked frames); beyond
    ``spill_bytes`` of buffered frames they go to a raw side file instead and
    the dump copies them from there."""

    def __init__(self, directory, basename, dtype, n, spill_bytes=256 << 20):
        self.path = os.path.join(directory, basename + '_{index}.npy')
        self.raw = os.path.join(directory, '.' + basename + '.frames')
        self.dtype = np.dtype(dtype)
        self.n = int(n)
        self.spill_bytes = int(spill_bytes)
        self.index = 0
        self.frames = []
        self.spilled = 0
        self._fp = None

    def append(self, records):
        rec = np.array(records, dtype=self.dtype, copy=True)
        assert rec.shape == (self.n,)
        if self._fp is None and (len(self.frames) + 1) * rec.nbytes > self.spill_bytes:
            self._fp = open(self.raw, 'wb')
            for f in self.frames:
                self._fp.write(f.tobytes())
            self.spilled = len(self.frames)
            self.frames = []
        if self._fp is not None:
            self._fp.write(rec.tobytes())
            self.spilled += 1
        else:
            self.frames.append(rec)

    def dump(self):
        path = self.path.format(index=self.index)
        if self._fp is None:
            np.save(path, np.stack(self.frames) if self.frames else
                    np.zeros((0, self.n), self.dtype))
        else:
            self._fp.close()
            self._fp = None
            out = np.lib.format.open_memmap(path, mode='w+', dtype=self.dtype,
                                            shape=(self.spilled, self.n))
            if self.spilled and self.n:
                out[:] = np.memmap(self.raw, dtype=self.dtype, mode='r',
                                   shape=(self.spilled, self.n))
            out.flush()
            del out
            os.unlink(self.raw)
        self.index += 1
        self.frames = []
        self.spilled = 0

    def close(self):
        if self._fp is not None:
            self._fp.close()
            self._fp = None
        if os.path.exists(self.raw):
            os.unlink(self.raw)


# -- csv: simulation data ----------------------------------------------------

def save_csv(directory, basename):
    """Coroutine appending dict rows to ``{basename}.csv``: the first dict
    writes its keys as the header; rows reach the file at each dump."""
    filepath = os.path.join(directory, basename + '.csv')
    buffer = StringIO()
    writer = csv.writer(buffer)

    def flush():
        with open(filepath, 'a') as fp:
            fp.write(buffer.getvalue())
        buffer.truncate(0)
        buffer.seek(0)

    data = yield
    writer.writerow(data.keys())
    writer.writerow(data.values())
    if (yield):
        flush()
    while True:
        data = yield
        writer.writerow(data.values())
        if (yield):
            flush()


# -- json: geometry ----------------------------------------------------------

def geometry_mapping(geom):
    """GeoJSON-like mapping of a geometry: shapely-like objects through their
    ``__geo_interface__``, a (xmin, ymin, xmax, ymax) box as a Polygon, wall
    records or (W, 4) rows as a MultiLineString; lists map element-wise."""
    if geom is None:
        return None
    if hasattr(geom, '__geo_interface__'):
        return geom.__geo_interface__
    if isinstance(geom, np.ndarray) and geom.dtype.names and 'p0' in geom.dtype.names:
        return {'type': 'MultiLineString',
                'coordinates': [[list(map(float, w['p0'])), list(map(float, w['p1']))]
                                for w in geom]}
    arr = np.asarray(geom, dtype=object)
    if arr.ndim == 1 and len(arr) == 4 and all(np.isscalar(v) for v in arr):
        x0, y0, x1, y1 = (float(v) for v in geom)
        return {'type': 'Polygon',
                'coordinates': [[[x0, y0], [x1, y0], [x1, y1], [x0, y1], [x0, y0]]]}
    if isinstance(geom, np.ndarray) and geom.ndim == 2 and geom.shape[1] == 4:
        return {'type': 'MultiLineString',
                'coordinates': [[[float(r[0]), float(r[1])], [float(r[2]), float(r[3])]]
                                for r in geom]}
    if isinstance(geom, (list, tuple)):
        return [geometry_mapping(g) for g in geom]
    raise TypeError('cannot map geometry of type %s' % type(geom).__name__)


def save_geometry_json(filename, geometries):
    """Append the mapping of every named geometry to ``filename``."""
    with open(filename, 'a') as fp:
        json.dump({name: geometry_mapping(g) for name, g in geometries.items()}, fp,
                  indent=2, separators=(', ', ': '))


def load_geometry_json(filename):
    with open(filename) as fp:
        return json.load(fp)
