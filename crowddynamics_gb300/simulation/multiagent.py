"""Device-backed ``MultiAgentSimulation`` (``simulation/multiagent.py:16-55``).

``update()`` walks the logic tree in post-order like the reference.  Device
nodes are queued; a run of queued nodes whose order matches the fused step's
fixed order (fluctuation, orientation, adjusting, agent-agent, agent-wall,
integrate, reset) is launched as one ``cd_step``.  A host node, or a device
node out of that order, first flushes the queue.

The agent state lives on the device between steps.  ``agents.array`` pulls
it back on access, and an accessed (possibly modified) array is uploaded
again before the next device step.  ``data['dt']`` and ``data['time_tot']``
are read from the device when looked up.
"""
import collections
import datetime
import math

import numpy as np

from crowddynamics_gb300 import _native as N
from crowddynamics_gb300.engine import DeviceBatch, grid_for_bounds, walls_as_rows
from crowddynamics_gb300.exceptions import InvalidValue
from crowddynamics_gb300.simulation.agents import Agents, max_extent
from crowddynamics_gb300.simulation.base import post_order
from crowddynamics_gb300.simulation.field import Field
from crowddynamics_gb300.simulation.logic import (
    AgentAgentInteractions, DeviceNode, Integrator)

_ORDER = [N.NODE_FLUCTUATION, N.NODE_NAVIGATION, N.NODE_ORIENTATION, N.NODE_ADJUSTING,
          N.NODE_AGENT_AGENT, N.NODE_AGENT_OBSTACLE, N.NODE_INTEGRATE, N.NODE_RESET]
_RANK = {f: k for k, f in enumerate(_ORDER)}


class _Data(collections.OrderedDict):
    """simulation.data with 'dt' / 'time_tot' fetched from the device."""

    def __init__(self, sim):
        super().__init__()
        self._sim = sim

    def __getitem__(self, key):
        if key in ('dt', 'time_tot') and self._sim._time_stale:
            self._sim._pull_time()
        return super().__getitem__(key)


class _Mirror:
    def __init__(self, sim):
        self.sim = sim
        self.device_newer = False
        self.host_dirty = True

    def pull(self):
        if self.device_newer:
            self.sim._batch.download(self.sim.agents._array)
            self.device_newer = False
        self.host_dirty = True

    def host_changed(self):
        self.host_dirty = True
        self.device_newer = False


class MultiAgentSimulation:
    """Simulation of ``agents`` in ``field`` driven by the ``logic`` tree.

    Fluctuation noise is drawn on the host from ``rng`` (numpy/scipy, as the
    reference does) unless ``device_noise_seed`` is set: then the device
    draws it from its counter generator with that seed, and the host round
    trip of the noise arrays disappears."""

    def __init__(self, agents=None, field=None, logic=None, name=None, rng=None,
                 grid_margin=20.0, device_noise_seed=None):
        self.name = name or self.__class__.__name__
        self.timestamp = datetime.datetime.now(tz=datetime.timezone.utc)
        self.metadata = collections.OrderedDict(name=self.name)
        self.metadata['timestamp'] = str(self.timestamp)
        self.data = _Data(self)
        self.data['iterations'] = 0
        self.data['time_tot'] = 0.0
        self.data['dt'] = 0.0
        self.exit_condition = None
        self.field = field if field is not None else Field()
        self.agents = agents if isinstance(agents, Agents) or agents is None else Agents(array=agents)
        self.logic = logic
        self.rng = rng if rng is not None else np.random.default_rng()
        self.grid_margin = grid_margin
        self._batch = None
        self._batch_key = None
        self._pending = 0
        self._pending_noise = None
        self._time_stale = False
        self.device_noise_seed = device_noise_seed

    # -- device management --
    def _config(self):
        cell = 3.6
        dt_min, dt_max = Integrator.dt_min, Integrator.dt_max
        if self.logic is not None:
            for node in post_order(self.logic.root):
                if isinstance(node, AgentAgentInteractions):
                    cell = node.cell_size
                if isinstance(node, Integrator):
                    dt_min, dt_max = node.dt_min, node.dt_max
        return float(cell), float(dt_min), float(dt_max)

    def _ensure_batch(self):
        arr = self.agents._array
        walls = self.field.obstacles if self.field is not None else None
        nw = 0 if walls is None else len(walls)
        cell, dt_min, dt_max = self._config()
        if self.field is not None and self.field.domain is not None:
            bounds = self.field.domain
        else:
            pts = [arr['position'].reshape(-1, 2)]
            if nw:
                w = walls_as_rows(walls)
                pts += [w[:, :2], w[:, 2:]]
            pts = np.concatenate(pts)
            pts = pts[np.isfinite(pts).all(axis=1)]
            if len(pts) == 0:
                pts = np.zeros((1, 2))
            m = self.grid_margin
            bounds = (pts[:, 0].min() - m, pts[:, 1].min() - m, pts[:, 0].max() + m,
                      pts[:, 1].max() + m)
        key = (self.agents.model, len(arr), nw, cell, dt_min, dt_max)
        if self._batch is None or self._batch_key != key:
            if self._batch is not None:
                self._batch.close()
            grid = grid_for_bounds(bounds, cell)
            self._batch = DeviceBatch(self.agents.model, [dict(
                n_agents=len(arr), n_walls=nw, grid=grid, dt_min=dt_min, dt_max=dt_max)])
            self._batch_key = key
            if nw:
                self._batch.set_walls(walls)
            self.agents._mirror = _Mirror(self)
            self._time_offset = self.data.get('time_tot', 0.0) if 'time_tot' in self.data else 0.0
            if self.device_noise_seed is not None:
                self._batch.set_noise_mode(True, self.device_noise_seed,
                                           int(self.data.get('iterations', 0)))
        return self._batch

    def _device_state(self):
        """The device batch holding the current state, for host nodes that act
        on it (pending device nodes already flushed; host edits uploaded)."""
        b = self._ensure_batch()
        mirror = self.agents._mirror
        if mirror is not None and mirror.host_dirty:
            b.upload(self.agents._array)
            mirror.host_dirty = False
        return b

    def _device_changed(self):
        """A host node changed the device state."""
        if self.agents._mirror is not None:
            self.agents._mirror.device_newer = True

    def _use_direction_maps(self, node):
        """Upload the Navigation node's maps when they change."""
        b = self._ensure_batch()
        key = (id(node), tuple((id(mx), id(my)) for mx, my in node.direction_maps),
               float(node.step), tuple(node.origin))
        if getattr(self, '_nav_key', None) != key or getattr(self, '_nav_batch', None) is not b:
            self._flush()
            mx = np.stack([np.asarray(m[0], dtype=np.float64) for m in node.direction_maps])
            my = np.stack([np.asarray(m[1], dtype=np.float64) for m in node.direction_maps])
            b.set_direction_maps(0, mx, my, node.origin[0], node.origin[1], node.step)
            self._nav_key = key
            self._nav_batch = b

    def _queue_device_node(self, node):
        flag = node.FLAG
        if self._pending and _RANK[flag] <= max(_RANK[f] for f in _ORDER if self._pending & f):
            self._flush()
        self._pending |= flag

    def _flush(self):
        nodes = self._pending
        if not nodes:
            return
        self._pending = 0
        b = self._ensure_batch()
        mirror = self.agents._mirror
        if mirror.host_dirty:
            b.upload(self.agents._array)
            mirror.host_dirty = False
        if nodes & N.NODE_FLUCTUATION and self.device_noise_seed is None:
            f, m = self._pending_noise
            b.set_noise(f, m)
            self._pending_noise = None
        b.step(nodes)
        mirror.device_newer = True
        if nodes & N.NODE_INTEGRATE:
            self._time_stale = True

    def _pull_time(self):
        dt, tt = self._batch.time()
        collections.OrderedDict.__setitem__(self.data, 'dt', float(dt[0]))
        collections.OrderedDict.__setitem__(self.data, 'time_tot',
                                            float(tt[0]) + self._time_offset)
        self._time_stale = False

    # -- reference API --
    def update(self):
        """Execute one iteration (``simulation/multiagent.py:51-55``)."""
        if self.logic is None:
            raise InvalidValue('simulation has no logic tree')
        for node in post_order(self.logic.root):
            if isinstance(node, DeviceNode):
                node.update()
            else:
                self._flush()
                node.update()
        self._flush()
        self.data['iterations'] += 1

    @property
    def name_with_timestamp(self):
        """Name with timestamp (``simulation/base.py:115-118``)."""
        return '_'.join((self.name, str(self.timestamp).replace(' ', '_')))

    def run(self):
        """Update until ``exit_condition(self)`` is true (``simulation/base.py:123-125``);
        then wait for background writers (SaveSimulationData) to finish."""
        while self.exit_condition is None or not self.exit_condition(self):
            self.update()
        self.finish_writers()

    def finish_writers(self):
        """Wait until every queued save has reached the disk."""
        if self.logic is not None:
            for node in post_order(self.logic.root):
                if hasattr(node, 'drain'):
                    node.drain()

    def close(self):
        if self.logic is not None:
            for node in post_order(self.logic.root):
                if hasattr(node, 'close'):
                    node.close()
        if self._batch is not None:
            if self.agents._mirror is not None:
                self.agents._mirror.pull()
                self.agents._mirror = None
            self._batch.close()
            self._batch = None
