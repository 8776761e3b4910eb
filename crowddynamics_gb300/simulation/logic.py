"""Logic nodes of the per-step update (``crowddynamics/simulation/logic.py``).

The motion and interaction nodes run on the device: their ``update()`` only
queues the node with the simulation, and ``MultiAgentSimulation.update()``
launches consecutive queued nodes as one fused device step (so a standard
tree costs one launch sequence per iteration instead of one pass per node).
Host nodes (any other ``LogicNode``) see an up-to-date ``agents.array``.

Traits keep the reference's names and defaults.  As in the reference, the
``sight_soc`` and ``f_soc_max`` traits of ``AgentAgentInteractions`` only
shape the cell size; the kernels use the reference's constants 3.0 m and
2000 N (``core/interactions.py:45``, ``core/motion/power_law.py:52``).
"""
import math
import os
import queue
import threading

import numpy as np

from crowddynamics_gb300 import _native as N
from crowddynamics_gb300.io import AgentFrameWriter, save_csv, save_geometry_json
from crowddynamics_gb300.scenarios import draw_noise
from crowddynamics_gb300.simulation.base import LogicNodeBase


class LogicNode(LogicNodeBase):
    """Node bound to a simulation (``simulation/logic.py:31-54``)."""

    def __init__(self, simulation, name=None, **traits):
        super().__init__(name=name)
        self.simulation = simulation
        for k, v in traits.items():
            if not hasattr(self, k):
                raise TypeError('%s has no trait %r' % (self.__class__.__name__, k))
            setattr(self, k, v)

    def update(self):
        raise NotImplementedError


class DeviceNode(LogicNode):
    """A node executed by the device step; ``FLAG`` is its CD_NODE_* bit."""
    FLAG = 0

    def update(self):
        self.simulation._queue_device_node(self)


class Reset(DeviceNode):
    """force = 0 (and torque = 0) -- ``simulation/logic.py:59-64``."""
    FLAG = N.NODE_RESET


class Integrator(DeviceNode):
    """Adaptive velocity Verlet -- ``simulation/logic.py:67-75``."""
    FLAG = N.NODE_INTEGRATE
    dt_min = 0.01
    dt_max = 0.01


class Fluctuation(DeviceNode):
    """Random force and torque (``simulation/logic.py:78-86``): drawn on the
    host each step with ``simulation.rng`` and added on the device, or drawn
    on the device when the simulation has a ``device_noise_seed``."""
    FLAG = N.NODE_FLUCTUATION

    def update(self):
        if getattr(self.simulation, 'device_noise_seed', None) is None:
            agents = self.simulation.agents._array
            self.simulation._pending_noise = draw_noise(agents, self.simulation.rng)
        super().update()


class Adjusting(DeviceNode):
    """Adjusting force/torque -- ``simulation/logic.py:89-94``."""
    FLAG = N.NODE_ADJUSTING


class AgentAgentInteractions(DeviceNode):
    """Agent-agent forces over the cell list -- ``simulation/logic.py:97-119``."""
    FLAG = N.NODE_AGENT_AGENT
    sight_soc = 3.0
    max_agent_radius = 0.3
    f_soc_max = 2e3
    _cell_size = None

    @property
    def cell_size(self):
        if self._cell_size is not None:
            return self._cell_size
        return self.sight_soc + 2 * self.max_agent_radius

    @cell_size.setter
    def cell_size(self, value):
        self._cell_size = float(value)


class AgentObstacleInteractions(DeviceNode):
    """Agent-wall forces -- ``simulation/logic.py:122-130``; walls come from
    ``simulation.field.obstacles``."""
    FLAG = N.NODE_AGENT_OBSTACLE


class Orientation(DeviceNode):
    """target_orientation = angle(target_direction) --
    ``simulation/logic.py:258-261``."""
    FLAG = N.NODE_ORIENTATION


class Navigation(DeviceNode):
    """Target direction from direction maps (``simulation/logic.py:135-165``):
    every agent whose ``target`` is t takes map t's direction at its nearest
    meshgrid index (``core/steering/navigation.py:69-78`` with the indicer of
    ``core/steering/quickest_path.py:40-43``); other agents and agents outside
    the map keep theirs.  Runs on the device.  The reference computes the maps
    by fast marching (``field.navigation_to_target``); here they are inputs:
    ``direction_maps`` is a list of (dir_x, dir_y) arrays indexed [y, x], one
    per target, on the meshgrid with origin ``origin`` and spacing ``step``."""
    FLAG = N.NODE_NAVIGATION
    direction_maps = None
    step = 0.1
    origin = (0.0, 0.0)

    def update(self):
        if not self.direction_maps:
            return
        self.simulation._use_direction_maps(self)
        super().update()


class SaveSimulationData(LogicNode):
    """Saving simulation data (``simulation/logic.py:264-337``) in the
    reference's formats (``crowddynamics/io.py``): ``metadata.csv`` and
    ``geometry.json`` once, then every update one frame of agent records and
    one row of ``simulation.data``; ``agents_{k}.npy`` and ``data.csv`` are
    written when ``save_condition(simulation)`` is true.

    The frame comes from the device without stopping it: the update enqueues
    an asynchronous copy of the state (and of dt, time_tot) into one of a few
    page-locked slots, behind the steps already enqueued; a writer thread
    waits for each copy, keeps the frame and writes the data row; a dump
    writes the buffered frames.  The host never waits for the device here
    except when all slots are busy.
    (The reference buffers references to the live agent array, so every frame
    of one of its files shows the state at the dump; here each frame is the
    state at its own update.)"""
    save_condition = None
    base_directory = '.'
    save_directory = None
    slots = 4

    def __init__(self, simulation, name=None, **traits):
        super().__init__(simulation, name=name, **traits)
        if self.save_condition is None:
            self.save_condition = lambda sim: True
        if self.save_directory is None:
            self.save_directory = simulation.name_with_timestamp
        os.makedirs(self.full_path, exist_ok=True)
        meta = save_csv(self.full_path, 'metadata')
        meta.send(None)
        meta.send(simulation.metadata)
        meta.send(True)
        field = simulation.field
        save_geometry_json(os.path.join(self.full_path, 'geometry.json'),
                           {name: getattr(field, name, None)
                            for name in ('domain', 'obstacles', 'targets', 'spawns')})
        self._data_csv = save_csv(self.full_path, 'data')
        self._data_csv.send(None)
        self._frames = None
        self._thread = None

    @property
    def full_path(self):
        return os.path.join(os.path.abspath(self.base_directory), self.save_directory)

    def add_to_simulation_logic(self):
        self.simulation.logic['Reset'].inject_before(self)

    def _start(self, batch, dtype, n):
        import torch                                  # page-locked host memory
        k = max(1, min(int(self.slots), N.SNAPSHOT_SLOTS))
        self._pinned = [torch.empty(max(n, 1) * dtype.itemsize, dtype=torch.uint8,
                                    pin_memory=True) for _ in range(k)]
        self._records = [p.numpy()[:n * dtype.itemsize].view(dtype) for p in self._pinned]
        self._times = [np.zeros((2, batch.n_scenarios)) for _ in range(k)]
        self._free = queue.Queue()
        for q in range(k):
            self._free.put(q)
        self._work = queue.Queue()
        self._frames = AgentFrameWriter(self.full_path, 'agents', dtype, n)
        self._error = None
        self._thread = threading.Thread(target=self._writer, daemon=True)
        self._thread.start()

    def _writer(self):
        while True:
            item = self._work.get()
            if item is None:
                self._work.task_done()
                return
            batch, slot, keys, values, save, offset = item
            try:
                batch.snapshot_wait(slot)
                self._frames.append(self._records[slot])          # copies the slot
                dt, tt = float(self._times[slot][0][0]), float(self._times[slot][1][0])
                self._free.put(slot)
                row = {k: (dt if k == 'dt' else tt + offset if k == 'time_tot' else values[k])
                       for k in keys}
                self._data_csv.send(row)
                self._data_csv.send(save)
                if save:
                    self._frames.dump()
            except Exception as exc:                    # reported by the next update
                self._error = exc
                self._free.put(slot)
            self._work.task_done()

    def update(self):
        sim = self.simulation
        save = bool(self.save_condition(sim))
        b = sim._ensure_batch()
        arr = sim.agents._array
        mirror = sim.agents._mirror
        if mirror is not None and mirror.host_dirty:    # host edits since the last step
            b.upload(arr)
            mirror.host_dirty = False
        if self._thread is None:
            self._start(b, arr.dtype, len(arr))
        if self._error is not None:
            raise self._error
        slot = self._free.get()
        times = self._times[slot]
        b.snapshot(slot, self._records[slot], times[0], times[1])
        keys = list(sim.data.keys())
        values = {k: dict.__getitem__(sim.data, k) for k in keys if k not in ('dt', 'time_tot')}
        self._work.put((b, slot, keys, values, save, getattr(sim, '_time_offset', 0.0)))

    def drain(self):
        """Wait until every queued frame has been written."""
        if self._thread is not None:
            self._work.join()
            if self._error is not None:
                raise self._error

    def close(self):
        if self._thread is not None:
            self.drain()
            self._work.put(None)
            self._thread.join()
            self._thread = None
            self._frames.close()


def _polygon_of(geom):
    """(m, 2) vertices of a polygon given as a shapely-like object (its
    exterior ring), a (xmin, ymin, xmax, ymax) box, or a vertex array."""
    if hasattr(geom, 'exterior'):
        return np.asarray(geom.exterior.coords, dtype=np.float64)
    arr = np.asarray(geom, dtype=np.float64)
    if arr.shape == (4,):
        x0, y0, x1, y1 = arr
        return np.array([[x0, y0], [x1, y0], [x1, y1], [x0, y1], [x0, y0]])
    return arr.reshape(-1, 2)


class LeaderFollower(LogicNode):
    """Followers steer towards the nearest visible leader heading away from
    them, or keep following a leader behind an obstacle, or fall back on a
    familiar exit (``simulation/logic.py:168-180``,
    ``core/steering/collective_motion.py:158-243``).  Runs on the device."""
    sight = 20.0

    def update(self):
        b = self.simulation._device_state()
        b.herding(False, sight_follower=1.0, sight_leader=self.sight)
        self.simulation._device_changed()


class LeaderFollowerWithHerding(LogicNode):
    """Followers average the heading of their ``size_nearest_other`` nearest
    unobstructed neighbours within ``sight_follower`` that head away from them
    and combine it with leader following (``simulation/logic.py:183-217``,
    ``core/steering/collective_motion.py:71-155,246-279``).  Runs on the
    device."""
    sight_follower = 10.0
    size_nearest_other = 5

    def update(self):
        b = self.simulation._device_state()
        b.herding(True, sight_follower=self.sight_follower,
                  size_nearest_other=self.size_nearest_other)
        self.simulation._device_changed()


class InsideDomain(LogicNode):
    """Agents outside the field's domain become inactive; counts state changes
    in ``data['inactive']`` (``simulation/logic.py:343-357``).  Runs on the
    device (crossings point-in-polygon test)."""

    def __init__(self, simulation, name=None, **traits):
        super().__init__(simulation, name=name, **traits)
        self.simulation.data['inactive'] = 0
        self.polygon = _polygon_of(simulation.field.domain)

    def update(self):
        sim = self.simulation
        changed = sim._device_state().inside_domain(0, self.polygon)
        sim._device_changed()
        sim.data['inactive'] = dict.__getitem__(sim.data, 'inactive') + changed


class TargetReached(LogicNode):
    """Counts, per target polygon of the field, the agents that have reached
    it, in ``data['target_{index}']`` (``simulation/logic.py:360-387``; the
    reference passes the whole agent array where the positions are meant).
    Runs on the device."""
    prefix = 'target_{index}'

    def __init__(self, simulation, name=None, **traits):
        super().__init__(simulation, name=name, **traits)
        self.polygons = [_polygon_of(t) for t in simulation.field.targets]
        self.names = [self.prefix.format(index=i) for i in range(len(self.polygons))]
        for name_ in self.names:
            self.simulation.data[name_] = 0
        self._first = True

    def update(self):
        if not self.polygons:
            return
        sim = self.simulation
        counts = sim._device_state().target_reached(0, self.polygons, reset=self._first)
        self._first = False
        for name_, c in zip(self.names, counts):
            sim.data[name_] = int(c)


class ExitDetection(LogicNode):
    """Followers that see the centre of a target (door) within
    ``detection_range`` take the nearest as their target and stop following
    (``simulation/logic.py:220-237``, ``core/evacuation.py:139-174``).  Door
    centres are the means of the targets' vertices.  Runs on the device."""
    detection_range = 20.0

    def update(self):
        sim = self.simulation
        centers = np.array([np.mean(_polygon_of(t), axis=0) for t in sim.field.targets])
        if not len(centers):
            return
        sim._device_state().exit_detection(0, centers, self.detection_range)
        sim._device_changed()
