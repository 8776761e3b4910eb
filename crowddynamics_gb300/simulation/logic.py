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
import numpy as np

from crowddynamics_gb300 import _native as N
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
