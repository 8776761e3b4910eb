"""Target orientation from target direction on the device.

Drop-in for ``crowddynamics/core/steering/orientation.py:17-21``:
``target_orientation = atan2(e0.y, e0.x)`` for ThreeCircle agents.
"""
from crowddynamics_gb300 import _native as N
from crowddynamics_gb300.core._device_call import run_nodes
from crowddynamics_gb300.exceptions import InvalidType
from crowddynamics_gb300.simulation.agents import is_model


def orient_towards_target_direction(agents):
    if not is_model(agents, 'three_circle'):
        raise InvalidType('orient_towards_target_direction needs agent_type_three_circle')
    if len(agents) == 0:
        return
    out, _ = run_nodes(agents, N.NODE_ORIENTATION, write_back=False)
    agents['target_orientation'] = out['target_orientation']
