"""Adjusting force and torque on the device.

Drop-ins for ``crowddynamics/core/motion/adjusting.py:98-121``:
``force += (mass / tau_adj) * (v0 * e0 - v)`` and, for ThreeCircle agents,
``torque += inertia_rot / tau_rot * (wrap_to_pi(phi0 - phi) / pi * omega0 - omega)``.
"""
from crowddynamics_gb300 import _native as N
from crowddynamics_gb300.core._device_call import run_nodes
from crowddynamics_gb300.exceptions import InvalidType
from crowddynamics_gb300.simulation.agents import is_model


def force_adjust_agents(agents):
    """Add the adjusting force to every agent, in place."""
    if len(agents) == 0:
        return
    out, _ = run_nodes(agents, N.NODE_ADJUSTING, write_back=False)
    agents['force'] = out['force']


def torque_adjust_agents(agents):
    """Add the adjusting torque to every ThreeCircle agent, in place."""
    if not is_model(agents, 'three_circle'):
        raise InvalidType('torque_adjust_agents needs agent_type_three_circle')
    if len(agents) == 0:
        return
    out, _ = run_nodes(agents, N.NODE_ADJUSTING, write_back=False)
    agents['torque'] = out['torque']
