"""Adaptive-timestep velocity Verlet on the device.

Drop-ins for ``crowddynamics/core/integrator.py:29-97,209-256``.  The
position update uses the already-updated velocity, ``force_prev`` takes the
current force, ThreeCircle agents also update orientation (wrapped to
[-pi, pi]) and shoulder positions -- as in the reference.
"""
import numpy as np

from crowddynamics_gb300 import _native as N
from crowddynamics_gb300.core._device_call import run_nodes


def adaptive_timestep(agents, dt_min, dt_max):
    """Timestep in [dt_min, dt_max] from max |v| and max target velocity
    (``core/integrator.py:29-97``); ``agents`` is not modified."""
    if len(agents) == 0:
        return dt_max
    _, dt = run_nodes(agents, N.NODE_INTEGRATE, dt_min=dt_min, dt_max=dt_max,
                      write_back=False)
    return dt


def velocity_verlet_integrator(agents, dt_min, dt_max):
    """Advance ``agents`` in place by one adaptive step; returns the timestep
    (``core/integrator.py:209-256``)."""
    if len(agents) == 0:
        return dt_max
    _, dt = run_nodes(agents, N.NODE_INTEGRATE, dt_min=dt_min, dt_max=dt_max)
    return dt
