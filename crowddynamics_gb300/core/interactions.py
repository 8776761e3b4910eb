"""Agent-agent and agent-obstacle interactions on the device.

Drop-ins for ``crowddynamics/core/interactions.py:191-214``: same names,
arguments and in-place semantics.  ``agents`` is an ``agent_type_circular`` or
``agent_type_three_circle`` structured array; anything else raises
``InvalidType`` like the reference's dispatchers.  Forces (and torques)
accumulate into ``agents['force']`` (``agents['torque']``).

The neighbour grid of ``agent_agent_block_list`` starts at the lower-left
corner of the agents' bounding box with square cells of ``cell_size``; every
unordered pair of agents in the same or adjacent cells is a candidate, each
evaluated with the reference's (owner, other) orientation.
"""
from crowddynamics_gb300 import _native as N
from crowddynamics_gb300.core._device_call import run_nodes, DEFAULT_CELL
from crowddynamics_gb300.simulation.agents import body_type_of

SIGTH_SOC = 3.0


def agent_agent_block_list(agents, cell_size):
    """Agent-agent social and contact forces over a cell list
    (``core/interactions.py:191-205``)."""
    body_type_of(agents)
    run_nodes(agents, N.NODE_AGENT_AGENT, cell_size=float(cell_size))


def agent_obstacle(agents, obstacles):
    """Agent-wall contact forces (``core/interactions.py:208-214``);
    ``obstacles`` is an ``obstacle_type_linear`` array."""
    body_type_of(agents)
    if obstacles is None or len(obstacles) == 0:
        return
    run_nodes(agents, N.NODE_AGENT_OBSTACLE, cell_size=DEFAULT_CELL, walls=obstacles)
