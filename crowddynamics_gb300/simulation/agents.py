"""Agent record layouts for the device path.

The reference builds its structured dtypes from traitlets classes
(``crowddynamics/simulation/agents.py:32-292``) by walking the MRO and
emitting each class's own traits in definition order, skipping ``BodyType``
(``crowddynamics/simulation/agents.py:299-307``,
``crowddynamics/traits.py:158-219``).  The records are *packed*
(``numpy.dtype`` of a field list, no ``align=True``), so float64 fields sit at
4-byte-aligned offsets.  A caller's ``agents.array`` must keep exactly this
layout for the device upload/download to be a drop-in, so the field order
here is the reference's order, restated field by field.
"""
import numpy as np

from crowddynamics_gb300.exceptions import InvalidType

# States (crowddynamics/simulation/agents.py:32-60)
_STATES = [
    ('active', np.bool_),
    ('target_reached', np.bool_),
    ('target', np.int64),
    ('is_leader', np.bool_),
    ('is_follower', np.bool_),
    ('index_leader', np.int64),
    ('familiar_exit', np.int64),
]
# Body (crowddynamics/simulation/agents.py:63-95)
_BODY = [
    ('radius', np.float64),
    ('r_t', np.float64),
    ('r_s', np.float64),
    ('r_ts', np.float64),
    ('mass', np.float64),
    ('inertia_rot', np.float64),
    ('target_velocity', np.float64),
    ('target_angular_velocity', np.float64),
]
# TranslationalMotion (crowddynamics/simulation/agents.py:195-257)
_TRANSLATIONAL = [
    ('position', np.float64, (2,)),
    ('velocity', np.float64, (2,)),
    ('target_direction', np.float64, (2,)),
    ('force', np.float64, (2,)),
    ('force_prev', np.float64, (2,)),
    ('tau_adj', np.float64),
    ('k_soc', np.float64),
    ('tau_0', np.float64),
    ('mu', np.float64),
    ('kappa', np.float64),
    ('damping', np.float64),
    ('std_rand_force', np.float64),
]
# RotationalMotion (crowddynamics/simulation/agents.py:260-292)
_ROTATIONAL = [
    ('orientation', np.float64),
    ('angular_velocity', np.float64),
    ('target_orientation', np.float64),
    ('torque', np.float64),
    ('torque_prev', np.float64),
    ('tau_rot', np.float64),
    ('std_rand_torque', np.float64),
]
# ThreeCircle's own fields come first in its MRO
# (crowddynamics/simulation/agents.py:393-399).
_THREE_CIRCLE_OWN = [
    ('position_ls', np.float64, (2,)),
    ('position_rs', np.float64, (2,)),
]

#: Structured dtype of a Circular agent (228 bytes, packed).
agent_type_circular = np.dtype(_STATES + _BODY + _TRANSLATIONAL)
#: Structured dtype of a ThreeCircle agent (316 bytes, packed).
agent_type_three_circle = np.dtype(
    _THREE_CIRCLE_OWN + _STATES + _BODY + _TRANSLATIONAL + _ROTATIONAL)

AgentModelToType = {
    'circular': agent_type_circular,
    'three_circle': agent_type_three_circle,
}

#: Body-type codes shared with the C ABI (``CD_BODY_CIRCULAR`` /
#: ``CD_BODY_THREE_CIRCLE`` in ``include/cdgpu.h``).
BODY_CIRCULAR = 0
BODY_THREE_CIRCLE = 1

#: Field identifiers of the C ABI's offset table, in ``CD_F_*`` order.  Each
#: entry names a float64 field (vectors are two consecutive float64s), except
#: the integer and bool state fields from ``target`` on.
FIELD_NAMES = (
    'position', 'velocity', 'target_direction', 'force', 'force_prev',
    'radius', 'r_t', 'r_s', 'r_ts', 'mass', 'inertia_rot', 'target_velocity',
    'target_angular_velocity', 'tau_adj', 'k_soc', 'tau_0', 'mu', 'kappa',
    'damping', 'std_rand_force', 'position_ls', 'position_rs', 'orientation',
    'angular_velocity', 'target_orientation', 'torque', 'torque_prev',
    'tau_rot', 'std_rand_torque', 'target', 'active', 'is_leader', 'is_follower',
    'index_leader', 'familiar_exit',
)


def is_model(agents, model):
    """True if ``agents`` has the dtype of ``model`` ('circular' or
    'three_circle'); restates ``crowddynamics/simulation/agents.py:460-470``.
    """
    return hash(agents.dtype) == hash(AgentModelToType[model])


def body_type_of(agents):
    """Body-type code of a structured agent array, or raise ``InvalidType``
    as the reference dispatchers do (``core/interactions.py:197-205``)."""
    if is_model(agents, 'circular'):
        return BODY_CIRCULAR
    if is_model(agents, 'three_circle'):
        return BODY_THREE_CIRCLE
    raise InvalidType('agents must have dtype agent_type_circular or '
                      'agent_type_three_circle, got {}'.format(agents.dtype))


def field_offsets(dtype):
    """Byte offset of every ``FIELD_NAMES`` entry in ``dtype`` (-1 if absent),
    as an int64 array ready for the C ABI."""
    out = np.full(len(FIELD_NAMES), -1, dtype=np.int64)
    for k, name in enumerate(FIELD_NAMES):
        if name in dtype.fields:
            out[k] = dtype.fields[name][1]
    return out


def shoulders(agents):
    """Shoulder positions from torso position and orientation; restates
    ``crowddynamics/simulation/agents.py:473-486`` on the host:
    ``offset = r_ts * rotate270((cos phi, sin phi)) = r_ts * (sin phi, -cos phi)``.
    """
    phi = agents['orientation']
    offset = np.stack((np.sin(phi), -np.cos(phi)), axis=-1) * \
        agents['r_ts'][:, None]
    agents['position_ls'][:] = agents['position'] - offset
    agents['position_rs'][:] = agents['position'] + offset


def max_extent(agents):
    """Largest distance from an agent's torso centre to its skin.

    Circular: ``radius``.  ThreeCircle: the larger of ``r_t`` and the
    shoulder-centre distance plus ``r_s`` (using the stored shoulder
    positions).  Used to check that a cell size covers the social cut-off.
    """
    if len(agents) == 0:
        return 0.0
    if is_model(agents, 'circular'):
        return float(np.max(agents['radius']))
    x = agents['position']
    dl = np.hypot(*(agents['position_ls'] - x).T) + agents['r_s']
    dr = np.hypot(*(agents['position_rs'] - x).T) + agents['r_s']
    return float(np.max(np.maximum(agents['r_t'], np.maximum(dl, dr))))


def new_agents(n, model):
    """Zero-initialised agent array with the reference's defaults for the
    fields the hot path reads (``crowddynamics/simulation/agents.py:223-292``)."""
    a = np.zeros(n, dtype=AgentModelToType[model])
    a['active'] = True
    a['target'] = -1
    a['index_leader'] = -1
    a['familiar_exit'] = -1
    a['tau_adj'] = 0.5
    a['k_soc'] = 1.5
    a['tau_0'] = 3.0
    a['mu'] = 1.2e5
    a['kappa'] = 4e4
    a['damping'] = 500.0
    a['std_rand_force'] = 0.1
    if model == 'three_circle':
        a['tau_rot'] = 0.2
        a['std_rand_torque'] = 0.1
    return a


def agents_wrap_orientation(rad):
    """Element-wise ``wrap_to_pi`` (crowddynamics/core/vector2D.py:8-36) for
    host-side set-up: angles to [-pi, pi], odd negative multiples of pi to
    -pi.  ``numpy.mod`` has Python's float-modulo semantics."""
    rad = np.asarray(rad, dtype=np.float64)
    r = np.mod(rad, 2 * np.pi)
    out = np.where(r > np.pi, r - 2 * np.pi, r)
    return np.where((rad < 0) & (r == np.pi), -np.pi, out)


class Agents:
    """Container of the agent structured array (``simulation/agents.py:605-680``).

    ``array`` is the host view.  When the agents belong to a device-backed
    simulation, reading ``array`` first copies the newest device state into
    it, and the simulation re-uploads the array before its next device step
    (the caller may have modified it in place).
    """

    def __init__(self, agent_type='circular', array=None, size=0):
        if array is not None:
            agent_type = 'circular' if body_type_of(np.asarray(array)) == BODY_CIRCULAR \
                else 'three_circle'
        if isinstance(agent_type, str):
            model = agent_type
        elif isinstance(agent_type, np.dtype):
            model = 'circular' if agent_type == agent_type_circular else 'three_circle'
        else:
            model = getattr(agent_type, 'model', 'circular')
        self.model = model
        self._array = np.ascontiguousarray(array) if array is not None else new_agents(size, model)
        body_type_of(self._array)
        self._mirror = None

    @property
    def array(self):
        if self._mirror is not None:
            self._mirror.pull()
        return self._array

    @array.setter
    def array(self, value):
        self._array = np.ascontiguousarray(value)
        body_type_of(self._array)
        if self._mirror is not None:
            self._mirror.host_changed()

    @property
    def size(self):
        return len(self._array)
