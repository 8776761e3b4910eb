"""Exception hierarchy of the reference (``crowddynamics/exceptions.py:10-43``),
restated so callers catching the reference's exceptions keep working.  The
device path adds ``DeviceError`` for CUDA-level failures and
``CellOverflow`` for an agent count that exceeds a fixed device capacity."""


class CrowdDynamicsException(Exception):
    """CrowdDynamics base exception."""


class InvalidType(CrowdDynamicsException, TypeError):
    """Arguments had an invalid type (for example an agent array whose dtype
    is neither ``agent_type_circular`` nor ``agent_type_three_circle``)."""


class InvalidValue(CrowdDynamicsException, ValueError):
    """Arguments had an incorrect value (non-finite state, bad sizes)."""


class OverlappingError(CrowdDynamicsException):
    """Two agents are overlapping."""


class AgentStructureFull(CrowdDynamicsException):
    """Agent structure is full."""


class DeviceError(CrowdDynamicsException, RuntimeError):
    """A CUDA call or kernel of the device path reported an error."""


class CellOverflow(CrowdDynamicsException):
    """A fixed-capacity device buffer was too small for the input."""
