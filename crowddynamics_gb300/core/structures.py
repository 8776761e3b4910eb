"""Line-obstacle record (``crowddynamics/core/structures.py:6-9``): a wall
segment from ``p0`` to ``p1``, 32 bytes, the layout ``geom_to_linear_obstacles``
produces (``crowddynamics/core/geometry.py:99-102``)."""
import numpy as np

obstacle_type_linear = np.dtype([
    ('p0', np.float64, 2),
    ('p1', np.float64, 2),
])
