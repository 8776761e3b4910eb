"""GB300-native per-step agent update for crowddynamics.

Hand-written FP64 CUDA kernels for sm_103a behind a C ABI (``libcdgpu.so``),
with a host-side mirror of the reference's logic-node and numba-kernel
interfaces so that existing simulations switch by changing imports.
"""
__version__ = '0.1.0'
