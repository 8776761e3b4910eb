"""ctypes binding of ``libcdgpu.so`` (the C ABI in ``include/cdgpu.h``).

The library is built in-tree by ``crowddynamics_gb300.build``.  There is no
fallback: if the library cannot be loaded, or no CUDA device is usable, every
entry point raises ``DeviceError``.
"""
import ctypes
import os

import numpy as np

from crowddynamics_gb300.exceptions import (
    CellOverflow, CrowdDynamicsException, DeviceError, InvalidType, InvalidValue)

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'libcdgpu.so')

CD_OK = 0
CD_ERR_INVALID_TYPE = 1
CD_ERR_INVALID_VALUE = 2
CD_ERR_CUDA = 3
CD_ERR_NOT_FINITE = 4
CD_ERR_CAPACITY = 5

NODE_FLUCTUATION = 1
NODE_ORIENTATION = 2
NODE_ADJUSTING = 4
NODE_AGENT_AGENT = 8
NODE_AGENT_OBSTACLE = 16
NODE_INTEGRATE = 32
NODE_RESET = 64
NODE_ALL = 127
NODE_NAVIGATION = 128
SNAPSHOT_SLOTS = 8

#: Exported entry points (every function declared in include/cdgpu.h).
SYMBOLS = (
    'cd_last_error', 'cd_create', 'cd_destroy', 'cd_upload_agents',
    'cd_download_agents', 'cd_step_records', 'cd_set_walls', 'cd_set_noise', 'cd_step', 'cd_run',
    'cd_synchronize', 'cd_get_time', 'cd_get_cell_list', 'cd_pair_counts',
    'cd_sizes', 'cd_set_timing', 'cd_kernel_time', 'cd_kernels_per_step',
    'cd_measure_fp64_peak', 'cd_agent_agent_noalloc', 'cd_variant_count',
    'cd_variant_shape', 'cd_set_variant', 'cd_set_near_list_capacity', 'cd_pair_kernel_time', 'cd_pair_kernel_times', 'cd_pair_split',
    'cd_set_direction_maps', 'cd_set_noise_mode', 'cd_set_direct_host_access', 'cd_snapshot_agents', 'cd_snapshot_wait',
    'cd_herding', 'cd_inside_domain', 'cd_target_reached', 'cd_exit_detection',
    'cd_launch',
    'cd_rollout_loss',
    'cd_group_create', 'cd_group_launch', 'cd_group_synchronize', 'cd_group_last_error',
    'cd_group_destroy',
)

#: Limits and column order of cd_agent_agent_noalloc.
NOALLOC_MAX_AGENTS = 16384
NOALLOC_MAX_CELLS = 16384
NA_COLS = ('x', 'y', 'vx', 'vy', 'mass', 'k_soc', 'tau_0', 'mu', 'kappa', 'damping', 'radius',
           'r_t', 'r_s', 'r_ts', 'x_ls', 'y_ls', 'x_rs', 'y_rs', 'orientation')

#: Columns of cd_pair_counts.
COUNT_COLS = ('candidates', 'near', 'interacting', 'contact', 'walls_near', 'walls_contact',
              'social', 'social_defined', 'social_valid')


class Scenario(ctypes.Structure):
    """``cd_scenario`` of include/cdgpu.h."""
    _fields_ = [
        ('agent_begin', ctypes.c_int64), ('agent_count', ctypes.c_int64),
        ('wall_begin', ctypes.c_int64), ('wall_count', ctypes.c_int64),
        ('x0', ctypes.c_double), ('y0', ctypes.c_double), ('cell_size', ctypes.c_double),
        ('nx', ctypes.c_int64), ('ny', ctypes.c_int64),
        ('dt_min', ctypes.c_double), ('dt_max', ctypes.c_double),
    ]


_lib = None


def load(path=None):
    """Load the library (once) and declare the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise DeviceError('libcdgpu.so not found at %s; run crowddynamics_gb300.build.build()'
                          % path)
    try:
        L = ctypes.CDLL(path)
    except OSError as e:
        raise DeviceError('cannot load libcdgpu.so: %s' % e)
    P = ctypes.c_void_p
    i64 = ctypes.c_int64
    pi64 = ctypes.POINTER(ctypes.c_int64)
    pd = ctypes.POINTER(ctypes.c_double)
    sig = {
        'cd_last_error': (ctypes.c_char_p, [P]),
        'cd_create': (ctypes.c_int, [ctypes.POINTER(P), ctypes.c_int, i64, ctypes.POINTER(Scenario)]),
        'cd_destroy': (None, [P]),
        'cd_upload_agents': (ctypes.c_int, [P, P, i64, i64, pi64]),
        'cd_download_agents': (ctypes.c_int, [P, P, i64, i64, pi64]),
        'cd_step_records': (ctypes.c_int, [P, P, i64, i64, pi64, ctypes.c_int, i64]),
        'cd_set_walls': (ctypes.c_int, [P, P, i64]),
        'cd_set_noise': (ctypes.c_int, [P, P, P]),
        'cd_step': (ctypes.c_int, [P, ctypes.c_int, pd]),
        'cd_run': (ctypes.c_int, [P, ctypes.c_int, i64]),
        'cd_synchronize': (ctypes.c_int, [P]),
        'cd_get_time': (ctypes.c_int, [P, pd, pd]),
        'cd_get_cell_list': (ctypes.c_int, [P, pi64, pi64, pi64, pi64]),
        'cd_pair_counts': (ctypes.c_int, [P, pi64]),
        'cd_sizes': (ctypes.c_int, [P, pi64, pi64, pi64]),
        'cd_set_timing': (ctypes.c_int, [P, ctypes.c_int]),
        'cd_kernel_time': (ctypes.c_int, [P, pd, pi64, pd, pd, pi64]),
        'cd_kernels_per_step': (ctypes.c_int, [P, ctypes.c_int, pi64]),
        'cd_measure_fp64_peak': (ctypes.c_int, [pd]),
        'cd_variant_count': (ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
        'cd_variant_shape': (ctypes.c_int, [ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 4),
        'cd_set_variant': (ctypes.c_int, [P, ctypes.c_int]),
        'cd_set_near_list_capacity': (ctypes.c_int, [P, i64]),
        'cd_pair_kernel_time': (ctypes.c_int, [P, pd, pi64]),
        'cd_pair_kernel_times': (ctypes.c_int, [P, pd, pd, pi64]),
        'cd_pair_split': (ctypes.c_int, [P, pi64, pi64, pi64]),
        'cd_set_noise_mode': (ctypes.c_int, [P, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64]),
        'cd_set_direct_host_access': (ctypes.c_int, [P, ctypes.c_int]),
        'cd_snapshot_agents': (ctypes.c_int, [P, ctypes.c_int, P, i64, i64, pi64, pd, pd]),
        'cd_snapshot_wait': (ctypes.c_int, [P, ctypes.c_int]),
        'cd_herding': (ctypes.c_int, [P, ctypes.c_int, ctypes.c_double, i64, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double]),
        'cd_inside_domain': (ctypes.c_int, [P, i64, P, i64, pi64]),
        'cd_exit_detection': (ctypes.c_int, [P, i64, P, i64, ctypes.c_double]),
        'cd_target_reached': (ctypes.c_int, [P, i64, i64, P, pi64, ctypes.c_int, pi64]),
        'cd_set_direction_maps': (ctypes.c_int, [P, i64, i64, P, P, i64, i64, ctypes.c_double,
                                                 ctypes.c_double, ctypes.c_double]),
        'cd_launch': (ctypes.c_int, [P, ctypes.c_int, i64]),
        'cd_rollout_loss': (ctypes.c_int, [P, i64, P, i64, pd, pd, pd, pd]),
        'cd_agent_agent_noalloc': (ctypes.c_int, [ctypes.c_int, i64, P, P, P, P, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_double, i64, i64, P]),
        'cd_group_create': (ctypes.c_int, [ctypes.POINTER(P), ctypes.POINTER(P), i64, ctypes.c_int,
                                           i64]),
        'cd_group_launch': (ctypes.c_int, [P, i64]),
        'cd_group_synchronize': (ctypes.c_int, [P]),
        'cd_group_last_error': (ctypes.c_char_p, [P]),
        'cd_group_destroy': (None, [P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc, ctx=None):
    """Map a CD_* status to the reference's exception hierarchy."""
    if rc == CD_OK:
        return
    raise_status(rc, load().cd_last_error(ctx).decode(errors='replace'))


def check_group(rc, group=None):
    """check() for the cd_group_* calls (the group's own message)."""
    if rc == CD_OK:
        return
    raise_status(rc, load().cd_group_last_error(group).decode(errors='replace'))


def raise_status(rc, msg):
    if rc == CD_ERR_INVALID_TYPE:
        raise InvalidType(msg)
    if rc in (CD_ERR_INVALID_VALUE, CD_ERR_NOT_FINITE):
        raise InvalidValue(msg)
    if rc == CD_ERR_CAPACITY:
        raise CellOverflow(msg)
    if rc == CD_ERR_CUDA:
        raise DeviceError(msg)
    raise CrowdDynamicsException('cdgpu status %d: %s' % (rc, msg))


def ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def i64ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def variants():
    """[(threads_per_block, staged_per_thread, lanes_per_agent, pair_pipeline)]
    of the force-kernel variants (pair_pipeline 0: per-agent kernels, 1: the
    pair pipeline, 2: the pair pipeline with a separate force pass)."""
    L = load()
    n = ctypes.c_int()
    check(L.cd_variant_count(ctypes.byref(n)))
    out = []
    for v in range(n.value):
        f = [ctypes.c_int() for _ in range(4)]
        check(L.cd_variant_shape(v, *[ctypes.byref(x) for x in f]))
        out.append(tuple(x.value for x in f))
    return out


def measure_fp64_peak():
    """FP64 FMA throughput of the current device, GFLOP/s."""
    g = ctypes.c_double()
    check(load().cd_measure_fp64_peak(ctypes.byref(g)))
    return g.value
