"""Python handle on one device context (a batch of scenarios).

``DeviceBatch`` is a thin owner of a ``cd_ctx``: every method is one C-ABI
call.  A plain simulation is a batch of one scenario; the batched form packs
many independent scenarios (their agents and walls concatenated) into one
context so that one launch advances all of them.
"""
import ctypes
import math

import numpy as np

from crowddynamics_gb300 import _native as N
from crowddynamics_gb300.exceptions import InvalidType, InvalidValue
from crowddynamics_gb300.simulation.agents import (
    BODY_CIRCULAR, BODY_THREE_CIRCLE, body_type_of)
from crowddynamics_gb300.simulation.agents import field_offsets as _field_offsets

_OFFSETS = {}
_OFFSET_PTRS = {}


def field_offsets(dtype):
    """The C ABI offset table of ``dtype`` (computed once per dtype, read-only)."""
    off = _OFFSETS.get(dtype)
    if off is None:
        off = _field_offsets(dtype)
        off.flags.writeable = False
        _OFFSETS[dtype] = off
    return off


def _offsets_arg(dtype):
    """``field_offsets(dtype)`` as the C ABI's int64 pointer (made once per
    dtype; the table it points at is kept alive by the cache)."""
    p = _OFFSET_PTRS.get(dtype)
    if p is None:
        p = _OFFSET_PTRS[dtype] = N.i64ptr(field_offsets(dtype))
    return p


def walls_as_rows(walls):
    """obstacle_type_linear array / (W, 4) array / sequence of ((x0, y0),
    (x1, y1)) -> contiguous (W, 4) float64 rows (p0x, p0y, p1x, p1y)."""
    if walls is None:
        return np.zeros((0, 4))
    a = np.asarray(walls)
    if a.dtype.names is not None:
        out = np.empty((len(a), 4))
        if len(a):
            out[:, 0:2] = a['p0']
            out[:, 2:4] = a['p1']
        return out
    a = np.asarray(a, dtype=np.float64)
    if a.size == 0:
        return np.zeros((0, 4))
    return np.ascontiguousarray(a.reshape(-1, 4))


def grid_for_bounds(bounds, cell_size):
    """(x0, y0, cell, nx, ny) covering bounds = (xmin, ymin, xmax, ymax)."""
    xmin, ymin, xmax, ymax = (float(v) for v in bounds)
    if not all(math.isfinite(v) for v in (xmin, ymin, xmax, ymax)):
        raise InvalidValue('grid bounds must be finite')
    nx = max(1, int(math.floor((xmax - xmin) / cell_size)) + 1)
    ny = max(1, int(math.floor((ymax - ymin) / cell_size)) + 1)
    return xmin, ymin, float(cell_size), nx, ny


class DeviceBatch:
    """One ``cd_ctx``: ``body`` is 'circular' or 'three_circle'; ``specs`` is
    a list of dicts with keys n_agents, n_walls, grid=(x0, y0, cell, nx, ny),
    dt_min, dt_max."""

    def __init__(self, body, specs):
        self._lib = N.load()
        self.body = body
        self.body_code = BODY_CIRCULAR if body == 'circular' else BODY_THREE_CIRCLE
        if body not in ('circular', 'three_circle'):
            raise InvalidType('body must be circular or three_circle')
        arr = (N.Scenario * len(specs))()
        a0 = w0 = 0
        for k, sp in enumerate(specs):
            x0, y0, cell, nx, ny = sp['grid']
            arr[k] = N.Scenario(a0, int(sp['n_agents']), w0, int(sp['n_walls']),
                                float(x0), float(y0), float(cell), int(nx), int(ny),
                                float(sp.get('dt_min', 0.001)), float(sp.get('dt_max', 0.01)))
            a0 += int(sp['n_agents'])
            w0 += int(sp['n_walls'])
        self.n_agents, self.n_walls, self.n_scenarios = a0, w0, len(specs)
        self.specs = list(specs)
        ctx = ctypes.c_void_p()
        N.check(self._lib.cd_create(ctypes.byref(ctx), self.body_code, len(specs), arr))
        self._ctx = ctx
        self._offsets = None
        ncell = ctypes.c_int64()
        N.check(self._lib.cd_sizes(ctx, None, None, ctypes.byref(ncell)), ctx)
        self.n_cells = ncell.value

    # -- lifetime --
    def close(self):
        if getattr(self, '_ctx', None):
            self._lib.cd_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _chk(self, rc):
        N.check(rc, self._ctx)

    # -- data --
    def upload(self, records):
        if body_type_of(records) != self.body_code:
            raise InvalidType('agent dtype does not match the context body type')
        if not records.flags.c_contiguous:
            raise InvalidValue('agent array must be C-contiguous')
        self._offsets = field_offsets(records.dtype)
        self._chk(self._lib.cd_upload_agents(self._ctx, records.ctypes.data, len(records),
                                             records.dtype.itemsize,
                                             _offsets_arg(records.dtype)))

    def download(self, records):
        if not records.flags.c_contiguous or not records.flags.writeable:
            raise InvalidValue('agent array must be C-contiguous and writeable')
        self._chk(self._lib.cd_download_agents(self._ctx, records.ctypes.data, len(records),
                                               records.dtype.itemsize,
                                               _offsets_arg(records.dtype)))

    def step_records(self, records, steps=1, nodes=N.NODE_ALL & ~N.NODE_FLUCTUATION):
        """``steps`` steps of the host ``records`` in place: upload, graph
        steps and download in one call (cd_step_records), the drop-in form of
        the reference's update() on a host array."""
        if body_type_of(records) != self.body_code:
            raise InvalidType('agent dtype does not match the context body type')
        if not records.flags.c_contiguous or not records.flags.writeable:
            raise InvalidValue('agent array must be C-contiguous and writeable')
        self._offsets = field_offsets(records.dtype)
        self._chk(self._lib.cd_step_records(self._ctx, records.ctypes.data, len(records),
                                            records.dtype.itemsize, _offsets_arg(records.dtype),
                                            int(nodes), int(steps)))

    def snapshot(self, slot, records, dt=None, time_tot=None):
        """Enqueue an asynchronous copy of the state (after the steps already
        enqueued) into ``records`` and the per-scenario ``dt`` / ``time_tot``
        arrays; completion is awaited with ``snapshot_wait(slot)``.  The
        buffers must stay alive until then; page-locked memory makes the copy
        asynchronous."""
        if not records.flags.c_contiguous or not records.flags.writeable:
            raise InvalidValue('agent array must be C-contiguous and writeable')
        off = field_offsets(records.dtype)
        self._chk(self._lib.cd_snapshot_agents(
            self._ctx, int(slot), N.ptr(records), len(records), records.dtype.itemsize,
            N.i64ptr(off), None if dt is None else N.dptr(dt),
            None if time_tot is None else N.dptr(time_tot)))

    def snapshot_wait(self, slot):
        self._chk(self._lib.cd_snapshot_wait(self._ctx, int(slot)))

    def herding(self, with_herding=True, sight_follower=10.0, size_nearest_other=5,
                sight_leader=20.0, phi=0.45 * math.pi, w_herding=0.15, w_leader=0.40,
                w_direction=0.65):
        """Leader-follower update of every follower's target direction,
        target and index_leader (with herding: nearest unobstructed
        neighbours as well); defaults are the reference's."""
        self._chk(self._lib.cd_herding(self._ctx, 1 if with_herding else 0, float(sight_follower),
                                       int(size_nearest_other), float(sight_leader), float(phi),
                                       float(w_herding), float(w_leader), float(w_direction)))

    def inside_domain(self, scenario, polygon):
        """Set ``active`` = inside ``polygon`` ((m, 2) vertices); returns the
        number of agents whose state changed."""
        xy = np.ascontiguousarray(polygon, dtype=np.float64).reshape(-1, 2)
        changed = ctypes.c_int64()
        self._chk(self._lib.cd_inside_domain(self._ctx, int(scenario), N.ptr(xy), len(xy),
                                             ctypes.byref(changed)))
        return changed.value

    def exit_detection(self, scenario, centers, detection_range=20.0):
        """Followers that see a door centre within range take the nearest as
        their target and stop following."""
        c = np.ascontiguousarray(centers, dtype=np.float64).reshape(-1, 2)
        self._chk(self._lib.cd_exit_detection(self._ctx, int(scenario), N.ptr(c), len(c),
                                              float(detection_range)))

    def target_reached(self, scenario, polygons, reset=False):
        """Agents that have been inside each target polygon (since the first
        call or ``reset``): counts per target."""
        polys = [np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 2) for p in polygons]
        if not polys:
            return np.zeros(0, np.int64)
        xy = np.ascontiguousarray(np.concatenate(polys))
        off = np.zeros(len(polys) + 1, np.int64)
        off[1:] = np.cumsum([len(p) for p in polys])
        counts = np.zeros(len(polys), np.int64)
        self._chk(self._lib.cd_target_reached(self._ctx, int(scenario), len(polys), N.ptr(xy),
                                              N.i64ptr(off), 1 if reset else 0,
                                              N.i64ptr(counts)))
        return counts

    def set_walls(self, walls):
        rows = walls_as_rows(walls)
        self._chk(self._lib.cd_set_walls(self._ctx, N.ptr(rows), len(rows)))

    def set_direction_maps(self, scenario, dir_x, dir_y, minx, miny, step):
        """Direction maps of one scenario for NODE_NAVIGATION: dir_x, dir_y of
        shape (targets, ny, nx) or (ny, nx), indexed [row = y, column = x] on
        the meshgrid with origin (minx, miny) and spacing ``step``.  Empty
        (0 targets) removes the scenario's maps."""
        mx = np.asarray(dir_x, dtype=np.float64)
        my = np.asarray(dir_y, dtype=np.float64)
        if mx.ndim == 2:
            mx, my = mx[None], my[None]
        if mx.ndim != 3 or mx.shape != my.shape:
            raise InvalidValue('direction maps must have shape (targets, ny, nx)')
        mx = np.ascontiguousarray(mx)
        my = np.ascontiguousarray(my)
        t, ny, nx = mx.shape
        self._chk(self._lib.cd_set_direction_maps(self._ctx, int(scenario), t, N.ptr(mx),
                                                  N.ptr(my), ny, nx, float(minx), float(miny),
                                                  float(step)))

    def set_direct_host_access(self, enable=True):
        """Pinned host records are read and written by the device directly
        (copy and transpose in one pass); False stages every transfer
        through a copy.  Both give the same bytes."""
        self._chk(self._lib.cd_set_direct_host_access(self._ctx, 1 if enable else 0))

    def set_noise_mode(self, device, seed=0, step=0):
        """Fluctuation noise from the host (``device=False``: set_noise before
        each step) or drawn on the device from the counter generator with
        ``seed``; the next step uses counter ``step + 1``."""
        self._chk(self._lib.cd_set_noise_mode(self._ctx, 1 if device else 0, int(seed),
                                              int(step)))

    def set_noise(self, force, torque=None):
        f = np.ascontiguousarray(force, dtype=np.float64)
        if f.shape != (self.n_agents, 2):
            raise InvalidValue('force noise must have shape (n, 2)')
        m = None
        if torque is not None:
            m = np.ascontiguousarray(torque, dtype=np.float64)
            if m.shape != (self.n_agents,):
                raise InvalidValue('torque noise must have shape (n,)')
        self._chk(self._lib.cd_set_noise(self._ctx, N.ptr(f), N.ptr(m)))

    # -- stepping --
    def step(self, nodes=N.NODE_ALL, want_dt=False):
        """One update with the given node flags; returns per-scenario dt when
        ``want_dt`` (waits for the step), else None."""
        if want_dt:
            dt = np.zeros(self.n_scenarios)
            self._chk(self._lib.cd_step(self._ctx, int(nodes), N.dptr(dt)))
            return dt
        self._chk(self._lib.cd_step(self._ctx, int(nodes), None))
        return None

    def run(self, steps, nodes=N.NODE_ALL & ~N.NODE_FLUCTUATION):
        """``steps`` updates as CUDA-graph launches; waits and checks status."""
        self._chk(self._lib.cd_run(self._ctx, int(nodes), int(steps)))

    def launch(self, steps, nodes=N.NODE_ALL & ~N.NODE_FLUCTUATION):
        """Enqueue ``steps`` graph launches and return without waiting."""
        self._chk(self._lib.cd_launch(self._ctx, int(nodes), int(steps)))

    def set_variant(self, variant):
        """Force-kernel launch variant (results identical; speed differs)."""
        self._chk(self._lib.cd_set_variant(self._ctx, int(variant)))
        self.variant = int(variant)

    def set_near_list_capacity(self, entries):
        """Fix the pair pipeline's near-list capacity (entries; a negative
        value returns to automatic sizing)."""
        self._chk(self._lib.cd_set_near_list_capacity(self._ctx, int(entries)))

    def rollout_loss(self, steps, target, checkpoint_every=20, grads=True):
        """Run ``steps`` updates, return (loss, grads, forward_ms, adjoint_ms):
        loss = mean over steps and agents of |x(t) - target[t]|^2, grads =
        d loss / d (tau_adj, target_velocity, tau_0, k_soc) per agent (n x 4,
        None unless ``grads``).  Circular agents, one scenario."""
        tgt = np.ascontiguousarray(target, dtype=np.float64)
        if tgt.shape != (int(steps), self.n_agents, 2):
            raise InvalidValue('target must have shape (steps, n, 2)')
        loss = ctypes.c_double()
        fms, ams = ctypes.c_double(), ctypes.c_double()
        g = np.zeros((self.n_agents, 4)) if grads else None
        self._chk(self._lib.cd_rollout_loss(self._ctx, int(steps), N.ptr(tgt),
                                            int(checkpoint_every), ctypes.byref(loss),
                                            None if g is None else N.dptr(g),
                                            ctypes.byref(fms), ctypes.byref(ams)))
        return loss.value, g, fms.value, ams.value

    def synchronize(self):
        self._chk(self._lib.cd_synchronize(self._ctx))

    def time(self):
        dt = np.zeros(self.n_scenarios)
        tt = np.zeros(self.n_scenarios)
        self._chk(self._lib.cd_get_time(self._ctx, N.dptr(dt), N.dptr(tt)))
        return dt, tt

    # -- diagnostics --
    def cell_list(self):
        keys = np.zeros(self.n_agents, np.int64)
        order = np.zeros(self.n_agents, np.int64)
        cnt = np.zeros(self.n_cells, np.int64)
        off = np.zeros(self.n_cells, np.int64)
        self._chk(self._lib.cd_get_cell_list(self._ctx, N.i64ptr(keys), N.i64ptr(order),
                                             N.i64ptr(cnt), N.i64ptr(off)))
        return keys, order, cnt, off

    def pair_counts(self):
        """Per-agent counts (n, 9): candidates, near, interacting (h < 3),
        contact (h < 0), walls near, walls in contact (pair columns count
        each unordered pair twice); then social-force branches over the
        pairs the agent comes first in (each pair once): sub-pair loop run,
        defined time-to-collision roots, valid time-to-collision."""
        c = np.zeros((self.n_agents, len(N.COUNT_COLS)), np.int64)
        self._chk(self._lib.cd_pair_counts(self._ctx, N.i64ptr(c)))
        return c

    def set_timing(self, enable=True, kernels=True):
        """CUDA-event timing; ``kernels=False`` times whole runs only, with no
        event node inside the step graph (see cd_set_timing)."""
        mode = 0 if not enable else (1 if kernels else 2)
        self._chk(self._lib.cd_set_timing(self._ctx, mode))

    def kernel_time(self):
        """dict(force_ms, force_launches, step_ms, run_ms, run_steps, pair_ms,
        pair_launches, light_ms, pairs_ms) since the last set_timing (pair_ms:
        the pair stage; light_ms, pairs_ms: its float32 pass and k_pairs)."""
        f, s, r = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        n, rn = ctypes.c_int64(), ctypes.c_int64()
        self._chk(self._lib.cd_kernel_time(self._ctx, ctypes.byref(f), ctypes.byref(n),
                                           ctypes.byref(s), ctypes.byref(r), ctypes.byref(rn)))
        pm, pn = ctypes.c_double(), ctypes.c_int64()
        self._chk(self._lib.cd_pair_kernel_time(self._ctx, ctypes.byref(pm), ctypes.byref(pn)))
        lm, km = ctypes.c_double(), ctypes.c_double()
        self._chk(self._lib.cd_pair_kernel_times(self._ctx, ctypes.byref(lm), ctypes.byref(km),
                                                 None))
        return dict(force_ms=f.value, force_launches=n.value, step_ms=s.value,
                    run_ms=r.value, run_steps=rn.value, pair_ms=pm.value,
                    pair_launches=pn.value, light_ms=lm.value, pairs_ms=km.value)

    def pair_split(self):
        """The last pair-pipeline step's flat pair list: dict(pairs,
        first_part, deferred) (see cd_pair_split)."""
        v = [ctypes.c_int64() for _ in range(3)]
        self._chk(self._lib.cd_pair_split(self._ctx, *[ctypes.byref(x) for x in v]))
        return dict(pairs=v[0].value, first_part=v[1].value, deferred=v[2].value)

    def kernels_per_step(self, nodes=N.NODE_ALL):
        k = ctypes.c_int64()
        self._chk(self._lib.cd_kernels_per_step(self._ctx, int(nodes), ctypes.byref(k)))
        return k.value


class DeviceGroup:
    """Several DeviceBatch contexts advanced by one CUDA-graph launch
    (``cd_group_*``): ``steps_per_launch`` steps of ``nodes`` of every
    member per launch, each member exactly as its own ``launch`` would run
    it.  The members must stay open while the group is used."""

    def __init__(self, batches, nodes=N.NODE_ALL & ~N.NODE_FLUCTUATION, steps_per_launch=1):
        self._lib = N.load()
        self.batches = list(batches)
        arr = (ctypes.c_void_p * len(self.batches))(*[b._ctx for b in self.batches])
        g = ctypes.c_void_p()
        N.check_group(self._lib.cd_group_create(ctypes.byref(g), arr, len(self.batches),
                                                int(nodes), int(steps_per_launch)))
        self._g = g
        self.steps_per_launch = int(steps_per_launch)

    def launch(self, launches=1):
        """Enqueue ``launches`` graph launches; returns without waiting."""
        N.check_group(self._lib.cd_group_launch(self._g, int(launches)), self._g)

    def synchronize(self):
        """Wait for the launches; raise on any member's device status."""
        N.check_group(self._lib.cd_group_synchronize(self._g), self._g)

    def close(self):
        if getattr(self, '_g', None):
            self._lib.cd_group_destroy(self._g)
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_from_scenarios(scenarios):
    """DeviceBatch holding every scenario of ``scenarios`` (same body type),
    with the concatenated agent array and walls uploaded.  Returns
    (batch, agents, walls_rows)."""
    bodies = {s.body for s in scenarios}
    if len(bodies) != 1:
        raise InvalidType('a batch holds one body type')
    specs = [dict(n_agents=len(s.agents), n_walls=len(s.walls), grid=s.grid,
                  dt_min=s.dt_min, dt_max=s.dt_max) for s in scenarios]
    b = DeviceBatch(bodies.pop(), specs)
    agents = np.ascontiguousarray(np.concatenate([s.agents for s in scenarios]))
    walls = np.concatenate([walls_as_rows(s.walls) for s in scenarios]) if scenarios else np.zeros((0, 4))
    b.upload(agents)
    b.set_walls(walls)
    return b, agents, walls
