"""cd_agent_agent_noalloc: agent-agent forces for callers that cannot
allocate device memory while they run (a host application that owns all
device memory through its own pool, or code where cudaMalloc is not
allowed).  The entry point keeps its scratch in a fixed array inside the
library; the caller passes device inputs and outputs only.

Checked through the C ABI against the context path (cd_step with
CD_NODE_AGENT_AGENT) on two calls in a row -- the second call finds the
first call's leftovers in the shared array -- within the parity tolerance
(1e-9 relative, 1e-12 absolute floor); both paths run the same kernels, so
the results are expected to be identical.  The device buffers below are
the test's own (allocated through torch), not the entry point's.
"""
import ctypes

import numpy as np
import pytest

from conftest import assert_vec_close
from crowddynamics_gb300 import _native as N
from crowddynamics_gb300 import scenarios as S
from crowddynamics_gb300.engine import batch_from_scenarios

pytestmark = pytest.mark.gpu

FIELD_OF = {'x': ('position', 0), 'y': ('position', 1), 'vx': ('velocity', 0),
            'vy': ('velocity', 1), 'x_ls': ('position_ls', 0), 'y_ls': ('position_ls', 1),
            'x_rs': ('position_rs', 0), 'y_rs': ('position_rs', 1)}


def columns(agents):
    three = 'position_ls' in agents.dtype.fields
    cols = []
    for name in N.NA_COLS:
        if name in FIELD_OF:
            f, k = FIELD_OF[name]
            if f not in agents.dtype.fields:
                cols.append(np.zeros(len(agents)))
                continue
            cols.append(agents[f][:, k])
        elif name in agents.dtype.fields:
            cols.append(agents[name])
        else:
            cols.append(np.zeros(len(agents)))
    if not three:
        cols = cols[:11]
    return np.ascontiguousarray(np.stack(cols).astype(np.float64))


def context_forces(scen):
    b, agents, _ = batch_from_scenarios([scen])
    b.step(N.NODE_AGENT_AGENT, want_dt=True)
    out = agents.copy()
    b.download(out)
    b.close()
    return out


def regridded(scen, bounds):
    """The scenario on another cell grid (same agents)."""
    return S.Scenario(scen.name, scen.agents, scen.walls, bounds, scen.cell_size)


def field_16k():
    """16,000 ThreeCircle agents on a 67 x 67 grid (4489 cells: the
    multi-block cell scan; the context path runs its pair pipeline here, the
    entry point its lane-group twin)."""
    return S.large_field(n=16000, size=240.0, n_walls=0, seed=8)


def hallway_max_cells():
    """The 400-agent hallway on a grid of exactly CD_NOALLOC_MAX_CELLS cells."""
    scen = S.hallway()
    side = int(N.NOALLOC_MAX_CELLS ** 0.5)
    return regridded(scen, (0.0, 0.0, side * scen.cell_size, side * scen.cell_size))


def room_outside_grid():
    """The room on a grid covering only its lower-left 12 m x 12 m: most
    agents lie outside it and are binned into its border cells."""
    scen = moving_room()
    return regridded(scen, (0.0, 0.0, 12.0, 12.0))


def moving_room():
    scen = S.room()
    scen.agents['velocity'] = np.random.default_rng(3).normal(0, 1.0, (len(scen.agents), 2))
    return scen


CASES = {'circular': S.hallway, 'three_circle': S.room, 'three_circle_16k': field_16k,
         'circular_max_cells': hallway_max_cells, 'three_circle_outside_grid': room_outside_grid}


@pytest.mark.parametrize('case', list(CASES))
def test_noalloc_matches_context_path(native, case):
    import torch
    scen = CASES[case]()
    assert len(scen.agents) <= N.NOALLOC_MAX_AGENTS
    assert scen.grid[3] * scen.grid[4] <= N.NOALLOC_MAX_CELLS
    ref = context_forces(scen)
    three = scen.body == 'three_circle'
    lib = native.load()
    dev_cols = torch.tensor(columns(scen.agents), device='cuda')
    x0, y0, cell, nx, ny = scen.grid
    for call in range(2):
        fx = torch.tensor(np.ascontiguousarray(scen.agents['force'][:, 0]), device='cuda')
        fy = torch.tensor(np.ascontiguousarray(scen.agents['force'][:, 1]), device='cuda')
        tq = torch.tensor(np.ascontiguousarray(scen.agents['torque']), device='cuda') if three \
            else None
        torch.cuda.synchronize()
        rc = lib.cd_agent_agent_noalloc(
            1 if three else 0, len(scen.agents), ctypes.c_void_p(dev_cols.data_ptr()),
            ctypes.c_void_p(fx.data_ptr()), ctypes.c_void_p(fy.data_ptr()),
            ctypes.c_void_p(tq.data_ptr()) if three else None,
            x0, y0, cell, nx, ny, None)
        assert rc == 0, lib.cd_last_error(None)
        got = np.stack((fx.cpu().numpy(), fy.cpu().numpy()), axis=1)
        assert_vec_close(got, ref['force'], 1e-9, 1e-12, 'force, call %d' % call)
        assert np.array_equal(got, ref['force'])
        if three:
            t = tq.cpu().numpy()
            assert_vec_close(t, ref['torque'], 1e-9, 1e-12, 'torque, call %d' % call)
            assert np.array_equal(t, ref['torque'])


def test_noalloc_rejects_oversize(native):
    lib = native.load()
    dummy = ctypes.c_void_p(16)          # never dereferenced: sizes are checked first
    rc = lib.cd_agent_agent_noalloc(0, N.NOALLOC_MAX_AGENTS + 1, dummy, dummy, dummy, None,
                                    0.0, 0.0, 3.6, 10, 10, None)
    assert rc == N.CD_ERR_CAPACITY
    assert b'CD_NOALLOC_MAX_AGENTS' in lib.cd_last_error(None)
    rc = lib.cd_agent_agent_noalloc(0, 100, dummy, dummy, dummy, None,
                                    0.0, 0.0, 3.6, 200, 200, None)
    assert rc == N.CD_ERR_CAPACITY
    assert b'CD_NOALLOC_MAX_CELLS' in lib.cd_last_error(None)
