"""CPU-only checks of the host side: C-ABI symbols, record layout, logic-node
tree, node fusion, error mapping, geometry helpers, scenario generators and
the shared elementary functions."""
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# ---- C ABI ---------------------------------------------------------------

def header_functions():
    text = open(os.path.join(ROOT, 'include', 'cdgpu.h')).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(cd_[a-z0-9_]+)\s*\(', text)))


def test_library_exports_every_declared_symbol(native):
    import ctypes
    lib = ctypes.CDLL(native.LIB_PATH)
    declared = header_functions()
    assert len(declared) >= 15
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(native.SYMBOLS)


def test_null_context_is_rejected(native):
    """Every entry point that takes a context answers a NULL context with
    CD_ERR_INVALID_VALUE and a message, before touching the device (so this
    runs without a GPU); cd_destroy(NULL) does nothing."""
    import ctypes
    lib = native.load()
    text = open(os.path.join(ROOT, 'include', 'cdgpu.h')).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    sigs = re.findall(r'\bint\s+(cd_[a-z0-9_]+)\s*\(([^)]*)\)', text)
    checked = 0
    for name, params in sigs:
        params = [q.strip() for q in params.split(',') if q.strip()]
        if not params or not re.match(r'(const )?cd_ctx \*ctx$', params[0]):
            continue
        f = getattr(lib, name)
        args = [None]
        for t in f.argtypes[1:]:
            pointer = t in (ctypes.c_void_p, ctypes.c_char_p) or issubclass(t, ctypes._Pointer)
            args.append(None if pointer else 0)
        assert f(*args) == 2, name
        assert lib.cd_last_error(None), name
        checked += 1
    assert checked >= 25
    lib.cd_destroy(None)


def test_status_codes_map_to_reference_exceptions(native, monkeypatch):
    from crowddynamics_gb300 import exceptions as E

    class FakeLib:
        def cd_last_error(self, ctx):
            return b'msg'
    monkeypatch.setattr(native, '_lib', FakeLib())
    native.check(0)
    for rc, exc in ((1, E.InvalidType), (2, E.InvalidValue), (4, E.InvalidValue),
                    (3, E.DeviceError), (5, E.CellOverflow), (99, E.CrowdDynamicsException)):
        with pytest.raises(exc):
            native.check(rc)
    assert issubclass(E.InvalidType, TypeError) and issubclass(E.InvalidValue, ValueError)


# ---- record layout -------------------------------------------------------

def test_record_layout():
    from crowddynamics_gb300.simulation import agents as A
    c, t = A.agent_type_circular, A.agent_type_three_circle
    assert c.itemsize == 228 and t.itemsize == 316
    assert c.fields['radius'][1] == 28 and c.fields['position'][1] == 92
    assert t.fields['position'][1] == 124 and t.fields['orientation'][1] == 260
    for dt in (c, t):
        off = A.field_offsets(dt)[:29]          # float64 fields: 4-byte aligned
        assert np.all(off[off >= 0] % 4 == 0)
        assert off[A.FIELD_NAMES.index('position')] == dt.fields['position'][1]
    # Circular records have none of the ThreeCircle fields; both have target
    assert np.all(A.field_offsets(c)[20:29] == -1)
    assert A.field_offsets(c)[A.FIELD_NAMES.index('target')] == c.fields['target'][1]


def test_layout_matches_reference_definition():
    """The dtypes equal those the reference's trait classes produce: field
    order follows the MRO walk of crowddynamics/simulation/agents.py with
    BodyType skipped (checked by parsing the reference source)."""
    from oracle import ref_loader as RL
    if not RL.available():
        pytest.skip('reference source tree not present')
    src = open(os.path.join(RL.REFERENCE_ROOT, 'crowddynamics', 'simulation', 'agents.py')).read()

    def traits_of(cls):
        body = re.search(r'class %s\(.*?\):\n(.*?)(?=\nclass |\Z)' % cls, src, re.S).group(1)
        return re.findall(r'^    (\w+) = (?:Bool|Int|Float|Array)\(', body, re.M)
    order_c = traits_of('States') + traits_of('Body') + traits_of('TranslationalMotion')
    order_t = traits_of('ThreeCircle') + order_c + traits_of('RotationalMotion')
    from crowddynamics_gb300.simulation import agents as A
    assert list(A.agent_type_circular.names) == order_c
    assert list(A.agent_type_three_circle.names) == order_t


# ---- logic tree ------------------------------------------------------------

def test_tree_semantics():
    from crowddynamics_gb300.simulation.base import LogicNodeBase, post_order

    class Nd(LogicNodeBase):
        def update(self):
            pass
    r, a, b, c, d = (Nd(name=x) for x in 'rabcd')
    tree = r << a << (b << c, d)
    assert tree is r
    assert [n.name for n in r.children] == ['a', 'b', 'd']
    assert [n.name for n in post_order(r)] == ['a', 'c', 'b', 'd', 'r']
    e = Nd(name='e')
    b.inject_before(e)
    assert b.parent is e and e.parent is r
    assert r['c'] is c
    with pytest.raises(KeyError):
        r['zz']


def test_standard_tree_fuses_into_one_step(monkeypatch):
    from crowddynamics_gb300 import _native as N
    from crowddynamics_gb300.simulation import logic as L
    from crowddynamics_gb300.simulation.multiagent import MultiAgentSimulation
    from crowddynamics_gb300.simulation.agents import Agents
    sim = MultiAgentSimulation(agents=Agents('circular', size=3))
    sim.logic = L.Reset(sim) << (L.Integrator(sim) << (
        L.Adjusting(sim) << L.Orientation(sim), L.AgentAgentInteractions(sim),
        L.AgentObstacleInteractions(sim)))
    launched = []
    monkeypatch.setattr(sim, '_flush', lambda: (launched.append(sim._pending),
                                                setattr(sim, '_pending', 0)))
    sim.update()
    launched = [x for x in launched if x]
    assert launched == [N.NODE_ORIENTATION | N.NODE_ADJUSTING | N.NODE_AGENT_AGENT |
                        N.NODE_AGENT_OBSTACLE | N.NODE_INTEGRATE | N.NODE_RESET]
    assert sim.data['iterations'] == 1


def test_host_node_splits_fusion(monkeypatch):
    from crowddynamics_gb300 import _native as N
    from crowddynamics_gb300.simulation import logic as L
    from crowddynamics_gb300.simulation.multiagent import MultiAgentSimulation
    from crowddynamics_gb300.simulation.agents import Agents
    sim = MultiAgentSimulation(agents=Agents('three_circle', size=2))
    seen = []

    class Probe(L.LogicNode):
        def update(self):
            seen.append('probe')
    sim.logic = L.Reset(sim) << (L.Integrator(sim) << (L.Adjusting(sim) << Probe(sim),
                                                        L.AgentAgentInteractions(sim)))
    launched = []

    def fake_flush():
        if sim._pending:
            launched.append(sim._pending)
        sim._pending = 0
    monkeypatch.setattr(sim, '_flush', fake_flush)
    sim.update()
    assert seen == ['probe']
    assert launched == [N.NODE_ADJUSTING | N.NODE_AGENT_AGENT | N.NODE_INTEGRATE | N.NODE_RESET]
    # a device node out of the fused order starts a new launch
    sim.logic = L.Integrator(sim) << (L.Reset(sim), L.Adjusting(sim))
    launched.clear()
    sim.update()
    assert launched == [N.NODE_RESET, N.NODE_ADJUSTING | N.NODE_INTEGRATE]


def test_node_traits():
    from crowddynamics_gb300.simulation import logic as L
    n = L.AgentAgentInteractions(None)
    assert n.cell_size == 3.6
    n.max_agent_radius = 0.35
    assert abs(n.cell_size - 3.7) < 1e-12
    n.cell_size = 5.0
    assert n.cell_size == 5.0
    i = L.Integrator(None, dt_min=0.001, dt_max=0.02)
    assert (i.dt_min, i.dt_max) == (0.001, 0.02)
    with pytest.raises(TypeError):
        L.Integrator(None, nonsense=1)


# ---- geometry, engine helpers ---------------------------------------------

def test_walls_and_geometry_helpers():
    from crowddynamics_gb300.engine import walls_as_rows, grid_for_bounds
    from crowddynamics_gb300.simulation.field import geom_to_linear_obstacles, as_linear_obstacles
    from crowddynamics_gb300.core.structures import obstacle_type_linear
    w = np.zeros(2, obstacle_type_linear)
    w['p0'] = [(0, 0), (1, 1)]
    w['p1'] = [(2, 0), (1, 3)]
    assert np.array_equal(walls_as_rows(w), [[0, 0, 2, 0], [1, 1, 1, 3]])
    assert walls_as_rows(None).shape == (0, 4)

    class Line:
        coords = [(1, 2), (3, 4), (5, 6)]

    class Poly:
        class exterior:
            coords = [(5, 6), (7, 8), (9, 10), (5, 6)]

    class Multi:
        geoms = [Line(), Poly()]
    segs = geom_to_linear_obstacles(Multi())
    assert len(segs) == 5
    assert tuple(segs[2]['p0']) == (5, 6) and tuple(segs[4]['p1']) == (5, 6)
    assert len(as_linear_obstacles([[0, 0, 1, 1]])) == 1
    g = grid_for_bounds((0, 0, 40, 10), 3.7)
    assert g == (0.0, 0.0, 3.7, 11, 3)
    from crowddynamics_gb300.exceptions import InvalidValue
    with pytest.raises(InvalidValue):
        grid_for_bounds((0, 0, np.nan, 1), 3.0)


def test_scenarios_are_seeded():
    from crowddynamics_gb300 import scenarios as S
    a, b = S.hallway(seed=7), S.hallway(seed=7)
    assert a.agents.tobytes() == b.agents.tobytes()
    assert S.hallway(seed=8).agents.tobytes() != a.agents.tobytes()
    r = S.room(n=300, size=15.0, seed=3)
    from crowddynamics_gb300.simulation.agents import max_extent
    assert 3.0 + 2 * max_extent(r.agents) <= r.cell_size
    # no initial overlaps, clear of walls
    x = r.agents['position']
    d = np.hypot(*(x[:, None, :] - x[None, :, :]).transpose(2, 0, 1))
    np.fill_diagonal(d, np.inf)
    assert d.min() > 2 * 0.16
    f, m = S.draw_noise(r.agents, np.random.default_rng(0))
    assert f.shape == (300, 2) and m.shape == (300,)
    assert np.all(np.hypot(*f.T) <= 3 * 0.1 * r.agents['mass'] + 1e-9)


def test_direction_map_lookup():
    from crowddynamics_gb300 import scenarios as S
    mx, my, step = S.room_exit_direction_map(10.0, 10.0, 4.4, 5.6, step=0.5)
    e = S.lookup_direction(np.array([[1.0, 5.0], [9.9, 0.1], [50.0, 50.0]]), (mx, my), step,
                           defaults=np.array([[0, 0], [0, 0], [0.6, 0.8]]))
    assert np.allclose(e[0], (1.0, 0.0))
    assert np.allclose(np.hypot(*e[1]), 1.0)
    assert np.array_equal(e[2], (0.6, 0.8))       # outside the map keeps the default


# ---- shared elementary functions -------------------------------------------

def ulps(a, b):
    if a == b:
        return 0.0
    return abs(a - b) / abs(math.ulp(b))


def test_shared_math_accuracy(oracle):
    rng = np.random.default_rng(0)
    worst = dict(hypot=0, exp=0, sin=0, cos=0, atan2=0)
    for x, y in rng.uniform(-20, 20, (20000, 2)):
        worst['hypot'] = max(worst['hypot'], ulps(oracle.cdm('hypot', x, y), math.hypot(x, y)))
        worst['exp'] = max(worst['exp'], ulps(oracle.cdm('exp', x * 5), math.exp(x * 5)))
        if abs(math.sin(x)) > 1e-3:
            worst['sin'] = max(worst['sin'], ulps(oracle.cdm('sin', x), math.sin(x)))
        if abs(math.cos(x)) > 1e-3:
            worst['cos'] = max(worst['cos'], ulps(oracle.cdm('cos', x), math.cos(x)))
        worst['atan2'] = max(worst['atan2'], ulps(oracle.cdm('atan2', y, x), math.atan2(y, x)))
    assert max(worst.values()) <= 2, worst
    for y, x in ((0.0, 0.0), (-0.0, 0.0), (0.0, -0.0), (-0.0, -0.0), (1, 0), (-1, -0.0),
                 (math.inf, 1), (1, -math.inf), (math.inf, -math.inf)):
        r, e = oracle.cdm('atan2', y, x), math.atan2(y, x)
        assert r == e and math.copysign(1, r) == math.copysign(1, e), (y, x, r, e)
    assert math.isnan(oracle.cdm('exp', math.nan))
    assert oracle.cdm('exp', 800) == math.inf and oracle.cdm('exp', -800) == 0.0
    assert oracle.cdm('exp', -740) == math.exp(-740)
    assert math.isnan(oracle.cdm('sin', math.inf))


def test_navigation_fuses_into_the_step(monkeypatch):
    """Navigation (a device node) fuses with the rest of the standard tree
    into one launch; it runs first in the device step, which commutes with
    Fluctuation (different fields)."""
    from crowddynamics_gb300 import _native as N
    from crowddynamics_gb300.simulation import logic as L
    from crowddynamics_gb300.simulation.multiagent import MultiAgentSimulation
    from crowddynamics_gb300.simulation.agents import Agents
    sim = MultiAgentSimulation(agents=Agents('circular', size=3), rng=np.random.default_rng(0))
    nav = L.Navigation(sim)
    nav.direction_maps = [(np.zeros((2, 2)), np.zeros((2, 2)))]
    sim.logic = L.Reset(sim) << (L.Integrator(sim) << (
        L.Fluctuation(sim), L.Adjusting(sim) << (nav, L.Orientation(sim)),
        L.AgentAgentInteractions(sim)))
    launched = []
    monkeypatch.setattr(sim, '_use_direction_maps', lambda node: None)
    monkeypatch.setattr(sim, '_flush', lambda: (launched.append(sim._pending),
                                                setattr(sim, '_pending', 0)))
    sim.update()
    assert [x for x in launched if x] == [
        N.NODE_FLUCTUATION | N.NODE_NAVIGATION | N.NODE_ORIENTATION | N.NODE_ADJUSTING |
        N.NODE_AGENT_AGENT | N.NODE_INTEGRATE | N.NODE_RESET]
