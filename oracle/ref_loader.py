"""Execute the reference's own hot-path source under stub modules.

TEST INFRASTRUCTURE ONLY: used (in a container that has the reference source
tree) to pin the C oracle and to generate the golden fixtures under
``tests/golden/``.  Nothing on the product path imports it, and the GPU-side
tests never need it (they read the committed fixtures).

The reference cannot be imported as a package here: numba, cell_lists,
traitlets, anytree, shapely and other dependencies are missing, and
``simulation/agents.py`` uses pre-3.10 ``collections`` names.  Its hot-path
arithmetic, however, lives in plain numpy-compatible functions under numba
decorators.  This loader injects three stubs into ``sys.modules`` and then
executes the reference files by path, unchanged:

* ``numba``: ``jit`` / ``vectorize`` return the function unchanged,
  ``generated_jit`` dispatches on ``numpy.ndim``; signature objects are inert.
* ``cell_lists``: a restatement of ``add_to_cells``, ``neighboring_cells`` and
  ``iter_nearest_neighbors`` from their call sites
  (``crowddynamics/core/interactions.py:152-165,191-205``) on a configurable
  uniform grid: agents grouped by cell in ascending order, pairs within a cell
  (earlier, later) and with the forward half of the 3x3 stencil (owner cell
  first).  The package is pinned only as
  git+https://github.com/jaantollander/cell_lists.git without a version.
* ``crowddynamics.simulation.agents``: the agent dtypes (same field order as
  ``crowddynamics/simulation/agents.py:32-292,447-448``), ``is_model``
  (``:460-470``) and ``shoulders`` (``:473-486``).

Files executed: core/vector2D.py, core/structures.py, core/distance.py,
core/motion/contact.py, core/motion/power_law.py, core/motion/adjusting.py,
core/integrator.py, core/interactions.py, core/steering/orientation.py,
core/geom2D.py, core/sensory_region.py, core/steering/collective_motion.py,
core/evacuation.py, exceptions.py.
"""
import importlib.util
import os
import sys
import types

import numpy as np

# The reference source tree: the crowddynamics project root, named by the
# CROWDDYNAMICS_REFERENCE environment variable (unset: the tests that need it
# skip, and the committed fixtures stand in for it).
REFERENCE_ROOT = os.environ.get('CROWDDYNAMICS_REFERENCE', '')


def available():
    return bool(REFERENCE_ROOT) and os.path.exists(
        os.path.join(REFERENCE_ROOT, 'crowddynamics', 'core', 'interactions.py'))


class _Inert:
    """Stand-in for numba type objects: indexable and callable."""

    def __getitem__(self, item):
        return self

    def __call__(self, *args, **kwargs):
        return self


def _make_numba():
    nb = types.ModuleType('numba')

    def jit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    def vectorize(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    class Float:
        pass

    class Array:
        pass

    def generated_jit(*args, **kwargs):
        def deco(gen):
            def dispatch(x):
                t = Float() if np.ndim(x) == 0 else Array()
                return gen(t)(x)
            return dispatch
        if len(args) == 1 and callable(args[0]):
            return deco(args[0])
        return deco

    nb.jit = jit
    nb.njit = jit
    nb.vectorize = vectorize
    nb.generated_jit = generated_jit
    for name in ('f8', 'i8', 'void', 'float64', 'int64', 'boolean', 'b1', 'optional'):
        setattr(nb, name, _Inert())
    nb.typeof = lambda x: _Inert()
    tys = types.ModuleType('numba.types')
    tys.Tuple = _Inert()
    tys.UniTuple = _Inert()
    tys.f8 = _Inert()
    tys.boolean = _Inert()
    tys.Float = Float
    tys.Array = Array
    nb.types = tys
    return nb, tys


class CellGrid:
    """Grid used by the stub cell_lists: origin, cell size and shape."""
    x0 = 0.0
    y0 = 0.0
    cell = 1.0
    nx = 1
    ny = 1


def _make_cell_lists():
    cl = types.ModuleType('cell_lists')
    g = CellGrid

    def _axis(v, v0, n):
        q = np.floor((v - v0) / g.cell)
        return int(min(max(q, 0.0), n - 1))

    def add_to_cells(points, cell_size):
        assert cell_size == g.cell, 'configure CellGrid.cell to the cell size'
        n = len(points)
        keys = np.empty(n, np.int64)
        for i in range(n):
            x, y = points[i][0], points[i][1]
            if not (np.isfinite(x) and np.isfinite(y)):
                raise ValueError('non-finite position')
            keys[i] = _axis(x, g.x0, g.nx) * g.ny + _axis(y, g.y0, g.ny)
        ncells = g.nx * g.ny
        cells_count = np.bincount(keys, minlength=ncells).astype(np.int64)
        cells_offset = np.zeros(ncells, np.int64)
        cells_offset[1:] = np.cumsum(cells_count)[:-1]
        points_indices = np.argsort(keys, kind='stable').astype(np.int64)
        return points_indices, cells_count, cells_offset, np.array((g.nx, g.ny))

    def neighboring_cells(grid_shape):
        # forward half of the 3x3 stencil, ascending flat offset
        return np.array([(0, 1), (1, -1), (1, 0), (1, 1)], dtype=np.int64)

    def iter_nearest_neighbors(cell_indices, neigh_cells, points_indices,
                               cells_count, cells_offset):
        for c in cell_indices:
            ix, iy = divmod(int(c), g.ny)
            s0, cnt = cells_offset[c], cells_count[c]
            for s in range(cnt):
                a = points_indices[s0 + s]
                for t in range(s + 1, cnt):
                    yield a, points_indices[s0 + t]
                for dx, dy in neigh_cells:
                    jx, jy = ix + dx, iy + dy
                    if not (0 <= jx < g.nx and 0 <= jy < g.ny):
                        continue
                    c2 = jx * g.ny + jy
                    for t in range(cells_count[c2]):
                        yield a, points_indices[cells_offset[c2] + t]

    cl.add_to_cells = add_to_cells
    cl.neighboring_cells = neighboring_cells
    cl.iter_nearest_neighbors = iter_nearest_neighbors
    return cl


def _make_agents_module():
    # local import keeps the restated dtype definition in one place
    from crowddynamics_gb300.simulation import agents as A
    m = types.ModuleType('crowddynamics.simulation.agents')
    m.agent_type_circular = A.agent_type_circular
    m.agent_type_three_circle = A.agent_type_three_circle
    m.AgentModelToType = A.AgentModelToType
    m.is_model = A.is_model
    m.NO_TARGET = -1                  # simulation/agents.py:27-28
    m.NO_LEADER = -1

    def shoulders(agents):
        # simulation/agents.py:482-486, element by element
        vector2D = m.vector2D
        for agent in agents:
            tangent = vector2D.rotate270(vector2D.unit_vector(agent['orientation']))
            offset = tangent * agent['r_ts']
            agent['position_ls'][:] = agent['position'] - offset
            agent['position_rs'][:] = agent['position'] + offset

    m.shoulders = shoulders
    return m


_FILES = [
    ('crowddynamics.core.vector2D', 'crowddynamics/core/vector2D.py'),
    ('crowddynamics.core.structures', 'crowddynamics/core/structures.py'),
    ('crowddynamics.exceptions', 'crowddynamics/exceptions.py'),
    ('crowddynamics.core.distance', 'crowddynamics/core/distance.py'),
    ('crowddynamics.core.motion.contact', 'crowddynamics/core/motion/contact.py'),
    ('crowddynamics.core.motion.power_law', 'crowddynamics/core/motion/power_law.py'),
    ('crowddynamics.core.motion.adjusting', 'crowddynamics/core/motion/adjusting.py'),
    ('crowddynamics.core.integrator', 'crowddynamics/core/integrator.py'),
    ('crowddynamics.core.interactions', 'crowddynamics/core/interactions.py'),
    ('crowddynamics.core.steering.orientation', 'crowddynamics/core/steering/orientation.py'),
    ('crowddynamics.core.geom2D', 'crowddynamics/core/geom2D.py'),
    ('crowddynamics.core.sensory_region', 'crowddynamics/core/sensory_region.py'),
    ('crowddynamics.core.steering.collective_motion',
     'crowddynamics/core/steering/collective_motion.py'),
    ('crowddynamics.core.evacuation', 'crowddynamics/core/evacuation.py'),
]

_loaded = {}


def _libm_numpy():
    """A stand-in for ``numpy`` in the reference modules that evaluates the
    elementary functions as numba's compiled code does: on float64 scalars,
    numba lowers ``np.exp``, ``np.sin``, ``np.cos`` and ``np.arctan2`` to the
    C library's ``exp``, ``sin``, ``cos`` and ``atan2``, and ``np.hypot`` to
    its ``hypot`` (numba's math implementation calls the platform function).
    numpy's own loops for exp, hypot and arctan2 round differently from the C
    library in a few percent of calls, which chaos amplifies to millimetres
    over tens of steps.  Everything else is numpy itself."""
    import ctypes
    import ctypes.util
    libm = ctypes.CDLL(ctypes.util.find_library('m'))
    proxy = types.ModuleType('numpy')
    proxy.__dict__.update(np.__dict__)

    def wrap(cfn, nargs):
        cfn.restype = ctypes.c_double
        cfn.argtypes = [ctypes.c_double] * nargs
        vec = np.vectorize(lambda *a: cfn(*a), otypes=[np.float64])

        def f(*args):
            if all(np.ndim(a) == 0 for a in args):
                return np.float64(cfn(*(float(a) for a in args)))
            return vec(*args)
        return f

    proxy.exp = wrap(libm.exp, 1)
    proxy.sin = wrap(libm.sin, 1)
    proxy.cos = wrap(libm.cos, 1)
    proxy.arctan2 = wrap(libm.atan2, 2)
    proxy.hypot = wrap(libm.hypot, 2)
    return proxy


def _numba_ipow(a, n):
    """``a ** n`` for a literal integer n as numba lowers it: exponentiation
    by squaring from 1 (so a ** 2 is exactly a * a), the reciprocal for
    n < 0.  CPython evaluates a float ** 2 with the C library's pow, which
    differs from a * a in about one case in a thousand."""
    one = 1.0 if isinstance(a, (float, np.floating)) else 1
    r, e = one, abs(n)
    while e:
        if e & 1:
            r = r * a
        e >>= 1
        if e:
            a = a * a
    return one / r if n < 0 else r


class _PowLowering(__import__('ast').NodeTransformer):
    """Rewrites ``x ** k`` with an integer literal k into _numba_ipow(x, k)."""

    def visit_BinOp(self, node):
        import ast
        self.generic_visit(node)
        if isinstance(node.op, ast.Pow):
            k = node.right
            neg = isinstance(k, ast.UnaryOp) and isinstance(k.op, ast.USub)
            lit = k.operand if neg else k
            if isinstance(lit, ast.Constant) and type(lit.value) is int:
                call = ast.Call(func=ast.Name('_numba_ipow', ast.Load()),
                                args=[node.left, ast.Constant(-lit.value if neg else lit.value)],
                                keywords=[])
                return ast.copy_location(call, node)
        return node


def _exec_numba_semantics(mod, path):
    """Execute a reference file in `mod` with numba's lowering of literal
    integer powers (the source itself is read unchanged)."""
    import ast
    tree = ast.parse(open(path).read(), path)
    tree = ast.fix_missing_locations(_PowLowering().visit(tree))
    mod.__dict__['_numba_ipow'] = _numba_ipow
    exec(compile(tree, path, 'exec'), mod.__dict__)


def load(math='numpy'):
    """Load the reference hot-path modules; returns a namespace of them.

    ``math='numpy'`` runs them as CPython executes them (numpy's elementary
    functions, the C library's pow for ``x ** 2``); ``math='libm'`` runs them
    with numba's scalar semantics: the C library's elementary functions (see
    _libm_numpy) and literal integer powers as multiplications (see
    _numba_ipow).  The stubs are installed only for
    the duration of the load and the loaded modules keep references to them,
    so other imports are unaffected.
    """
    if math in _loaded:
        return _loaded[math]
    if math not in ('numpy', 'libm'):
        raise ValueError(math)
    if not available():
        raise RuntimeError('reference source tree not found at ' + REFERENCE_ROOT)
    nb, tys = _make_numba()
    traitlets = types.ModuleType('traitlets')
    traitlets.TraitError = type('TraitError', (Exception,), {})
    typing_mod = types.ModuleType('numba.typing')
    typeof_mod = types.ModuleType('numba.typing.typeof')
    typeof_mod.typeof = lambda x: _Inert()
    typing_mod.typeof = typeof_mod
    stubs = {
        'numba': nb, 'numba.types': tys, 'traitlets': traitlets,
        'numba.typing': typing_mod, 'numba.typing.typeof': typeof_mod,
        'cell_lists': _make_cell_lists(),
    }
    for pkg in ('crowddynamics', 'crowddynamics.core', 'crowddynamics.core.motion',
                'crowddynamics.core.steering', 'crowddynamics.simulation'):
        p = types.ModuleType(pkg)
        p.__path__ = []
        stubs[pkg] = p
    stubs['crowddynamics.simulation.agents'] = _make_agents_module()
    saved = {k: sys.modules.get(k) for k in list(stubs) + [n for n, _ in _FILES]}
    np_libm = _libm_numpy() if math == 'libm' else None
    sys.modules.update(stubs)
    ns = types.SimpleNamespace()
    try:
        for name, rel in _FILES:
            spec = importlib.util.spec_from_file_location(
                name, os.path.join(REFERENCE_ROOT, rel))
            mod = importlib.util.module_from_spec(spec)
            sys.modules[name] = mod
            if math == 'libm':
                _exec_numba_semantics(mod, os.path.join(REFERENCE_ROOT, rel))
                if hasattr(mod, 'np'):
                    mod.np = np_libm
            else:
                spec.loader.exec_module(mod)
            setattr(ns, name.rsplit('.', 1)[-1], mod)
            if name == 'crowddynamics.core.vector2D':
                stubs['crowddynamics.simulation.agents'].vector2D = mod
        ns.agents_module = stubs['crowddynamics.simulation.agents']
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    if math == 'libm':
        ns.agents_module.np = np_libm
    ns.grid = CellGrid
    _loaded[math] = ns
    return ns


def _extract(rel, names, ns):
    """Execute the top-level definitions ``names`` of a reference file (parsed
    unchanged, other statements and imports left out) in ``ns``."""
    import ast
    path = os.path.join(REFERENCE_ROOT, rel)
    tree = ast.parse(open(path).read(), path)
    body = [n for n in tree.body
            if (isinstance(n, ast.FunctionDef) and n.name in names) or
            (isinstance(n, ast.Assign) and
             any(isinstance(t, ast.Name) and t.id in names for t in n.targets))]
    missing = set(names) - {getattr(n, 'name', None) or n.targets[0].id for n in body}
    if missing:
        raise RuntimeError('not found in %s: %s' % (rel, sorted(missing)))
    exec(compile(ast.Module(body=body, type_ignores=[]), path, 'exec'), ns)


_nav = None


def load_navigation():
    """The reference's navigation lookup: ``meshgrid`` (with its indicer) from
    core/steering/quickest_path.py:22-49 and ``is_inside`` / ``getdefault``
    from core/steering/navigation.py:59-78.  Their modules import fast
    marching, shapely and skimage, absent here, so only these definitions are
    executed (with the numba stub)."""
    global _nav
    if _nav is not None:
        return _nav
    if not available():
        raise RuntimeError('reference source tree not found at ' + REFERENCE_ROOT)
    import typing
    nb, _ = _make_numba()
    ns = {'np': np, 'numba': nb, 'f8': nb.f8, 'i8': nb.i8, 'NamedTuple': typing.NamedTuple,
          'Callable': typing.Callable, 'Tuple': typing.Tuple, 'Optional': typing.Optional}
    _extract('crowddynamics/core/steering/quickest_path.py', ('MeshGrid', 'meshgrid'), ns)
    _extract('crowddynamics/core/steering/navigation.py', ('is_inside', 'getdefault'), ns)
    _nav = types.SimpleNamespace(meshgrid=ns['meshgrid'], getdefault=ns['getdefault'],
                                 is_inside=ns['is_inside'])
    return _nav


def navigation(agents, dir_maps, step, bounds):
    """Navigation.update (simulation/logic.py:152-165) with the reference's own
    meshgrid indicer and getdefault, for precomputed maps: ``dir_maps`` is a
    list of (dir_x, dir_y) per target on ``meshgrid(step, *bounds)``."""
    nav = load_navigation()
    mgrid = nav.meshgrid(step, *bounds)
    for target in range(len(dir_maps)):
        has_target = agents['target'] == target
        if not has_target.size:
            continue
        indices = np.fliplr(mgrid.indicer(agents[has_target]['position']))
        new_direction = nav.getdefault(indices, dir_maps[target],
                                       agents[has_target]['target_direction'])
        agents['target_direction'][has_target] = new_direction
    return mgrid


def configure_grid(x0, y0, cell, nx, ny):
    CellGrid.x0, CellGrid.y0, CellGrid.cell = float(x0), float(y0), float(cell)
    CellGrid.nx, CellGrid.ny = int(nx), int(ny)


def step(agents, cell_size, walls=None, noise_f=None, noise_m=None,
         dt_min=0.001, dt_max=0.01, nodes=('fluctuation', 'orientation', 'adjusting',
                                           'agent_agent', 'agent_obstacle',
                                           'integrate', 'reset'), math='numpy'):
    """One update() of the standard tree with the reference's own functions
    (node bodies restated from simulation/logic.py:59-130,258-261)."""
    R = load(math)
    three = R.agents_module.is_model(agents, 'three_circle')
    dt = 0.0
    if 'fluctuation' in nodes and noise_f is not None:
        agents['force'] += noise_f
        if three and noise_m is not None:
            agents['torque'] += noise_m
    if 'orientation' in nodes and three:
        R.orientation.orient_towards_target_direction(agents)
    if 'adjusting' in nodes:
        R.adjusting.force_adjust_agents(agents)
        if three:
            R.adjusting.torque_adjust_agents(agents)
    if 'agent_agent' in nodes:
        R.interactions.agent_agent_block_list(agents, cell_size)
    if 'agent_obstacle' in nodes:
        from crowddynamics_gb300.core.structures import obstacle_type_linear
        obs = np.zeros(0, obstacle_type_linear) if walls is None else walls
        R.interactions.agent_obstacle(agents, obs)
    if 'integrate' in nodes:
        dt = R.integrator.velocity_verlet_integrator(agents, dt_min, dt_max)
    if 'reset' in nodes:
        agents['force'] = 0
        if three:
            agents['torque'] = 0
    return dt
