"""Logic-node tree (``crowddynamics/simulation/base.py:27-84``).

The reference builds its trees on anytree's ``NodeMixin``; this restates the
parts the simulation uses -- ``parent``/``children``, ``<<``,
``inject_before``/``inject_after``, name lookup and post-order traversal --
without the dependency.  ``a << b`` adds ``b`` as a child of ``a`` and
returns ``a``, so ``Reset << InsideDomain << (Integrator << (...))`` makes
``InsideDomain`` and ``Integrator`` both children of ``Reset`` as in the
reference (``simulation/tests/test_base.py:13-19``).
"""


class LogicNodeBase:
    """Node of the simulation's logic tree."""

    def __init__(self, name=None):
        self._parent = None
        self._children = []
        self.name = name or self.__class__.__name__

    @property
    def parent(self):
        return self._parent

    @parent.setter
    def parent(self, node):
        if self._parent is not None:
            self._parent._children.remove(self)
        self._parent = node
        if node is not None:
            node._children.append(self)

    @property
    def children(self):
        return tuple(self._children)

    @property
    def root(self):
        n = self
        while n._parent is not None:
            n = n._parent
        return n

    def update(self):
        """Called when the node is evaluated."""
        raise NotImplementedError

    def inject_before(self, node):
        """Insert ``node`` between this node and its parent."""
        parent = self.parent
        self.parent = node
        node.parent = parent

    def inject_after(self, node):
        """Move this node's children under ``node`` and make ``node`` a child."""
        for child in self.children:
            child.parent = node
        node.parent = self

    def add_children(self, node):
        node.parent = self
        return self

    def __lshift__(self, other):
        if isinstance(other, LogicNodeBase):
            self.add_children(other)
        else:
            for o in other:
                self.add_children(o)
        return self

    def __repr__(self):
        return self.name

    def __getitem__(self, item):
        for node in pre_order(self.root):
            if node.name == item:
                return node
        raise KeyError('no node named %r in this logic tree' % (item,))


def pre_order(node):
    yield node
    for c in node.children:
        yield from pre_order(c)


def post_order(node):
    """anytree.PostOrderIter: children (in order) before their parent."""
    for c in node.children:
        yield from post_order(c)
    yield node
