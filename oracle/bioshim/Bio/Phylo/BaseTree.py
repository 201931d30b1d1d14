"""Minimal Bio.Phylo.BaseTree stand-in (test-only).

Semantics kept from Biopython's documentation:
  * find_clades(order='preorder') is depth-first, node before its children,
    children in list order; 'postorder' visits children first; 'level' is
    breadth-first.  The default yields every clade.
  * get_terminals / get_nonterminals follow the same order argument.
  * ladderize(reverse=False) sorts each clade's children by count_terminals()
    with a stable sort, recursively.
  * Iterating a Clade yields its direct children.
"""


def _iter_preorder(root):
    stack = [root]
    while stack:
        node = stack.pop()
        yield node
        stack.extend(reversed(node.clades))


def _iter_postorder(root):
    stack = [(root, False)]
    while stack:
        node, expanded = stack.pop()
        if expanded or not node.clades:
            yield node
        else:
            stack.append((node, True))
            stack.extend((c, False) for c in reversed(node.clades))


def _iter_level(root):
    queue = [root]
    i = 0
    while i < len(queue):
        node = queue[i]
        i += 1
        yield node
        queue.extend(node.clades)


_ORDERS = {"preorder": _iter_preorder, "postorder": _iter_postorder, "level": _iter_level}


class TreeMixin:
    def _root_clade(self):
        return self.root if isinstance(self, Tree) else self

    def find_clades(self, target=None, terminal=None, order="preorder"):
        it = _ORDERS[order](self._root_clade())
        for node in it:
            if terminal is not None and node.is_terminal() != terminal:
                continue
            if target is not None:
                if isinstance(target, str) and node.name != target:
                    continue
                if callable(target) and not target(node):
                    continue
            yield node

    def get_terminals(self, order="preorder"):
        return [c for c in self.find_clades(order=order) if c.is_terminal()]

    def get_nonterminals(self, order="preorder"):
        return [c for c in self.find_clades(order=order) if not c.is_terminal()]

    def count_terminals(self):
        return sum(1 for c in self.find_clades() if c.is_terminal())

    def total_branch_length(self):
        return sum(c.branch_length for c in self.find_clades() if c.branch_length)

    def ladderize(self, reverse=False):
        for node in _iter_postorder(self._root_clade()):
            if node.clades:
                counts = {id(c): c.count_terminals() for c in node.clades}
                node.clades.sort(key=lambda c: counts[id(c)], reverse=reverse)

    def is_terminal(self):
        return self._root_clade().is_terminal()


class Clade(TreeMixin):
    def __init__(self, branch_length=None, name=None, clades=None, confidence=None, **kwargs):
        self.branch_length = branch_length
        self.name = name
        self.clades = list(clades or [])
        self.confidence = confidence

    def is_terminal(self):
        return not self.clades

    def __iter__(self):
        return iter(self.clades)

    def __len__(self):
        return len(self.clades)

    def __getitem__(self, i):
        return self.clades[i]

    def __repr__(self):
        return "Clade(name=%r, branch_length=%r)" % (self.name, self.branch_length)


class Tree(TreeMixin):
    def __init__(self, root=None, rooted=True, name=None):
        self.root = root if root is not None else Clade()
        self.rooted = rooted
        self.name = name

    @property
    def clade(self):
        return self.root

    def __iter__(self):
        return iter(self.root.clades)
