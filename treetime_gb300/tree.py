"""Rooted trees with the traversal interface TreeTime relies on.

``Clade`` and ``Tree`` expose the Bio.Phylo.BaseTree calls that the
reconstruction path uses (find_clades with 'preorder' / 'postorder' / 'level',
get_terminals, get_nonterminals, count_terminals, ladderize,
total_branch_length, is_terminal, iteration over children), with Biopython's
documented order semantics: preorder is depth-first with children in list
order, postorder visits children first, ladderize is a stable ascending sort
of each clade's children by their number of tips.  Node order fixes internal
node names and so it is part of the output contract.

All traversals are iterative, so caterpillar trees with many thousands of
levels do not hit Python's recursion limit.  Any object with the same
attributes (for instance a real Bio.Phylo tree) works wherever a ``Tree`` is
accepted.
"""

import io
import operator
import os


def _iter_preorder(root):
    stack = [root]
    while stack:
        node = stack.pop()
        yield node
        ch = node.clades
        for i in range(len(ch) - 1, -1, -1):
            stack.append(ch[i])


def _iter_postorder(root):
    stack = [(root, False)]
    while stack:
        node, expanded = stack.pop()
        if expanded or not node.clades:
            yield node
        else:
            stack.append((node, True))
            ch = node.clades
            for i in range(len(ch) - 1, -1, -1):
                stack.append((ch[i], False))


def _iter_level(root):
    queue = [root]
    i = 0
    while i < len(queue):
        node = queue[i]
        i += 1
        yield node
        queue.extend(node.clades)


_ORDERS = {"preorder": _iter_preorder, "postorder": _iter_postorder, "level": _iter_level}


def iter_clades(root, order="preorder"):
    """Traverse any duck-typed clade (``.clades`` lists) in the given order."""
    return _ORDERS[order](root)


class _Traversal:
    def _start(self):
        raise NotImplementedError

    def find_clades(self, target=None, terminal=None, order="preorder"):
        for node in _ORDERS[order](self._start()):
            if terminal is not None and (not node.clades) != terminal:
                continue
            if target is not None:
                if isinstance(target, str):
                    if node.name != target:
                        continue
                elif callable(target):
                    if not target(node):
                        continue
            yield node

    def get_terminals(self, order="preorder"):
        return [c for c in _ORDERS[order](self._start()) if not c.clades]

    def get_nonterminals(self, order="preorder"):
        return [c for c in _ORDERS[order](self._start()) if c.clades]

    def count_terminals(self):
        return sum(1 for c in _iter_preorder(self._start()) if not c.clades)

    def total_branch_length(self):
        return sum(c.branch_length for c in _iter_preorder(self._start()) if c.branch_length)

    def ladderize(self, reverse=False):
        """Stable sort of every clade's children by number of tips."""
        ntips = {}
        for node in _iter_postorder(self._start()):
            if node.clades:
                node.clades.sort(key=lambda c: ntips[id(c)], reverse=reverse)
                ntips[id(node)] = sum(ntips[id(c)] for c in node.clades)
            else:
                ntips[id(node)] = 1


# Per-node results of a reconstruction, read from the device results of the
# latest reconstruction (anc_gpu.ResultStore) when first accessed.
LAZY_ATTRS = ("_cseq", "marginal_profile", "marginal_subtree_LH", "marginal_outgroup_LH", "branch_state")


class _Result:
    """Data descriptor of one per-node result.  A clade of a reconstruction
    session holds the session's result holder in ``_anc_src``; reading the
    attribute asks the holder (which answers from the latest reconstruction),
    so installing a new reconstruction is one assignment for the whole tree
    instead of a walk over its nodes.  A value assigned to the attribute
    overrides the holder's until the next reconstruction (the holder is told,
    and clears the overrides it was told of), as TreeTime's next
    reconstruction overwrites what was assigned before."""

    def __init__(self, name):
        self.name = name

    def __get__(self, node, owner=None):
        if node is None:
            return self
        d = node.__dict__
        ov = d.get("_anc_override")
        if ov is not None and self.name in ov:
            return ov[self.name]
        src = d.get("_anc_src")
        if src is not None:
            val = src.fetch(self.name, node)
            if val is not None:
                return val
        raise AttributeError(self.name)

    def __set__(self, node, value):
        d = node.__dict__
        ov = d.get("_anc_override")
        if ov is None:
            ov = d["_anc_override"] = {}
        ov[self.name] = value
        src = d.get("_anc_src")
        if src is not None and hasattr(src, "overridden"):
            src.overridden(node)

    def __delete__(self, node):
        ov = node.__dict__.get("_anc_override")
        if not ov or self.name not in ov:
            raise AttributeError(self.name)
        del ov[self.name]


# Bumped by every change to a Clade's children or mask: a mutation of a children list, a new list
# or a new or deleted mask.  A device session built from a tree of these clades stays valid while
# the epoch has not moved (an O(1) check per call instead of a walk over the tree); any change,
# to any tree, sends the next call through the full check.
_EPOCH = [0]


def topology_epoch():
    """The current value of the change counter of Clade children and masks."""
    return _EPOCH[0]


# Bumped by every assignment of a Clade's branch length: a session whose device copy of the
# lengths was made at the current value needs neither the walk over the nodes that reads them
# nor the upload.
_BL_EPOCH = [0]


def length_epoch():
    """The current value of the change counter of Clade branch lengths."""
    return _BL_EPOCH[0]


def assign_lengths(dicts, lengths, dist2root=None):
    """New branch lengths for many Clades, given their ``__dict__``s, with one
    bump of the change counter (the caller then owns keeping any device copy
    in step): branch_length and mutation_length take the length, dist2root the
    given distance.  One loop of dictionary stores, ~25 ns a value, where three
    loops of attribute assignments cost ~75 ns a value."""
    _BL_EPOCH[0] += 1
    if dist2root is None:
        for d, v in zip(dicts, lengths):
            d["_branch_length"] = v
            d["mutation_length"] = v
    else:
        for d, v, r in zip(dicts, lengths, dist2root):
            d["_branch_length"] = v
            d["mutation_length"] = v
            d["dist2root"] = r


class _Children(list):
    """A Clade's list of children: every mutation bumps the change counter."""

    __slots__ = ()

    def __setitem__(self, i, v):
        _EPOCH[0] += 1
        list.__setitem__(self, i, v)

    def __delitem__(self, i):
        _EPOCH[0] += 1
        list.__delitem__(self, i)

    def __iadd__(self, other):
        _EPOCH[0] += 1
        list.extend(self, other)
        return self

    def __imul__(self, n):
        _EPOCH[0] += 1
        return list.__imul__(self, n)

    def append(self, v):
        _EPOCH[0] += 1
        list.append(self, v)

    def extend(self, it):
        _EPOCH[0] += 1
        list.extend(self, it)

    def insert(self, i, v):
        _EPOCH[0] += 1
        list.insert(self, i, v)

    def remove(self, v):
        _EPOCH[0] += 1
        list.remove(self, v)

    def pop(self, *i):
        _EPOCH[0] += 1
        return list.pop(self, *i)

    def clear(self):
        _EPOCH[0] += 1
        list.clear(self)

    def sort(self, *args, **kwargs):
        _EPOCH[0] += 1
        list.sort(self, *args, **kwargs)

    def reverse(self):
        _EPOCH[0] += 1
        list.reverse(self)


def _set_clades(node, value):
    _EPOCH[0] += 1
    node.__dict__["_clades"] = value if type(value) is _Children else _Children(value)


def _set_branch_length(node, value):
    _BL_EPOCH[0] += 1
    node.__dict__["_branch_length"] = value


def _get_mask(node):
    try:
        return node.__dict__["mask"]
    except KeyError:
        raise AttributeError("mask") from None


def _set_mask(node, value):
    _EPOCH[0] += 1
    node.__dict__["mask"] = value


def _del_mask(node):
    _EPOCH[0] += 1
    try:
        del node.__dict__["mask"]
    except KeyError:
        raise AttributeError("mask") from None


class Clade(_Traversal):
    # children, mask and branch length go through the change counters; the reads of `clades` and
    # `branch_length` are C-level getters
    clades = property(operator.attrgetter("_clades"), _set_clades)
    mask = property(_get_mask, _set_mask, _del_mask)
    branch_length = property(operator.attrgetter("_branch_length"), _set_branch_length)

    def __init__(self, branch_length=None, name=None, clades=None, confidence=None):
        self.branch_length = branch_length
        self.name = name
        self.clades = list(clades) if clades else []
        self.confidence = confidence

    def _start(self):
        return self

    @property
    def cseq(self):
        """Compressed sequence: the alignment for tips (unless tip states were
        reconstructed), the reconstruction otherwise (treetime/treeanc.py:14-24)."""
        tt = self.__dict__.get("tt")
        if tt is not None and tt.data is not None and self.name in tt.data.name_to_row \
                and not tt.reconstructed_tip_sequences:
            return tt.data.compressed_alignment[self.name]
        try:
            return self._cseq
        except AttributeError:
            if not self.clades:
                return None
            raise ValueError("Ancestral sequences are not yet inferred")

    @property
    def sequence(self):
        return self.tt.sequence(self, as_string=False)

    @property
    def mutations(self):
        """(ancestral, position, derived) list of the branch above this node
        (treetime/treeanc.py:27-42)."""
        tt = self.tt
        up = self.__dict__.get("up")
        if up is None:
            return []
        mask = self.__dict__.get("mask")
        if not tt.reconstructed_tip_sequences and self.name in tt.data.name_to_row:
            return tt.data.differences(up.cseq, tt.data.aln[self.name], seq2_compressed=False, mask=mask)
        if not self.clades and self.name not in tt.data.name_to_row:
            return []
        return tt.data.differences(up.cseq, self.cseq, mask=mask)

    def is_terminal(self):
        return not self.clades

    def __iter__(self):
        return iter(self.clades)

    def __len__(self):
        return len(self.clades)

    _cseq = _Result("_cseq")
    marginal_profile = _Result("marginal_profile")
    marginal_subtree_LH = _Result("marginal_subtree_LH")
    marginal_outgroup_LH = _Result("marginal_outgroup_LH")
    branch_state = _Result("branch_state")

    def __getitem__(self, i):
        return self.clades[i]

    def __repr__(self):
        return "Clade(name=%r, branch_length=%r)" % (self.name, self.branch_length)


class Tree(_Traversal):
    def __init__(self, root=None, rooted=True, name=None):
        self.root = root if root is not None else Clade()
        self.rooted = rooted
        self.name = name

    def _start(self):
        return self.root

    @property
    def clade(self):
        return self.root

    def is_terminal(self):
        return not self.root.clades

    def __iter__(self):
        return iter(self.root.clades)


# --------------------------------------------------------------------------
# Newick I/O
# --------------------------------------------------------------------------

def _is_number(s):
    try:
        float(s)
        return True
    except ValueError:
        return False


def parse_newick(text):
    """Parse one Newick tree.  A label after ')' that parses as a number is a
    support value (``confidence``), otherwise the clade name, as in
    Bio.Phylo's Newick reader."""
    root = Clade()
    stack = []
    cur = root
    i, n = 0, len(text)
    expect_len = False
    after_close = False
    while i < n:
        ch = text[i]
        if ch == "(":
            child = Clade()
            cur.clades.append(child)
            stack.append(cur)
            cur = child
            after_close = False
            i += 1
        elif ch == ",":
            if not stack:
                raise ValueError("malformed Newick: ',' at top level")
            child = Clade()
            stack[-1].clades.append(child)
            cur = child
            after_close = False
            expect_len = False
            i += 1
        elif ch == ")":
            if not stack:
                raise ValueError("malformed Newick: unbalanced ')'")
            cur = stack.pop()
            after_close = True
            expect_len = False
            i += 1
        elif ch == ":":
            expect_len = True
            i += 1
        elif ch == ";":
            break
        elif ch == "[":
            j = text.find("]", i)
            i = n if j < 0 else j + 1
        elif ch.isspace():
            i += 1
        else:
            if ch == "'":
                j = text.index("'", i + 1)
                tok = text[i + 1:j]
                i = j + 1
            else:
                j = i
                while j < n and text[j] not in "(),:;[" and not text[j].isspace():
                    j += 1
                tok = text[i:j]
                i = j
            if expect_len:
                cur.branch_length = float(tok)
                expect_len = False
            elif after_close and _is_number(tok):
                cur.confidence = float(tok)
            else:
                cur.name = tok
    if stack:
        raise ValueError("malformed Newick: unbalanced '('")
    return Tree(root=root, rooted=False)


def read_newick(source):
    """Tree from a Newick string, a file name or an open file."""
    if hasattr(source, "read"):
        return parse_newick(source.read())
    if isinstance(source, str) and os.path.isfile(source):
        with open(source) as fh:
            return parse_newick(fh.read())
    if isinstance(source, str) and source.strip().endswith(";"):
        return parse_newick(source)
    raise ValueError("not a Newick string or file: %r" % (source[:80] if isinstance(source, str) else source))


def to_newick(tree, precision=None):
    """Newick text of a tree (iterative, no recursion limit)."""
    out = io.StringIO()
    root = tree.root if hasattr(tree, "root") else tree
    fmt = (lambda x: repr(float(x))) if precision is None else (lambda x: ("%." + str(precision) + "g") % x)
    # explicit stack of (node, state): state 0 = open, 1 = close
    stack = [(root, 0)]
    parts = []
    while stack:
        node, state = stack.pop()
        if state == 0:
            if node.clades:
                parts.append("(")
                stack.append((node, 1))
                for k in range(len(node.clades) - 1, -1, -1):
                    stack.append((node.clades[k], 0))
                    if k > 0:
                        stack.append((None, 2))
            else:
                parts.append(_label(node, fmt))
        elif state == 1:
            parts.append(")" + _label(node, fmt))
        else:
            parts.append(",")
    out.write("".join(parts) + ";")
    return out.getvalue()


def _label(node, fmt):
    s = node.name or ""
    if node.branch_length is not None:
        s += ":" + fmt(node.branch_length)
    return s
