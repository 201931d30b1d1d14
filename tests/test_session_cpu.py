"""The session cache's change detection (host logic, no GPU): a device
session is reused only while every node keeps the same children, in the same
order, and the same mask objects; anything else rebuilds it."""

from treetime_gb300.anc_gpu import _children, _masks, _same_children, _same_masks
from treetime_gb300.tree import Clade, parse_newick


def _nodes(tree):
    return list(tree.find_clades())


def test_unchanged_tree_matches():
    t = parse_newick("((A:0.1,B:0.2)x:0.05,(C:0.1,D:0.1)y:0.2,E:0.3)r;")
    nodes = _nodes(t)
    ch, ms = _children(nodes), _masks(nodes)
    assert _same_children(nodes, ch)
    assert _same_masks(nodes, ms)
    # branch lengths are not part of the check (they are refreshed on every call)
    nodes[1].branch_length = 0.7
    assert _same_children(nodes, ch)


def test_topology_changes_are_seen():
    t = parse_newick("((A:0.1,B:0.2)x:0.05,(C:0.1,D:0.1)y:0.2,E:0.3)r;")
    nodes = _nodes(t)
    ch = _children(nodes)
    x = next(n for n in nodes if n.name == "x")
    # a child gained (the list grows past the reference)
    x.clades.append(Clade(name="F", branch_length=0.1))
    assert not _same_children(nodes, ch)
    x.clades.pop()
    assert _same_children(nodes, ch)
    # a child lost (the list ends early)
    gone = x.clades.pop()
    assert not _same_children(nodes, ch)
    x.clades.append(gone)
    assert _same_children(nodes, ch)
    # children reordered
    x.clades.reverse()
    assert not _same_children(nodes, ch)
    x.clades.reverse()
    # a child replaced by another object with the same name
    x.clades[0] = Clade(name=x.clades[0].name, branch_length=0.1)
    assert not _same_children(nodes, ch)


def test_mask_changes_are_seen():
    t = parse_newick("((A:0.1,B:0.2)x:0.05,C:0.3)r;")
    nodes = _nodes(t)
    ms = _masks(nodes)
    nodes[2].mask = [1.0, 0.0]
    assert not _same_masks(nodes, ms)
    ms = _masks(nodes)
    assert _same_masks(nodes, ms)
    nodes[2].mask = [1.0, 0.0]  # an equal but new mask object
    assert not _same_masks(nodes, ms)


def test_dist2root_by_levels_equals_the_preorder_sums():
    """The distances to the root that optimize_branch_lengths_joint sets after
    new lengths are the sums of TreeTime's _calc_dist2root
    (treetime/treeanc.py:499-510), bit for bit."""
    import numpy as np
    from treetime_gb300 import engine, synth
    from treetime_gb300.anc_gpu import _set_dist2root
    from treetime_gb300.tree import iter_clades
    tree = synth.coalescent_tree(300, 0.01, np.random.default_rng(3))
    lay = engine.TreeLayout(tree.root)
    lengths = np.random.default_rng(4).random(lay.n_nodes) * 0.01
    lengths[lay.n_int - 1] = 0.0
    for n, v in zip(lay.nodes, lengths.tolist()):
        n.mutation_length = v
    _set_dist2root(lay, lengths)
    fast = [n.dist2root for n in lay.nodes]
    lay.root.dist2root = 0.0
    for c in iter_clades(lay.root):
        for ch in c.clades:
            ch.dist2root = c.dist2root + ch.mutation_length
    assert fast == [n.dist2root for n in lay.nodes]


def test_change_counter_moves_on_every_change_and_only_then():
    """The O(1) session check: the counter moves on any mutation of a children
    list, a new list, a new or deleted mask, and not on reads or on other
    attributes (branch lengths have their own counter)."""
    from treetime_gb300.tree import topology_epoch
    t = parse_newick("((A:0.1,B:0.2)x:0.05,C:0.3)r;")
    x = next(n for n in t.find_clades() if n.name == "x")
    e = topology_epoch()
    _ = [n.clades for n in t.find_clades()], getattr(x, "mask", None)
    x.branch_length = 0.9
    x.name = "y"
    assert topology_epoch() == e
    for change in (lambda: x.clades.append(Clade(name="D")), lambda: x.clades.pop(),
                   lambda: x.clades.reverse(), lambda: x.clades.sort(key=lambda c: c.name),
                   lambda: x.clades.insert(0, Clade(name="E")), lambda: x.clades.remove(x.clades[0]),
                   lambda: x.clades.__setitem__(0, x.clades[0]), lambda: x.clades.extend([]),
                   lambda: setattr(x, "clades", list(x.clades)), lambda: setattr(x, "mask", None),
                   lambda: delattr(x, "mask")):
        before = topology_epoch()
        change()
        assert topology_epoch() > before
    # a list assigned to a clade is wrapped, so its own later mutations are seen too
    x.clades = [Clade(name="F")]
    before = topology_epoch()
    x.clades += [Clade(name="G")]
    assert topology_epoch() > before and [c.name for c in x.clades] == ["F", "G"]


def test_length_counter_moves_on_every_assignment_and_only_then():
    """Branch lengths reach the device again only when the length counter moved
    since the session's copy: every assignment of a Clade's branch_length moves
    it (to the same value too), reads and other attributes do not, and the bulk
    assignment of new lengths moves it once."""
    import copy
    from treetime_gb300.tree import assign_lengths, length_epoch, topology_epoch
    t = parse_newick("((A:0.1,B:0.2)x:0.05,C:0.3)r;")
    nodes = _nodes(t)
    e, te = length_epoch(), topology_epoch()
    _ = [n.branch_length for n in nodes]
    nodes[1].mutation_length = 0.4
    nodes[1].name = "z"
    assert length_epoch() == e
    nodes[1].branch_length = nodes[1].branch_length
    assert length_epoch() == e + 1 and topology_epoch() == te
    assign_lengths([n.__dict__ for n in nodes[1:]], [0.5, 0.6, 0.7, 0.8])
    assert length_epoch() == e + 2
    assert [n.branch_length for n in nodes[1:]] == [0.5, 0.6, 0.7, 0.8]
    assert [n.mutation_length for n in nodes[1:]] == [0.5, 0.6, 0.7, 0.8]
    assign_lengths([n.__dict__ for n in nodes[1:3]], [0.1, 0.2], dist2root=[1.0, 2.0])
    assert length_epoch() == e + 3
    assert [(n.branch_length, n.mutation_length, n.dist2root) for n in nodes[1:3]] == [(0.1, 0.1, 1.0),
                                                                                      (0.2, 0.2, 2.0)]
    # a clade without a length reads None; copies keep the lengths
    assert Clade(name="N").branch_length is None
    c = copy.deepcopy(t)
    assert [n.branch_length for n in c.find_clades()] == [n.branch_length for n in nodes]


def test_vector_draws_equal_scalar_draws():
    """The Fitch root's ambiguous positions draw rng.integers(bounds) in one call; TreeTime
    draws rng.integers(bound) position by position (treetime/treeanc.py:615-617).  The two give
    the same numbers and leave the generator in the same state (numpy's bounded draws take the
    bit generator's 32-bit outputs in order either way)."""
    import numpy as np
    for seed in range(6):
        bounds = np.random.default_rng(50 + seed).integers(2, 5, size=700)
        a = np.random.default_rng(seed)
        b = np.random.default_rng(seed)
        assert [int(a.integers(k)) for k in bounds] == b.integers(bounds).tolist()
        assert a.random() == b.random()
