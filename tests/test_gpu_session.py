"""GPU: the reconstruction session keeps its device copy of the branch lengths
between calls while no Clade's length was assigned (an O(1) check instead of a
walk over the nodes).  Every way a length changes -- one assignment, the bulk
update of optimize_branch_lengths_joint, TreeTime's root-pair update of the
marginal optimisation -- must reach the next reconstruction: the results equal
those of a fresh TreeAnc on a copy of the same tree (new clade objects from its
Newick text), bit for bit (FP64)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _workload():
    from treetime_gb300 import synth
    return synth.make_workload("c0", seed=11, n=80, L=600)


def _fresh_lh(t, wl):
    from treetime_gb300 import TreeAnc
    from treetime_gb300.tree import parse_newick, to_newick
    # the same topology, names and lengths (repr of each length: exact) in new clade objects
    f = TreeAnc(tree=parse_newick(to_newick(t.tree)), aln=wl["aln"], gtr=t.gtr, verbose=0, precision="f64")
    f.infer_ancestral_sequences(marginal=True)
    return f.tree.sequence_LH.copy(), {n.name: n._cseq.copy() for n in f.tree.get_nonterminals()}


def _same(t, ref):
    lh, seqs = ref
    assert np.array_equal(t.tree.sequence_LH, lh)
    for n in t.tree.get_nonterminals():
        assert np.array_equal(n._cseq, seqs[n.name])


def test_length_changes_reach_the_next_reconstruction():
    from treetime_gb300 import TreeAnc
    wl = _workload()
    t = TreeAnc(tree=wl["tree"], aln=wl["aln"], gtr=wl["gtr"], verbose=0, precision="f64")
    t.infer_ancestral_sequences(marginal=True)
    first = t.tree.sequence_LH.copy()
    t.infer_ancestral_sequences(marginal=True)  # unchanged lengths: the copy on the device is reused
    assert np.array_equal(t.tree.sequence_LH, first)
    _same(t, _fresh_lh(t, wl))
    # one assignment
    node = list(t.tree.find_clades())[5]
    node.branch_length = node.branch_length * 3 + 0.01
    t.infer_ancestral_sequences(marginal=True)
    assert not np.array_equal(t.tree.sequence_LH, first)
    _same(t, _fresh_lh(t, wl))
    # the joint optimisation's bulk update, then a reconstruction
    t.infer_ancestral_sequences(marginal=False)
    t.optimize_branch_lengths_joint()
    t.infer_ancestral_sequences(marginal=True)
    _same(t, _fresh_lh(t, wl))
    # a length set back to an earlier value is still a change
    before = node.branch_length
    node.branch_length = before * 0.5
    t.infer_ancestral_sequences(marginal=True)
    mid = t.tree.sequence_LH.copy()
    node.branch_length = before
    t.infer_ancestral_sequences(marginal=True)
    assert not np.array_equal(t.tree.sequence_LH, mid)
    _same(t, _fresh_lh(t, wl))


def test_marginal_optimisation_lengths_reach_the_reconstruction():
    from treetime_gb300 import TreeAnc
    wl = _workload()
    t = TreeAnc(tree=wl["tree"], aln=wl["aln"], gtr=wl["gtr"], verbose=0, precision="f64")
    t.optimize_tree_marginal(max_iter=2)
    t.infer_ancestral_sequences(marginal=True)
    _same(t, _fresh_lh(t, wl))
