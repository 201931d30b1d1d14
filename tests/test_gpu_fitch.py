"""Fitch parsimony on the GPU (TreeAnc.infer_ancestral_sequences(method=
'fitch')) against TreeTime's own reconstructions: internal-node characters
bit-exact (including characters outside the alphabet: ambiguity codes, N,
gaps), N_diff exact, the root's random choices from the same generator."""

import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

CASES = gc.fitch_names()


def _tree_anc(g):
    from treetime_gb300 import TreeAnc
    tree, aln, model, _ = gc.inputs_from(g)
    return TreeAnc(tree=tree, aln=aln, gtr=model, compress=True, verbose=0, rng_seed=int(g["rng_seed"]))


def _check(t, g, key):
    nodes = {n.name: n for n in t.tree.find_clades()}
    for i, k in enumerate(g["fitch_names"].tolist()):
        np.testing.assert_array_equal(gc.codes_of(nodes[k].cseq), g[key][i], err_msg=k)


@pytest.mark.parametrize("case", CASES)
def test_fitch_matches_treetime(case):
    g = gc.load(case)
    t = _tree_anc(g)
    assert t.infer_ancestral_sequences(method="fitch") == int(g["fitch_N_diff"])
    assert t.sequence_reconstruction == "parsimony"
    _check(t, g, "fitch_cseq")
    assert t.infer_ancestral_sequences(method="parsimony") == int(g["fitch_N_diff_again"])
    _check(t, g, "fitch_cseq_again")


@pytest.mark.parametrize("case", CASES)
def test_fitch_after_marginal_matches_treetime(case):
    g = gc.load(case)
    t = _tree_anc(g)
    t.infer_ancestral_sequences(marginal=True)
    assert t.infer_ancestral_sequences(method="fitch") == int(g["fitch_after_marginal_N_diff"])
    _check(t, g, "fitch_after_marginal_cseq")
    # an ML reconstruction after Fitch counts its changes against the Fitch characters
    nd = t.infer_ancestral_sequences(marginal=True)
    nodes = [n for n in t.tree.find_clades() if n.clades and n.up is not None]
    assert 0 <= nd <= len(nodes) * t.data.compressed_length
