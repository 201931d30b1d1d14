"""Edge cases of the reconstruction path on the GPU against the CPU oracle:
the smallest tree TreeTime accepts (three tips at the root), a single
alignment column, identical sequences (only
constant patterns), tips without sequences, very short and very long
branches, and a 20-state alphabet on a three-tip tree.

Tolerances: FP64 log-likelihoods 1e-10 relative, FP32 1e-6 relative;
states bit-exact except where the oracle's top-two margin is below 1e-9."""

import numpy as np
import pytest

from oracle import anc

pytestmark = pytest.mark.gpu


def _run(newick, aln, gtr, precision, marginal=True):
    from treetime_gb300 import TreeAnc
    from treetime_gb300.tree import parse_newick
    t = TreeAnc(tree=parse_newick(newick), aln=dict(aln), gtr=gtr, verbose=0, precision=precision)
    t.infer_ancestral_sequences(marginal=marginal)
    return t


def _oracle(newick, aln, gtr, marginal=True):
    from treetime_gb300.tree import parse_newick
    from treetime_gb300.seqdata import SequenceData
    tree = parse_newick(newick)
    anc.prepare_tree(tree)
    sd = SequenceData(dict(aln), compress=True, ambiguous=gtr.ambiguous)
    chars = np.asarray(sd.compressed_codes).view("S1").astype("U1")
    caln = {k: chars[i] for i, k in enumerate(sd.sequence_names)}
    f = anc.marginal if marginal else anc.joint
    return f(tree, caln, sd.multiplicity(), gtr, sd.full_length)


def _gtr(alphabet="nuc_nogap", q=4, seed=0):
    from treetime_gb300.gtr import GTR
    rng = np.random.default_rng(seed)
    W = rng.uniform(0.5, 2.0, size=(q, q))
    return GTR.custom(mu=1.0, pi=rng.dirichlet(np.ones(q)), W=W + W.T, alphabet=alphabet)


CASES = {
    "three_tips": ("(A:0.1,B:0.2,C:0.05);", {"A": "ACGTACGTAA", "B": "ACGTTCGTAC", "C": "ACGTACGTTC"}),
    "one_column": ("((A:0.1,B:0.2):0.05,C:0.3);", {"A": "G", "B": "T", "C": "G"}),
    "identical": ("((A:0.1,B:0.2):0.05,(C:0.3,D:0.01):0.02);", {k: "ACGTTGCA" * 5 for k in "ABCD"}),
    "missing_tip": ("((A:0.1,B:0.2):0.05,(C:0.3,D:0.01):0.02);", {"A": "ACGTTGCAAC", "B": "ACGTTGCATC",
                                                                  "C": "ACGATGCAAC"}),
    "short_and_long": ("((A:1e-9,B:0.0):1e-7,(C:3.0,D:0.5):2.5);", {"A": "ACGTTGCAAC", "B": "ACGTTGCATC",
                                                                    "C": "TTGATCCAAG", "D": "ACGAAGCAAC"}),
}


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_marginal_edge_cases_match_oracle(case, precision):
    newick, aln = CASES[case]
    g = _gtr()
    t = _run(newick, aln, g, precision)
    o = _oracle(newick, aln, _gtr())
    rel = 1e-10 if precision == "f64" else 1e-6
    assert abs(t.tree.total_sequence_LH - o["total_sequence_LH"]) <= rel * abs(o["total_sequence_LH"]) + 1e-12
    nodes = {n.name: n for n in t.tree.find_clades()}
    for name, prof in o["profile"].items():
        if name not in nodes or not nodes[name].clades:
            continue
        top2 = np.sort(prof, axis=1)
        ok = (top2[:, -1] - top2[:, -2]) > 1e-9
        got = np.asarray(nodes[name].cseq)
        np.testing.assert_array_equal(got[ok], o["cseq"][name][ok], err_msg=name)


@pytest.mark.parametrize("case", sorted(CASES))
def test_joint_edge_cases_match_oracle(case):
    newick, aln = CASES[case]
    t = _run(newick, aln, _gtr(), "f64", marginal=False)
    o = _oracle(newick, aln, _gtr(), marginal=False)
    want = o["sequence_joint_LH"]
    assert abs(t.tree.sequence_joint_LH - want) <= 1e-10 * abs(want) + 1e-12
    nodes = {n.name: n for n in t.tree.find_clades()}
    for name, seq in o["cseq"].items():
        if name in nodes and nodes[name].clades:
            np.testing.assert_array_equal(np.asarray(nodes[name].cseq), seq, err_msg=name)


def test_twenty_states_three_tips():
    from treetime_gb300.gtr import GTR
    rng = np.random.default_rng(3)
    W = rng.random((20, 20))
    pi = rng.dirichlet(np.ones(20))
    newick = "((A:0.2,B:0.1):0.3,C:0.4);"
    aln = {"A": "ACDEFGHIKLMNPQRSTVWY", "B": "ACDEFGHIKLMNPQRSTVWW", "C": "YCDEFGHIKLMNPQRSTVWA"}
    for precision, rel in (("f64", 1e-10), ("f32", 1e-6)):
        t = _run(newick, aln, GTR.custom(mu=1.0, pi=pi, W=W, alphabet="aa_nogap"), precision)
        o = _oracle(newick, aln, GTR.custom(mu=1.0, pi=pi, W=W, alphabet="aa_nogap"))
        assert abs(t.tree.total_sequence_LH - o["total_sequence_LH"]) <= rel * abs(o["total_sequence_LH"])


def test_two_tips_rejected_like_treetime():
    """TreeTime refuses trees with fewer than three tips (MissingDataError)."""
    from treetime_gb300.errors import MissingDataError
    with pytest.raises(MissingDataError):
        _run("(A:0.1,B:0.2);", {"A": "ACGT", "B": "ACGA"}, _gtr(), "f64")


def test_branch_lengths_and_fitch_on_three_tips():
    newick, aln = CASES["three_tips"]
    t = _run(newick, aln, _gtr(), "f64", marginal=False)
    t.optimize_branch_lengths_joint()
    assert all(np.isfinite(n.branch_length) for n in t.tree.find_clades() if n.up is not None)
    assert t.infer_ancestral_sequences(method="fitch") >= 0
