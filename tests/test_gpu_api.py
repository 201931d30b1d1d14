"""GPU checks of the GTR-level entry points against the CPU oracle, and of
TreeTime's self-contained known-answer tests (test/test_treetime.py:137-307)
run through the GPU implementation."""

import io

import numpy as np
import pytest

from oracle import anc

pytestmark = pytest.mark.gpu


def _models():
    from treetime_gb300 import GTR
    rng = np.random.default_rng(5)
    out = [GTR.standard("JC69"), GTR.custom(pi=rng.dirichlet(np.ones(4)), W=rng.uniform(0.5, 2, (4, 4)),
                                             alphabet="nuc_nogap"),
           GTR.random(alphabet="aa", rng=rng)]
    return out


@pytest.mark.parametrize("mi", range(3))
def test_expqt_propagate_evolve(mi):
    g = _models()[mi]
    q = g.n_states
    rng = np.random.default_rng(mi)
    for t in (0.0, 1e-6, 0.013, 0.7, 3.9):
        np.testing.assert_allclose(g.expQt(t), anc.expQt(g, t), rtol=1e-12, atol=1e-14)
        prof = rng.random((50, q))
        np.testing.assert_allclose(g.propagate_profile(prof, t), anc.propagate_profile(g, prof, t), rtol=1e-12)
        np.testing.assert_allclose(g.evolve(prof, t, return_log=True), anc.evolve(g, prof, t, return_log=True),
                                   rtol=1e-12, atol=1e-13)
    ts = np.linspace(0, 2, 7)
    np.testing.assert_allclose(g.expQt(ts), np.stack([anc.expQt(g, t) for t in ts]), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("mi", range(3))
def test_state_pair_and_branch_length(mi):
    g = _models()[mi]
    rng = np.random.default_rng(10 + mi)
    P = 300
    a = g.alphabet[rng.integers(g.n_states, size=P)]
    b = a.copy()
    flip = rng.random(P) < 0.1
    b[flip] = g.alphabet[rng.integers(g.n_states, size=flip.sum())]
    b[:3] = "N" if g.n_states < 10 else "X"
    mult = rng.integers(1, 5, size=P).astype(float)
    for ig in (False, True):
        pairs, counts = g.state_pair(a, b, pattern_multiplicity=mult, ignore_gaps=ig)
        rp, rc = anc.state_pair(g, a, b, pattern_multiplicity=mult, ignore_gaps=ig)
        assert sorted(map(tuple, pairs.tolist())) == sorted(map(tuple, rp.tolist()))
        assert dict(zip(map(tuple, pairs.tolist()), counts)) == dict(zip(map(tuple, rp.tolist()), rc))
        for t in (0.0, 0.05, 1.0):
            v = g.prob_t_compressed(pairs, counts, t, return_log=True)
            assert abs(v - anc.prob_t_compressed(g, rp, rc, t, return_log=True)) <= 1e-10 * abs(v) + 1e-12
        got = g.optimal_t_compressed(pairs, counts)
        want, _ = anc.optimal_t_compressed(g, rp, rc)
        assert abs(got - want) <= 1e-6 * want + 1e-10, (got, want)


def test_profile_branch_length():
    g = _models()[1]
    rng = np.random.default_rng(3)
    P = 500
    pp = rng.dirichlet(np.ones(4) * 0.3, size=P)
    # child profiles correlated with the parent through a branch of length 0.05
    pc = anc.propagate_profile(g, pp, 0.05) + 0.05 * rng.dirichlet(np.ones(4), size=P)
    pc /= pc.sum(axis=1, keepdims=True)
    m = rng.integers(1, 4, size=P).astype(float)
    got = g.optimal_t_compressed((pp, pc), m, profiles=True)
    want, _ = anc.optimal_t_compressed(g, (pp, pc), m, profiles=True)
    assert abs(got - want) <= 1e-6 * want + 1e-10, (got, want)
    v = g.prob_t_profiles((pp, pc), m, 0.1, return_log=True)
    assert abs(v - anc.prob_t_profiles(g, (pp, pc), m, 0.1, return_log=True)) < 1e-9 * abs(v)


def test_site_specific_expqt():
    from treetime_gb300 import synth
    rng = np.random.default_rng(2)
    for approx in (True, False):
        g = synth.gtr_c2(rng, 12, approximate=approx)
        for t in (0.0, 0.03, 0.4, 200.0):
            np.testing.assert_allclose(g.expQt(t), anc.expQt(g, t), rtol=1e-10, atol=1e-12)


# ---------------------------------------------------------------- known answers
def test_lh_normalization_over_all_patterns():
    """Sum over all 64 site patterns of exp(sequence_LH) is 1
    (test/test_treetime.py:137-155)."""
    from treetime_gb300 import GTR, TreeAnc
    from treetime_gb300.tree import parse_newick
    aln = {"A": "AAAAAAAAAAAAAAAACCCCCCCCCCCCCCCCGGGGGGGGGGGGGGGGTTTTTTTTTTTTTTTT",
           "B": "AAAACCCCGGGGTTTTAAAACCCCGGGGTTTTAAAACCCCGGGGTTTTAAAACCCCGGGGTTTT",
           "C": "ACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGT"}
    for precision in ("f64", "f32"):
        gtr = GTR.custom(alphabet=np.array(["A", "C", "G", "T"]), pi=np.array([0.9, 0.06, 0.02, 0.02]),
                         W=np.ones((4, 4)))
        t = TreeAnc(gtr=gtr, tree=parse_newick("((A:0.60100000009,B:0.3010000009):0.1,C:0.2):0.001;"), aln=aln,
                    rng_seed=1234, verbose=0, precision=precision)
        t.reconstruct_anc("ml", marginal=True, debug=True)
        lhsum = np.exp(t.sequence_LH(pos=np.arange(4 ** 3))).sum()
        assert abs(lhsum - 1.0) < 1e-6
        t.optimize_branch_len()


def _tiny_joint_tree(seq_len=400):
    from treetime_gb300 import GTR, TreeAnc
    from treetime_gb300.tree import parse_newick
    mygtr = GTR.custom(alphabet=np.array(["A", "C", "G", "T"]), pi=np.array([0.15, 0.95, 0.05, 0.3]),
                       W=np.ones((4, 4)))
    tree = parse_newick("((A:.060,B:.01200)C:.020,D:.0050)E:.004;")
    rng = np.random.default_rng(1234)
    root = rng.choice(mygtr.alphabet, p=mygtr.Pi, size=seq_len)
    seqs = {}
    stack = [(tree.root, root)]
    while stack:
        node, s = stack.pop()
        seqs[node.name] = s
        for c in node.clades:
            p = mygtr.evolve(anc.seq2prof(s, mygtr.profile_map), c.branch_length)
            p = (p.T / p.sum(axis=1)).T
            idx = np.array([int(rng.choice(np.arange(p.shape[1]), p=p[k])) for k in range(p.shape[0])])
            stack.append((c, mygtr.alphabet[idx]))
    aln = {n.name: "".join(seqs[n.name]) for n in tree.get_terminals()}
    return TreeAnc(gtr=mygtr, tree=tree, aln=aln, verbose=0, rng_seed=1234, compress=False), seqs


def test_joint_lh_equals_ancestral_likelihood():
    """Joint per-site LH equals the likelihood of the reconstructed assignment
    (test/test_treetime.py:160-238)."""
    t, seqs = _tiny_joint_tree()
    t.infer_ancestral_sequences(marginal=False, reconstruct_tip_states=True)
    LH = t.ancestral_likelihood()
    assert abs((LH - t.tree.sequence_LH).sum()) < 1e-9
    diff = sum(int(np.sum(n.cseq != seqs[n.name])) for n in t.tree.find_clades() if n.up is not None)
    muts = sum(int(np.sum(seqs[n.name] != seqs[n.up.name])) for n in t.tree.find_clades() if n.up is not None)
    assert diff / 400 < 2 * (muts / 400) ** 2 + 0.05


def test_joint_lh_is_max_by_brute_force():
    """The joint LH equals the maximum over all 16 internal-state assignments
    (test/test_treetime.py:241-307)."""
    from treetime_gb300 import GTR, TreeAnc
    from treetime_gb300.tree import parse_newick
    gtr = GTR.custom(alphabet=np.array(["A", "C", "G", "T"]), pi=np.array([0.91, 0.05, 0.02, 0.02]),
                     W=np.ones((4, 4)))
    nwk = "((A:.0060,B:.30)C:.030,D:.020)E:.004;"
    t1 = TreeAnc(gtr=gtr, tree=parse_newick(nwk), aln={"A": "A", "B": "C", "D": "G"}, verbose=0)
    t1.reconstruct_anc(method="ml", marginal=False)
    real = t1.tree.sequence_LH
    # reference: log-LH of every assignment of the two internal nodes
    aln = {"A": "A" * 16, "B": "C" * 16, "D": "G" * 16, "C": "AAAACCCCGGGGTTTT", "E": "ACGTACGTACGTACGT"}
    t2 = TreeAnc(gtr=gtr, tree=parse_newick(nwk), aln=aln, verbose=0, compress=False)
    for n in t2.tree.find_clades():
        n._cseq = np.array(list(aln[n.name]))
    t2.reconstructed_tip_sequences = True
    ref = t2.ancestral_likelihood()
    assert abs(ref.max() - real[0]) < 1e-10
