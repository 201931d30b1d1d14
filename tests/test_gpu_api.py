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


def _bl_pair(n_tips, L, mean_bl, seed):
    """(FP32 lengths, FP64 lengths, FP64 objective) of every branch of one
    synthetic nucleotide tree, from profile-mode Brent."""
    from treetime_gb300 import TreeAnc, synth
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import parse_newick, to_newick
    rng = np.random.default_rng(seed)
    tree = synth.coalescent_tree(n_tips, mean_bl, rng)
    g = GTR.custom(mu=1.0, pi=rng.dirichlet(np.ones(4)), W=np.ones((4, 4)), alphabet="nuc_nogap")
    aln = synth._to_text(synth.evolve(tree, g, L, rng), g.alphabet, 0.0, rng)
    nwk = to_newick(tree)
    out = {}
    for prec in ("f32", "f64"):
        t = TreeAnc(tree=parse_newick(nwk), aln=aln, gtr=g, verbose=0, precision=prec)
        t.infer_ancestral_sequences(marginal=True)
        nodes = [n for n in t.tree.find_clades() if n.up is not None]
        out[prec] = (t, {n.name: x for n, x in zip(nodes, t._marginal_branch_lengths(nodes, 1e-10))})
    return out, g


def _heavy_pair():
    """The same comparison through the engine with every pattern's
    multiplicity scaled by 20 (TreeTime's compression only merges constant
    columns, so a TreeAnc never has more than a handful of heavy patterns)."""
    from treetime_gb300 import TreeAnc, engine, synth
    from treetime_gb300.gtr import GTR
    rng = np.random.default_rng(12)
    tree = synth.coalescent_tree(16, 0.05, rng)
    g = GTR.custom(mu=1.0, pi=rng.dirichlet(np.ones(4)), W=np.ones((4, 4)), alphabet="nuc_nogap")
    aln = synth._to_text(synth.evolve(tree, g, 400, rng), g.alphabet, 0.0, rng)
    t = TreeAnc(tree=tree, aln=aln, gtr=g, verbose=0)
    ti = t._get_session()["forest"].inputs[0]
    heavy = engine.TreeInput(ti.layout, ti.tip_codes, ti.tip_row, ti.mult * 20.0, ti.bl)
    assert (heavy.mult > 16).sum() > 64
    lay = ti.layout
    ks = np.arange(lay.n_nodes)
    ks = ks[ks != lay.n_int - 1]
    out = {}
    for prec in ("f32", "f64"):
        forest = engine.Forest([heavy], 4)
        model = engine.model_for(g)
        bufs = engine.Buffers(forest)
        res = engine.marginal(forest, model, bufs, precision=prec, keep_outgroup=True, tip_outgroup=True)
        P = int(forest.trees_host["n_patterns"][0])
        vals = {}
        for grp, pp in ((ks[ks < lay.n_int], res["outgroup"]), (ks[ks >= lay.n_int], res["tip_outgroup"])):
            tips = grp[0] >= lay.n_int
            pp_row = [((k - lay.n_int) if tips else k) * P for k in grp]
            pc_row = [-1 if tips else k * P for k in grp]
            tt, _ = engine.optimal_t_profiles(forest, model, grp, pp, pp_row, res["partial"], pc_row, prec, None,
                                              True, 1e-10)
            vals.update({lay.nodes[k].name: x for k, x in zip(grp, tt.cpu().numpy())})
        out[prec] = (t, vals)
    # the FP64 objective uses the FP64 reconstruction's profiles with the scaled multiplicities
    t.infer_ancestral_sequences(marginal=True)
    t.data._multiplicity = t.data.multiplicity() * 20.0
    return out, g


@pytest.mark.gpu
@pytest.mark.parametrize("shape", ["many_patterns", "many_heavy"])
def test_fp32_profile_brent_matches_fp64(shape):
    """FP32-profile Brent (FP32 objective) against the FP64 path: more
    patterns than the kernel's shared memory holds (rows staged in the CTA's
    workspace slice), and more than 64 heavy patterns (the first 64 in FP64).
    Lengths agree to 2e-3 relative, or the FP64 objective agrees to 1e-6."""
    from oracle import anc as oanc
    if shape == "many_patterns":
        out, g = _bl_pair(40, 6000, 0.2, 11)
        assert out["f32"][0].data.compressed_length > (100 * 1024) // 36
    else:
        out, g = _heavy_pair()
    t64 = out["f64"][0]
    nodes = {n.name: n for n in t64.tree.find_clades()}
    mult = t64.data.multiplicity()
    for name, x32 in out["f32"][1].items():
        x64 = out["f64"][1][name]
        if abs(x32 - x64) <= 2e-3 * abs(x64) + 1e-10:
            continue
        n = nodes[name]
        pp, pc = n.marginal_outgroup_LH, n.marginal_subtree_LH
        f = lambda tt: -oanc.prob_t_profiles(g, (pp, pc), mult, tt, return_log=True) + np.exp(tt * tt / 1e4)
        assert abs(f(x32) - f(x64)) <= 1e-6 * abs(f(x64)) + 1e-12, (name, x32, x64)


@pytest.mark.gpu
@pytest.mark.parametrize("invariant_frac", [0.0, 0.9])
def test_fp32_profile_brent_is_deterministic(invariant_frac):
    """Repeated launches of the FP32 profile Brent kernel give bit-identical
    lengths: the warps' roles move between launches (they follow the CTAs'
    placement), the patterns each thread sums do not.  With invariant sites
    the constant columns are heavy patterns (the helper warp's FP64 terms)."""
    from treetime_gb300 import TreeAnc, synth
    wl = synth.make_workload("c0", seed=5, n=60, L=3000, invariant_frac=invariant_frac, gap_frac=0.0)
    t = TreeAnc(tree=wl["tree"], aln=wl["aln"], gtr=wl["gtr"], verbose=0, precision="f32")
    t.infer_ancestral_sequences(marginal=True)
    nodes = [n for n in t.tree.find_clades() if n.up is not None]
    first = t._marginal_branch_lengths(nodes, 1e-10)
    for _ in range(4):
        np.testing.assert_array_equal(t._marginal_branch_lengths(nodes, 1e-10), first)
