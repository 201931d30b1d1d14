"""GPU: the FP32 site-specific kernel on trees with polytomies (including a
trifurcating root) and a one-child node, for several site-range widths: the
kernel switches between one thread per site (wide levels, siblings transported
together) and two lanes per site (narrow levels, one child each), and takes the
children of other nodes one at a time.  Against the FP64 site-specific kernel
(log domain) on the same session and against the oracle.

Tolerances: site log-likelihoods 1e-6 relative, posterior profiles 1e-5
absolute (FP32 profiles)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tree_with_shapes(seed=5, n=60, L=200):
    from treetime_gb300 import synth
    from treetime_gb300.tree import Clade
    wl = synth.make_workload("c2", seed=seed, n=n, L=L)
    tree = wl["tree"]
    # polytomies: splice three internal nodes' children into their parents (one of them a
    # child of the root, which makes the root trifurcating)
    for pick in (lambda inner: inner[len(inner) // 3], lambda inner: inner[2 * len(inner) // 3],
                 lambda inner: next(c for c in tree.root.clades if c.clades)):
        inner = [c for c in tree.find_clades(order="postorder") if c.clades and c is not tree.root]
        c = pick(inner)
        for par in tree.find_clades():
            if c in par.clades:
                i = par.clades.index(c)
                par.clades[i:i + 1] = c.clades
                break
    # a node with one child: a tip's branch split in two
    tip = next(iter(tree.get_terminals()))
    for par in tree.find_clades():
        if tip in par.clades:
            i = par.clades.index(tip)
            half = tip.branch_length / 2
            tip.branch_length = half
            par.clades[i] = Clade(branch_length=half, clades=[tip])
            break
    assert len(tree.root.clades) >= 3
    return wl


def test_site_specific_fp32_on_polytomies_and_one_child_nodes():
    from oracle import anc
    from treetime_gb300 import TreeAnc, engine
    from treetime_gb300.tree import parse_newick, to_newick
    wl = _tree_with_shapes()
    t = TreeAnc(tree=wl["tree"], aln=wl["aln"], gtr=wl["gtr"], compress=False, verbose=0, precision="f64")
    t.infer_ancestral_sequences(marginal=True)
    sess = t._get_session()
    forest, bufs, layout = sess["forest"], sess["bufs"], sess["layout"]
    ref = engine.marginal_site_specific(forest, t.gtr, bufs, precision="f64")
    lh64 = ref["site_lh"].cpu().numpy().copy()
    post64 = ref["posterior"].cpu().numpy().copy()
    # the oracle on the same tree
    tree_o = anc.prepare_tree(parse_newick(to_newick(t.tree)))
    res = anc.marginal(tree_o, t.data.compressed_alignment, t.data.multiplicity(), t.gtr, t.data.full_length)
    np.testing.assert_allclose(lh64, np.asarray(res["sequence_LH"]), rtol=1e-9, atol=0)
    P = t.data.compressed_length
    for rw in (None, 1, 3, 16, 32):
        out = engine.marginal_site_specific(forest, t.gtr, bufs, precision="f32", range_width=rw)
        lh32 = out["site_lh"].cpu().numpy()
        np.testing.assert_allclose(lh32, lh64, rtol=1e-6, atol=0, err_msg="range width %s" % rw)
        post32 = out["posterior"].cpu().numpy()
        n_int, w = layout.n_int, forest.w
        a = post32[:n_int * P].reshape(n_int, P, w)[..., :t.gtr.n_states]
        b = post64[:n_int * P].reshape(n_int, P, w)[..., :t.gtr.n_states]
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-5, err_msg="range width %s" % rw)
