"""GPU: every launch shape of the FP32 marginal kernel (CTA size, pattern-range
width) and the FP64 kernel give the oracle's
results, on a tree with polytomies, masks and missing data, for 4-, 5-, 20- and
21-state alphabets.  Also the multi-tree forest (one launch over several trees
of different sizes and models) against per-tree oracle runs."""

import numpy as np
import pytest

from oracle import anc

pytestmark = pytest.mark.gpu


def _workload(alphabet, seed, n=40, L=300):
    from treetime_gb300 import synth
    wl = synth.make_workload("c0", seed=seed, n=n, L=L, alphabet=alphabet, mean_bl=0.03)
    tree = wl["tree"]
    # a polytomy: splice one internal node's children into its parent
    inner = [c for c in tree.find_clades(order="postorder") if c.clades and c is not tree.root]
    c = inner[len(inner) // 2]
    for par in tree.find_clades():
        if c in par.clades:
            i = par.clades.index(c)
            par.clades[i:i + 1] = c.clades
            break
    return wl


def _oracle(t):
    from treetime_gb300.tree import parse_newick, to_newick
    tree = anc.prepare_tree(parse_newick(to_newick(t.tree)))
    byname = {n.name: n for n in t.tree.find_clades()}
    for n in anc.preorder(tree.root):
        n.mask = getattr(byname[n.name], "mask", None)
    return anc.marginal(tree, t.data.compressed_alignment, t.data.multiplicity(), t.gtr, t.data.full_length,
                        reconstruct_tip_states=True)


SHAPES = [(1024, None), (512, None), ("512x2", None), (1024, 1), (1024, 7), (512, 19), ("512x2", 19), (1024, 32),
          ("512x2", 32), (1024, 100), (512, 512), ("f64", 8), ("f64", 32)]


@pytest.mark.parametrize("alphabet", ["nuc_nogap", "nuc", "aa_nogap", "aa"])
@pytest.mark.parametrize("shape", SHAPES)
def test_marginal_launch_shapes(alphabet, shape):
    """shape = (CTA threads, or "512x2" for two 512-thread CTAs per SM;
    patterns per range, None = sized to fill the GPU)
    or ("f64", warps per CTA).  Range widths that do not divide the
    pattern count, one-pattern ranges and ranges wider than the alignment are
    all covered."""
    from treetime_gb300 import TreeAnc
    threads, rp = shape
    if alphabet.startswith("aa") and (threads in (1024, "512x2") or (threads == "f64" and rp == 32)):
        pytest.skip("20+ states run 512-thread CTAs, one pattern per 4 lanes (ranges rounded up to 8 patterns)")
    wl = _workload(alphabet, seed=7, L=300 if not alphabet.startswith("aa") else 120)
    prec = "f64" if threads == "f64" else "f32"
    if prec == "f64":
        kw = dict(warps_per_block=rp)
    elif threads == "512x2":
        kw = dict(threads=512, ctas_per_sm=2, range_patterns=rp)
    else:
        kw = dict(threads=threads, range_patterns=rp)
    t = TreeAnc(tree=wl["tree"], aln=wl["aln"], gtr=wl["gtr"], verbose=0, precision=prec, **kw)
    rng = np.random.default_rng(1)
    for n in list(t.tree.find_clades())[3:9]:
        n.mask = (rng.random(t.data.compressed_length) < 0.6).astype(float)
    t.infer_ancestral_sequences(marginal=True, reconstruct_tip_states=True)
    ref = _oracle(t)
    tol = 1e-10 if prec == "f64" else 1e-5
    assert abs(t.tree.total_sequence_LH - ref["total_sequence_LH"]) <= (1e-10 if prec == "f64" else 1e-6) * \
        abs(ref["total_sequence_LH"])
    for n in t.tree.find_clades():
        np.testing.assert_allclose(n.marginal_profile, ref["profile"][n.name], atol=tol, rtol=0)
        if n.up is not None:
            np.testing.assert_allclose(n.marginal_outgroup_LH, ref["outgroup_LH"][n.name], atol=tol, rtol=0)
        prof = ref["profile"][n.name]
        s = np.sort(prof, axis=1)
        ok = (n._cseq == ref["cseq"][n.name]) | (s[:, -1] - s[:, -2] < (1e-9 if prec == "f64" else 1e-5))
        assert ok.all(), n.name


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_forest_of_many_trees(precision):
    """One launch over trees of different sizes and models equals the
    per-tree oracle."""
    from treetime_gb300 import GTR, engine, synth
    from treetime_gb300.seqdata import SequenceData
    rng = np.random.default_rng(9)
    inputs, refs, models = [], [], []
    for k in range(6):
        n = int(rng.integers(5, 60))
        L = int(rng.integers(20, 400))
        tree = synth.coalescent_tree(n, float(rng.uniform(0.005, 0.1)), rng, prefix="t")
        gtr = GTR.random(alphabet="nuc_nogap", rng=rng)
        states = synth.evolve(tree, gtr, L, rng)
        aln = synth._to_text(states, gtr.alphabet, 0.02, rng)
        anc.prepare_tree(tree)
        sd = SequenceData(aln, ambiguous="N")
        layout = engine.TreeLayout(tree.root)
        tip_row = np.array([sd.name_to_row[n.name] for n in layout.nodes[layout.n_int:]], dtype=np.int32)
        bl = engine.branch_lengths(layout, sd.full_length)
        inputs.append(engine.TreeInput(layout, sd.compressed_codes, tip_row, sd.multiplicity(), bl, model=k))
        models.append(gtr)
        refs.append(anc.marginal(tree, sd.compressed_alignment, sd.multiplicity(), gtr, sd.full_length))
    forest = engine.Forest(inputs, 4)
    model = engine.DeviceModel(models)
    out = engine.marginal(forest, model, engine.Buffers(forest), precision=precision)
    tree_lh = out["tree_lh"].cpu().numpy()
    post = out["posterior"].cpu().numpy()
    for k, (ti, ref) in enumerate(zip(inputs, refs)):
        assert abs(tree_lh[k] - ref["total_sequence_LH"]) <= 1e-6 * abs(ref["total_sequence_LH"])
        tr = forest.trees_host[k]
        P = ti.n_patterns
        for j, n in enumerate(ti.layout.nodes[:ti.layout.n_int]):
            rows = post[tr["prof_base"] + j * P: tr["prof_base"] + (j + 1) * P, :4]
            np.testing.assert_allclose(rows, ref["profile"][n.name], atol=1e-5 if precision == "f32" else 1e-10)


@pytest.mark.parametrize("width", [1, 7, 32, None])
@pytest.mark.parametrize("approximate", [True, False])
def test_site_specific_f32_range_widths(width, approximate):
    """The FP32 site-specific kernel (site ranges of 1..32 sites with their
    eigenvectors in shared memory) against the FP64 kernel, with masks and
    tips reconstructed."""
    from treetime_gb300 import TreeAnc, engine, synth
    wl = synth.make_workload("c2", seed=4, n=30, L=70, approximate=approximate)
    t = TreeAnc(tree=wl["tree"], aln=wl["aln"], gtr=wl["gtr"], compress=False, verbose=0, precision="f64")
    rng = np.random.default_rng(3)
    for n in list(t.tree.find_clades())[2:7]:
        n.mask = (rng.random(t.data.compressed_length) < 0.5).astype(float)
    s = t._get_session()
    kw = dict(reconstruct_tips=True, keep_outgroup=True, tip_outgroup=True)
    r64 = engine.marginal_site_specific(s["forest"], t.gtr, engine.Buffers(s["forest"]), precision="f64", **kw)
    r32 = engine.marginal_site_specific(s["forest"], t.gtr, engine.Buffers(s["forest"]), precision="f32",
                                        range_width=width, **kw)
    lh64, lh32 = float(r64["tree_lh"][0]), float(r32["tree_lh"][0])
    assert abs(lh32 - lh64) <= 1e-6 * abs(lh64)
    for k in ("posterior", "tip_posterior", "outgroup", "tip_outgroup"):
        np.testing.assert_allclose(r32[k].cpu().numpy(), r64[k].cpu().numpy(), atol=1e-5, rtol=0)
