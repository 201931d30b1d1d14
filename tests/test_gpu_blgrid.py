"""Branch-length likelihood grids (TreeTime's BranchLenInterpolator values)
on the GPU through ``TreeAnc.branch_length_grids``, against TreeTime's own
grids and values (golden fixtures) and the CPU oracle.

Tolerances: grids bit-exact (host-built); -log P on the grid 1e-9 relative +
1e-8 absolute from FP64 profiles / pair counts, 1e-4 relative + 1e-3
absolute from FP32-scaled profiles (FP32 arithmetic for up to 5 states).  'joint' values are compared with
TreeTime's at the grid points where every observed state pair has
P(t) >= 1e-6; below that (t near 0) TreeTime's value is set by the rounding
of V diag(exp(Qt)) V^-1, and the kernel's (formed with expm1) is compared
with the oracle's expm1 form at every point instead."""

import numpy as np
import pytest

import golden_cases as gc
from oracle import anc

pytestmark = pytest.mark.gpu

CASES = gc.blgrid_names()


def _tree_anc(g, precision="f64"):
    from treetime_gb300 import TreeAnc
    tree, aln, model, _ = gc.inputs_from(g)
    return TreeAnc(tree=tree, aln=aln, gtr=model, compress=True, verbose=0, precision=precision)


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("mode", ["marginal", "joint"])
@pytest.mark.parametrize("case", CASES)
def test_branch_length_grids_match_treetime(case, mode, precision):
    if mode == "joint" and precision == "f32":
        pytest.skip("joint reconstruction and pair counts are FP64 only")
    g = gc.load(case)
    t = _tree_anc(g, precision)
    t.infer_ancestral_sequences(marginal=mode == "marginal")
    res = t.branch_length_grids(branch_length_mode=mode, n_grid_points=int(g["n_grid_points"]))
    by_name = {n.name: v for n, v in res.items()}
    assert set(by_name) == set(g[mode + "_names"].tolist())
    rtol, atol = (1e-9, 1e-8) if precision == "f64" else (1e-4, 1e-3)
    oe = gc.blgrid_oracle(g, mode, expm1_form=True) if mode == "joint" else None
    for i, name in enumerate(g[mode + "_names"].tolist()):
        L = int(g[mode + "_len"][i])
        grid, y = by_name[name]
        np.testing.assert_array_equal(grid, g[mode + "_x"][i, :L])
        want = g[mode + "_y"][i, :L] + g[mode + "_peak"][i]
        ok = np.ones(L, bool) if oe is None else oe[name][1] >= 1e-6
        np.testing.assert_allclose(y[ok], want[ok], rtol=rtol, atol=atol, err_msg=name)
        if oe is not None:
            np.testing.assert_allclose(y, oe[name][0], rtol=1e-9, atol=1e-8, err_msg=name)


def _masked_tree(g, precision, rng):
    t = _tree_anc(g, precision)
    P = t.data.compressed_length
    masks = {}
    for i, n in enumerate(t.tree.find_clades()):
        if n.up is not None and i % 3 == 1:
            n.mask = (rng.random(P) < 0.6).astype(float)
            masks[n.name] = n.mask
    return t, masks


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("case", CASES)
def test_branch_length_grids_with_masks_match_oracle(case, precision):
    """Per-node masks weight the patterns (data.multiplicity(mask=node.mask))."""
    g = gc.load(case)
    rng = np.random.default_rng(5)
    t, masks = _masked_tree(g, precision, rng)
    rtol, atol = (1e-9, 1e-8) if precision == "f64" else (1e-4, 1e-3)
    t.infer_ancestral_sequences(marginal=True)
    res = {n.name: v for n, v in t.branch_length_grids(branch_length_mode="marginal").items()}
    tree, aln, model, _ = gc.inputs_from(g)
    anc.prepare_tree(tree)
    for n in anc.preorder(tree.root):
        if n.name in masks:
            n.mask = masks[n.name]
    caln, mult, full = gc.compress_inputs(aln, model)
    o = anc.marginal(tree, caln, mult, model, full)
    for n in anc.preorder(tree.root):
        if n.up is None:
            continue
        grid, y = res[n.name]
        m = mult if getattr(n, "mask", None) is None else mult * n.mask
        want = anc.branch_len_log_prob(model, grid, "marginal",
                                       profile_pair=(o["outgroup_LH"][n.name], o["subtree_LH"][n.name]),
                                       multiplicity=m)
        np.testing.assert_allclose(y, want, rtol=rtol, atol=atol, err_msg=n.name)


def test_branch_length_grids_protein_beyond_shared_memory():
    """21-state alphabet with more patterns than the kernel keeps in shared
    memory: the coefficients past the cap go through the workspace."""
    from treetime_gb300 import TreeAnc, synth
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import parse_newick, to_newick
    rng = np.random.default_rng(9)
    tree = synth.coalescent_tree(12, 0.3, rng)
    pi = rng.dirichlet(np.ones(21))
    W = rng.random((21, 21))
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet=synth.AA21)
    states = synth.evolve(tree, g, 3000, rng)
    aln = synth._to_text(states, g.alphabet, 0.0, rng)
    nwk = to_newick(tree)
    t = TreeAnc(tree=parse_newick(nwk), aln=aln, gtr=g, compress=True, verbose=0)
    assert t.data.compressed_length > (200 * 1024) // (22 * 8)
    t.infer_ancestral_sequences(marginal=True)
    nodes = [n for n in t.tree.find_clades() if n.up is not None][:6]
    res = t.branch_length_grids(nodes=nodes, branch_length_mode="marginal", n_grid_points=40)
    model_o = GTR.custom(mu=1.0, pi=pi, W=W, alphabet=synth.AA21)
    tree_o = parse_newick(nwk)
    anc.prepare_tree(tree_o)
    caln, mult, full = gc.compress_inputs(aln, model_o)
    o = anc.marginal(tree_o, caln, mult, model_o, full)
    for n in nodes:
        grid, y = res[n]
        want = anc.branch_len_log_prob(model_o, grid, "marginal",
                                       profile_pair=(o["outgroup_LH"][n.name], o["subtree_LH"][n.name]),
                                       multiplicity=mult)
        np.testing.assert_allclose(y, want, rtol=1e-9, atol=1e-8, err_msg=n.name)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_branch_length_grids_odd_grid_length(precision):
    """n_grid_points = 200 gives 209-point grids (an odd row length, so the
    FP32 kernel's pattern rows start after a padded shared-memory table)."""
    g = gc.load("blgrid_nuc")
    t = _tree_anc(g, precision)
    t.infer_ancestral_sequences(marginal=True)
    res = {n.name: v for n, v in t.branch_length_grids(branch_length_mode="marginal", n_grid_points=200).items()}
    assert max(len(v[0]) for v in res.values()) % 2 == 1
    tree, aln, model, _ = gc.inputs_from(g)
    anc.prepare_tree(tree)
    caln, mult, full = gc.compress_inputs(aln, model)
    o = anc.marginal(tree, caln, mult, model, full)
    rtol, atol = (1e-9, 1e-8) if precision == "f64" else (1e-4, 1e-3)
    for n in anc.preorder(tree.root):
        if n.up is None:
            continue
        grid, y = res[n.name]
        want = anc.branch_len_log_prob(model, grid, "marginal",
                                       profile_pair=(o["outgroup_LH"][n.name], o["subtree_LH"][n.name]),
                                       multiplicity=mult)
        np.testing.assert_allclose(y, want, rtol=rtol, atol=atol, err_msg=n.name)
