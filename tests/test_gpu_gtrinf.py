"""GTR inference with the substitution counting on the GPU
(``TreeAnc.infer_gtr``, ``get_branch_mutation_matrix``) against TreeTime's
own counts and models (golden fixtures captured at TreeTime's call of
GTR.infer) and the CPU oracle's per-pattern counts.

Tolerances: counts and times 1e-10 relative (+1e-10 absolute) per pattern and
summed (FP64 profiles), 2e-5 of the largest entry (FP32 profiles, counted in
FP32); inferred W, pi, mu 1e-9 relative from FP64 profiles, 1e-5 relative
from FP32-scaled profiles; mutation matrices 1e-12 absolute (FP64; site-specific
models 1e-10 relative + 1e-12 absolute), 1e-5 absolute (FP32)."""

import numpy as np
import pytest

import golden_cases as gc
from oracle import anc

pytestmark = pytest.mark.gpu

CASES = gc.gtrinf_names()


def _modes(g):
    return [m for m in ("marginal", "joint") if m + "_nij" in g]


def _tree_anc(g, precision="f64"):
    from treetime_gb300 import TreeAnc
    tree, aln, model, masks = gc.inputs_from(g)
    t = TreeAnc(tree=tree, aln=aln, gtr=model, compress=bool(g["compress"]), verbose=0, precision=precision)
    if masks:
        for n in t.tree.find_clades():
            if n.name in masks:
                n.mask = masks[n.name]
    return t


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("case", CASES)
def test_substitution_counts_match_oracle_and_treetime(case, precision):
    g = gc.load(case)
    for mode in _modes(g):
        if mode == "joint" and precision == "f32":
            continue
        t = _tree_anc(g, precision)
        t.infer_ancestral_sequences(marginal=mode == "marginal")
        n_ija, T_ia = t._substitution_counts(mode == "marginal")
        n_ija, T_ia = n_ija.cpu().numpy(), T_ia.cpu().numpy()
        on, oT, _ = gc.gtrinf_oracle(g, mode)
        if precision == "f32":
            # FP32 profiles counted in FP32: 2e-5 of the largest entry of each array
            np.testing.assert_allclose(n_ija, on, rtol=0, atol=2e-5 * np.abs(on).max(), err_msg=mode)
            np.testing.assert_allclose(T_ia, oT, rtol=0, atol=2e-5 * np.abs(oT).max(), err_msg=mode)
            continue
        np.testing.assert_allclose(n_ija, on, rtol=1e-10, atol=1e-10, err_msg=mode)
        np.testing.assert_allclose(T_ia, oT, rtol=1e-10, atol=1e-10, err_msg=mode)
        if bool(g["site_specific"]):
            np.testing.assert_allclose(n_ija, g[mode + "_nij"], rtol=1e-10, atol=1e-10)
            np.testing.assert_allclose(T_ia, g[mode + "_Ti"], rtol=1e-10, atol=1e-10)
        else:
            np.testing.assert_allclose(n_ija.sum(axis=-1), g[mode + "_nij"], rtol=1e-10, atol=1e-10)
            np.testing.assert_allclose(T_ia.sum(axis=-1), g[mode + "_Ti"], rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("case", CASES)
def test_infer_gtr_matches_treetime(case, precision):
    g = gc.load(case)
    rtol = 1e-9 if precision == "f64" else 1e-5
    for mode in _modes(g):
        if mode == "joint" and precision == "f32":
            continue
        t = _tree_anc(g, precision)
        t.infer_ancestral_sequences(marginal=mode == "marginal")
        m = t.infer_gtr(marginal=mode == "marginal", site_specific=bool(g["site_specific"]), pc=float(g["pc"]))
        assert t.gtr is m
        np.testing.assert_allclose(m.W, g[mode + "_W"], rtol=rtol, atol=rtol * 1e-3, err_msg=mode)
        np.testing.assert_allclose(m.Pi, g[mode + "_Pi"], rtol=rtol, atol=rtol * 1e-3, err_msg=mode)
        np.testing.assert_allclose(m.mu, g[mode + "_mu"], rtol=rtol, err_msg=mode)
        # the new model drives the next reconstruction
        t.infer_ancestral_sequences(marginal=True)
        assert np.isfinite(t.sequence_LH())


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("case", ["gtrinf_nuc5", "gtrinf_ss_current"])
def test_branch_mutation_matrix_matches_oracle(case, precision):
    """A single-matrix model, and a site-specific one (each site's own
    interpolated P_a(t), treeanc.py:1106-1108)."""
    g = gc.load(case)
    t = _tree_anc(g, precision)
    t.infer_ancestral_sequences(marginal=True)
    _, _, res = gc.gtrinf_oracle(g, "marginal")
    _, _, model, _ = gc.inputs_from(g)
    nodes = [n for n in t.tree.find_clades() if n.up is not None]
    L = len(t.data.full_to_compressed_sequence_map)
    for n in nodes[:: max(1, len(nodes) // 8)]:
        got = t.get_branch_mutation_matrix(n)
        want = anc.branch_mutation_matrix(model, res["outgroup_LH"][n.name], res["subtree_LH"][n.name],
                                          anc.branch_length_to_gtr(n, L))
        if precision == "f32":
            np.testing.assert_allclose(got, want, rtol=0, atol=1e-5, err_msg=n.name)
        elif bool(g["site_specific"]):
            # each site's interpolated P_a(t) and the FP64 profiles summed in another order
            np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-12, err_msg=n.name)
        else:
            np.testing.assert_allclose(got, want, rtol=0, atol=1e-12, err_msg=n.name)
        full = t.get_branch_mutation_matrix(n, full_sequence=True)
        assert full.shape == (L,) + got.shape[1:]


def test_infer_gtr_iterative_and_through_reconstruction():
    """infer_gtr_iterative raises the likelihood; infer_ancestral_sequences
    (infer_gtr=True) fits the model before reconstructing."""
    g = gc.load("gtrinf_nuc")
    t = _tree_anc(g)
    t.infer_ancestral_sequences(marginal=True)
    lh0 = t.sequence_LH()
    t.infer_gtr_iterative(max_iter=3, pc=1.0)
    assert t.sequence_LH() >= lh0 - 1e-6
    t2 = _tree_anc(g)
    t2.infer_ancestral_sequences(marginal=True, infer_gtr=True, pc=float(g["pc"]))
    np.testing.assert_allclose(t2.gtr.W, g["marginal_W"], rtol=1e-9)
