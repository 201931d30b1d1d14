"""Loading of the golden fixtures in ``tests/golden`` into product-side inputs."""

import glob
import os

import numpy as np

from treetime_gb300.alphabets import extend_profile
from treetime_gb300.gtr import GTR, GTR_site_specific
from treetime_gb300.tree import parse_newick

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def case_names():
    """Reconstruction cases (every fixture but the branch-length grids and the
    GTR inference cases)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith(("blgrid_", "gtrinf_", "fitch_", "vcf_", "sample_",
                                                          "extra_", "optimize_", "prune_")))


def optimize_cases():
    """(tag, fixture view) of the optimize_tree_marginal fixture: each tree's
    arrays under the unprefixed keys the other fixtures use."""
    g = load("optimize_marginal")
    tags = sorted({k.split("_", 1)[0] for k in g})
    return [(tag, {k[len(tag) + 1:]: v for k, v in g.items() if k.startswith(tag + "_")} | {"kind": "gtr"})
            for tag in tags]


def fitch_names():
    """Fitch parsimony fixtures."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "fitch_*.npz")))


def gtrinf_names():
    """TreeAnc.infer_gtr fixtures."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "gtrinf_*.npz")))


def gtrinf_oracle(g, mode):
    """(n_ija, T_ia, root cseq) of the oracle's counting on the fixture's
    inputs after its own reconstruction in `mode`."""
    from oracle import anc
    tree, aln, model, masks = inputs_from(g)
    anc.prepare_tree(tree)
    if masks:
        for n in anc.preorder(tree.root):
            if n.name in masks:
                n.mask = masks[n.name]
    if bool(g["compress"]):
        caln, mult, full = compress_inputs(aln, model)
    else:
        arrays = {k: anc.seq2array(v, fill_overhangs=True, ambiguous=model.ambiguous) for k, v in aln.items()}
        caln, mult, f2c, _ = anc.compress_alignment(list(arrays), arrays, model.ambiguous)
        extend_profile(model, list(caln.values()))
        full = len(f2c)
    arrays = {k: anc.seq2array(v, fill_overhangs=True, ambiguous=model.ambiguous) for k, v in aln.items()}
    _, _, f2c, _ = anc.compress_alignment(list(arrays), arrays, model.ambiguous)
    if mode == "marginal":
        res = anc.marginal(tree, caln, mult, model, full)
        n_ija, T_ia = anc.substitution_counts_marginal(tree, res, mult, model, full)
        return n_ija, T_ia, res
    res = anc.joint(tree, caln, mult, model, full)
    cseq = dict(res["cseq"])
    cseq.update(caln)
    n_ija, T_ia = anc.substitution_counts_joint(tree, cseq, lambda k: arrays.get(k), np.asarray(f2c), mult, model,
                                                full)
    return n_ija, T_ia, res


def blgrid_names():
    """BranchLenInterpolator fixtures."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "blgrid_*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    return {k: z[k] for k in z.files}


def _scalar(x):
    x = np.asarray(x)
    return x.item() if x.ndim == 0 else x


def model_from(g):
    alphabet = _scalar(g["param_alphabet"])
    if str(g["kind"]) == "gtr":
        m = GTR.custom(mu=float(g["param_mu"]), pi=g["param_pi"], W=g["param_W"], alphabet=alphabet)
    else:
        m = GTR_site_specific(seq_len=g["param_pi"].shape[1], approximate=bool(g["param_approximate"]),
                              alphabet=alphabet)
        m.assign_rates(mu=float(g["param_mu"]), pi=g["param_pi"], W=g["param_W"])
    return m


def inputs_from(g):
    """(tree, aln dict, model, masks or None) rebuilt from a fixture."""
    tree = parse_newick(str(g["newick"]))
    aln = dict(zip(g["aln_names"].tolist(), g["aln_seqs"].tolist()))
    model = model_from(g)
    masks = None
    if "mask_names" in g:
        masks = dict(zip(g["mask_names"].tolist(), list(g["mask_rows"])))
    return tree, aln, model, masks


def compressed_from(g, model):
    """Compressed alignment of the fixture as name -> char array, after
    extending the model's profile map with unknown characters as TreeTime
    does."""
    names = g["compressed_names"].tolist()
    chars = g["compressed_codes"].view("S1").astype("U1")
    aln = {k: chars[i] for i, k in enumerate(names)}
    extend_profile(model, list(aln.values()))
    return aln


def compress_inputs(aln, model):
    """(name -> compressed char array, multiplicities, full length) of a raw
    alignment, by the host compression (pinned bit-exact to TreeTime's)."""
    from treetime_gb300.seqdata import SequenceData
    sd = SequenceData(aln, compress=True, ambiguous=model.ambiguous)
    chars = np.asarray(sd.compressed_codes).view("S1").astype("U1")
    caln = {k: chars[i] for i, k in enumerate(sd.sequence_names)}
    extend_profile(model, list(caln.values()))
    return caln, sd.multiplicity(), len(sd.full_to_compressed_sequence_map)


def blgrid_oracle(g, mode, expm1_form=False):
    """name -> (-log P on the fixture's grid, per-point resolution) by the
    oracle, from the oracle's own reconstruction of the fixture's inputs.
    Resolution: the smallest P(t) entry of the observed state pairs ('joint'),
    1 for 'marginal'."""
    from oracle import anc
    tree, aln, model, _ = inputs_from(g)
    anc.prepare_tree(tree)
    caln, mult, full = compress_inputs(aln, model)
    nodes = {n.name: n for n in anc.preorder(tree.root)}
    out = {}
    if mode == "marginal":
        res = anc.marginal(tree, caln, mult, model, full)
    else:
        res = anc.joint(tree, caln, mult, model, full)
        cseq = dict(res["cseq"])
        cseq.update(caln)
    for i, name in enumerate(g[mode + "_names"].tolist()):
        x = g[mode + "_x"][i, :int(g[mode + "_len"][i])]
        if mode == "marginal":
            v = anc.branch_len_log_prob(model, x, "marginal", profile_pair=(
                res["outgroup_LH"][name], res["subtree_LH"][name]), multiplicity=mult)
            out[name] = (v, np.ones(len(x)))
        else:
            node = nodes[name]
            pairs, pm = anc.state_pair(model, cseq[node.up.name], cseq[name], pattern_multiplicity=mult,
                                       ignore_gaps=True)
            v = anc.branch_len_log_prob(model, x, "joint", seq_pair=pairs, pair_multiplicity=pm,
                                        expm1_form=expm1_form)
            out[name] = (v, anc.pair_resolution(model, x, pairs))
    return out


def codes_of(arr):
    return np.frombuffer(np.asarray(arr).astype("S1").tobytes(), dtype=np.uint8)
