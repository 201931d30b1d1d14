"""Loading of the golden fixtures in ``tests/golden`` into product-side inputs."""

import glob
import os

import numpy as np

from treetime_gb300.alphabets import extend_profile
from treetime_gb300.gtr import GTR, GTR_site_specific
from treetime_gb300.tree import parse_newick

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def case_names():
    """Reconstruction cases (every fixture but the branch-length grids)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith("blgrid_"))


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
