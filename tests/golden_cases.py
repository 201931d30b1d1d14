"""Loading of the golden fixtures in ``tests/golden`` into product-side inputs."""

import glob
import os

import numpy as np

from treetime_gb300.alphabets import extend_profile
from treetime_gb300.gtr import GTR, GTR_site_specific
from treetime_gb300.tree import parse_newick

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def case_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


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


def codes_of(arr):
    return np.frombuffer(np.asarray(arr).astype("S1").tobytes(), dtype=np.uint8)
