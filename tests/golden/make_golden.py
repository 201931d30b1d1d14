"""Generate golden vectors by running the unmodified TreeTime package.

Run in a container where the TreeTime sources are available (they are not
shipped with this repository and are not needed to run the tests):

    python tests/golden/make_golden.py /path/to/treetime-source
    python tests/golden/make_golden.py /path/to/treetime-source --blgrid   (interpolator grids only)
    python tests/golden/make_golden.py /path/to/treetime-source --infer-gtr   (GTR inference only)
    python tests/golden/make_golden.py /path/to/treetime-source --infer-gtr-ss   (inference from a site-specific model)
    python tests/golden/make_golden.py /path/to/treetime-source --fitch   (Fitch parsimony only)
    python tests/golden/make_golden.py /path/to/treetime-source --vcf   (VCF reading and sparse alignments)
    python tests/golden/make_golden.py /path/to/treetime-source --sample   (states drawn at every node)
    python tests/golden/make_golden.py /path/to/treetime-source --extra-sites   (constant sites beyond the alignment)
    python tests/golden/make_golden.py /path/to/treetime-source --optimize   (optimize_tree_marginal iterations)
    python tests/golden/make_golden.py /path/to/treetime-source --prune   (short-branch pruning with a gap)
    python tests/golden/make_golden.py /path/to/treetime-source --optimize-joint   (optimize_tree, joint mode)

Biopython and pandas are replaced by the test-only stand-ins under
``oracle/bioshim``.  Inputs are seeded synthetic workloads from
``treetime_gb300.synth``; each case stores its inputs (Newick text, the
alignment, the raw model parameters) together with TreeTime's outputs in
``tests/golden/<case>.npz``.
"""

import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _setup(ref_path):
    sys.path.insert(0, os.path.join(REPO, "oracle", "bioshim"))
    sys.path.insert(0, ref_path)
    sys.path.insert(0, REPO)


def _bio_inputs(newick, aln):
    from Bio import Phylo
    from Bio.Align import MultipleSeqAlignment
    from Bio.Seq import Seq
    from Bio.SeqRecord import SeqRecord
    tree = Phylo.read(io.StringIO(newick), "newick")
    recs = MultipleSeqAlignment([SeqRecord(Seq(s), id=k, name=k) for k, s in aln.items()])
    return tree, recs


def _codes(chars):
    return np.frombuffer(np.asarray(chars).astype("S1").tobytes(), dtype=np.uint8)


def _ref_gtr(kind, params):
    from treetime import GTR, GTR_site_specific
    alphabet = params["alphabet"]
    if isinstance(alphabet, np.ndarray) and alphabet.ndim == 0:
        alphabet = str(alphabet)
    if kind == "gtr":
        return GTR.custom(mu=params["mu"], pi=params["pi"], W=params["W"], alphabet=alphabet)
    g = GTR_site_specific(seq_len=params["pi"].shape[1], approximate=bool(params["approximate"]),
                          alphabet=alphabet)
    g.assign_rates(mu=params["mu"], pi=params["pi"], W=params["W"])
    return g


def run_case(name, newick, aln, kind, params, compress=True, masks=None, reconstruct_tip_states=False,
             keep_profiles=True, marginal_bl=True, ignore_gaps=True, rng_seed=1234, sample_root=False):
    from treetime import TreeAnc
    out = {"case": name, "newick": newick, "kind": kind, "compress": compress,
           "reconstruct_tip_states": reconstruct_tip_states, "ignore_gaps": ignore_gaps,
           "aln_names": np.array(list(aln.keys())), "aln_seqs": np.array(list(aln.values())),
           "rng_seed": rng_seed, "sample_root": sample_root}
    for k, v in params.items():
        out["param_" + k] = np.asarray(v)

    def make():
        tree, recs = _bio_inputs(newick, aln)
        t = TreeAnc(tree=tree, aln=recs, gtr=_ref_gtr(kind, params), compress=compress, verbose=0,
                    rng_seed=rng_seed, ignore_gaps=ignore_gaps)
        if masks:
            for n in t.tree.find_clades():
                if n.name in masks:
                    n.mask = masks[n.name]
        return t

    # ---- marginal
    t = make()
    g = t.gtr
    out["eigenvals"], out["v"], out["v_inv"] = g.eigenvals, g.v, g.v_inv
    out["W_norm"], out["Pi"], out["mu"] = g.W, g.Pi, g.mu
    out["compressed_names"] = np.array(t.data.sequence_names)
    out["compressed_codes"] = np.stack([_codes(t.data.compressed_alignment[k]) for k in t.data.sequence_names])
    out["multiplicity"] = t.data.multiplicity()
    out["full_to_compressed"] = t.data.full_to_compressed_sequence_map
    nodes = list(t.tree.find_clades())
    out["node_names"] = np.array([n.name for n in nodes])
    out["node_parent"] = np.array([nodes.index(n.up) if n.up is not None else -1 for n in nodes])
    out["node_bl"] = np.array([n.branch_length for n in nodes], dtype=float)
    if masks:
        out["mask_names"] = np.array(list(masks.keys()))
        out["mask_rows"] = np.stack([masks[k] for k in masks])
    ndiff = t.infer_ancestral_sequences(marginal=True, reconstruct_tip_states=reconstruct_tip_states,
                                        sample_from_profile="root" if sample_root else False)
    out["marg_N_diff"] = ndiff
    out["marg_sequence_LH"] = t.tree.sequence_LH
    out["marg_total_LH"] = t.tree.total_sequence_LH
    recon = [n for n in nodes if hasattr(n, "_cseq")]
    out["marg_cseq_names"] = np.array([n.name for n in recon])
    out["marg_cseq"] = np.stack([_codes(n._cseq) for n in recon])
    if keep_profiles:
        inner = [n for n in nodes if not n.is_terminal() or reconstruct_tip_states]
        out["marg_profile_names"] = np.array([n.name for n in inner])
        out["marg_profile"] = np.stack([n.marginal_profile for n in inner])
        out["marg_subtree_names"] = np.array([n.name for n in nodes if not n.is_terminal()])
        out["marg_subtree"] = np.stack([n.marginal_subtree_LH for n in nodes if not n.is_terminal()])
        nr = [n for n in nodes if n.up is not None]
        out["marg_outgroup_names"] = np.array([n.name for n in nr])
        out["marg_outgroup"] = np.stack([n.marginal_outgroup_LH for n in nr])
    # second marginal call: N_diff against the first reconstruction
    out["marg_N_diff_again"] = t.infer_ancestral_sequences(marginal=True,
                                                           reconstruct_tip_states=reconstruct_tip_states)
    if marginal_bl and kind == "gtr":
        nr = [n for n in t.tree.find_clades() if n.up is not None]
        out["mbl_names"] = np.array([n.name for n in nr])
        out["mbl"] = np.array([t.optimal_marginal_branch_length(n) for n in nr])

    # ---- joint
    t = make()
    ndiff = t.infer_ancestral_sequences(marginal=False, reconstruct_tip_states=reconstruct_tip_states, debug=True,
                                        sample_from_profile="root" if sample_root else False)
    nodes = list(t.tree.find_clades())
    out["joint_N_diff"] = ndiff
    out["joint_sequence_LH"] = t.tree.sequence_LH
    out["joint_total_LH"] = t.tree.sequence_joint_LH
    recon = [n for n in nodes if hasattr(n, "_cseq")]
    out["joint_cseq_names"] = np.array([n.name for n in recon])
    out["joint_cseq"] = np.stack([_codes(n._cseq) for n in recon])
    # ---- joint branch lengths (TreeAnc.optimize_branch_lengths_joint)
    if kind == "gtr":
        t.optimize_branch_lengths_joint()
        nr = [n for n in t.tree.find_clades() if n.up is not None]
        out["jbl_names"] = np.array([n.name for n in nr])
        out["jbl"] = np.array([n.branch_length for n in nr])
        if not masks:
            # (TreeTime compares full-length sequences with the compressed-length
            # mask here, which fails for compressed alignments with masks)
            mut = [(n.name, a, int(p), d) for n in nr for (a, p, d) in n.mutations]
            out["mutations"] = np.array(["%s|%s|%d|%s" % m for m in mut])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return out


def run_blgrid(name, newick, aln, kind, params, n_grid_points=125):
    """BranchLenInterpolator grids and values of every branch, in 'marginal'
    mode (after a marginal reconstruction) and in 'joint' mode (after a joint
    one), as ClockTree.init_date_constraints builds them."""
    from treetime import TreeAnc
    from treetime.branch_len_interpolator import BranchLenInterpolator
    out = {"case": name, "newick": newick, "kind": kind, "n_grid_points": n_grid_points,
           "aln_names": np.array(list(aln.keys())), "aln_seqs": np.array(list(aln.values()))}
    for k, v in params.items():
        out["param_" + k] = np.asarray(v)
    for mode in ("marginal", "joint"):
        tree, recs = _bio_inputs(newick, aln)
        t = TreeAnc(tree=tree, aln=recs, gtr=_ref_gtr(kind, params), compress=True, verbose=0)
        t.infer_ancestral_sequences(marginal=mode == "marginal")
        nodes = [n for n in t.tree.find_clades() if n.up is not None]
        xs, ys, peaks, ml = [], [], [], []
        for n in nodes:
            if mode == "marginal":
                n.profile_pair = t.marginal_branch_profile(n)
            else:
                t.add_branch_state(n)
            bi = BranchLenInterpolator(n, t.gtr, pattern_multiplicity=t.data.multiplicity(mask=n.mask),
                                       one_mutation=t.one_mutation, branch_length_mode=mode,
                                       n_grid_points=n_grid_points)
            xs.append(np.asarray(bi._func.x))
            ys.append(np.asarray(bi._func.y))
            peaks.append(bi._peak_val)
            ml.append(n.mutation_length)
        G = max(len(x) for x in xs)
        out[mode + "_names"] = np.array([n.name for n in nodes])
        out[mode + "_mutation_length"] = np.array(ml)
        out[mode + "_len"] = np.array([len(x) for x in xs])
        out[mode + "_x"] = np.stack([np.pad(x, (0, G - len(x)), constant_values=-1.0) for x in xs])
        out[mode + "_y"] = np.stack([np.pad(y, (0, G - len(y))) for y in ys])
        out[mode + "_peak"] = np.array(peaks)
        out["one_mutation"] = t.one_mutation
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return out


def blgrid_cases():
    """Nucleotide tree with a few zero-length branches (both grid shapes) and
    a 5-state alphabet with gaps."""
    from treetime_gb300 import synth
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import to_newick
    rng = np.random.default_rng(21)
    tree = synth.coalescent_tree(20, 0.03, rng)
    pi = rng.dirichlet(np.ones(4))
    W = np.triu(rng.uniform(0.5, 2.0, size=(4, 4)), 1)
    W = W + W.T
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc_nogap")
    states = synth.evolve(tree, g, 150, rng)
    aln = synth._to_text(states, g.alphabet, 0.02, rng)
    for i, c in enumerate(c for c in tree.find_clades() if c is not tree.root):
        if i % 7 == 3:
            c.branch_length = 0.0
    run_blgrid("blgrid_nuc", to_newick(tree), aln, "gtr", {"pi": pi, "W": W, "alphabet": "nuc_nogap", "mu": 1.0})
    rng = np.random.default_rng(22)
    tree = synth.coalescent_tree(14, 0.06, rng)
    pi = rng.dirichlet(np.ones(5))
    W = np.triu(rng.uniform(0.5, 2.0, size=(5, 5)), 1)
    W = W + W.T
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc")
    states = synth.evolve(tree, g, 120, rng)
    aln = synth._to_text(states, g.alphabet, 0.0, rng)
    for k in list(aln)[:4]:
        aln[k] = "-" * 6 + aln[k][6:]
    run_blgrid("blgrid_nuc5", to_newick(tree), aln, "gtr", {"pi": pi, "W": W, "alphabet": "nuc", "mu": 1.0},
               n_grid_points=75)


def run_infer_gtr(name, newick, aln, kind, params, compress=True, masks=None, site_specific=False, pc=5.0):
    """TreeAnc.infer_gtr in 'marginal' and 'joint' mode: the counts TreeTime
    hands to GTR.infer / GTR_site_specific.infer (captured at the call) and the
    inferred model."""
    from treetime import TreeAnc, GTR, GTR_site_specific
    out = {"case": name, "newick": newick, "kind": kind, "compress": compress, "site_specific": site_specific,
           "pc": pc, "aln_names": np.array(list(aln.keys())), "aln_seqs": np.array(list(aln.values()))}
    for k, v in params.items():
        out["param_" + k] = np.asarray(v)
    if masks:
        out["mask_names"] = np.array(list(masks.keys()))
        out["mask_rows"] = np.stack([masks[k] for k in masks])
    cls = GTR_site_specific if site_specific else GTR
    captured = {}
    orig = cls.__dict__["infer"].__func__

    def capture(klass, *args, **kwargs):
        captured["args"] = [np.array(a, copy=True) for a in args]
        captured["root_state"] = np.array(kwargs.get("root_state", args[2] if len(args) > 2 else None), copy=True)
        return orig(klass, *args, **kwargs)

    modes = ("marginal",) if site_specific or masks else ("marginal", "joint")
    for mode in modes:
        tree, recs = _bio_inputs(newick, aln)
        t = TreeAnc(tree=tree, aln=recs, gtr=_ref_gtr(kind, params), compress=compress, verbose=0)
        if masks:
            for n in t.tree.find_clades():
                if n.name in masks:
                    n.mask = masks[n.name]
        t.infer_ancestral_sequences(marginal=mode == "marginal")
        cls.infer = classmethod(capture)
        try:
            g = t.infer_gtr(marginal=mode == "marginal", site_specific=site_specific, pc=pc)
        finally:
            cls.infer = classmethod(orig)
        a = captured["args"]
        out[mode + "_nij"] = a[0]
        out[mode + "_Ti"] = a[1]
        out[mode + "_root_state"] = captured["root_state"]
        out[mode + "_W"], out[mode + "_Pi"], out[mode + "_mu"] = np.asarray(g.W), np.asarray(g.Pi), np.asarray(g.mu)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return out


def infer_gtr_cases():
    """Nucleotides (4 states), 5 states with gaps and ambiguity codes, masks
    (marginal mode) and a site-specific inference from an uncompressed
    protein alignment."""
    from treetime_gb300 import synth
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import to_newick
    rng = np.random.default_rng(31)
    tree = synth.coalescent_tree(24, 0.04, rng)
    pi = rng.dirichlet(np.ones(4))
    W = np.triu(rng.uniform(0.5, 2.0, size=(4, 4)), 1)
    W = W + W.T
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc_nogap")
    states = synth.evolve(tree, g, 300, rng)
    aln = synth._to_text(states, g.alphabet, 0.02, rng)
    nwk = to_newick(tree)
    prm = {"pi": pi, "W": W, "alphabet": "nuc_nogap", "mu": 1.0}
    run_infer_gtr("gtrinf_nuc", nwk, aln, "gtr", prm)
    from treetime_gb300.seqdata import SequenceData
    P = SequenceData(aln, compress=True, ambiguous="N").compressed_length
    names = [c.name for c in tree.find_clades() if c.name][:5]
    masks = {k: (rng.random(P) < 0.7).astype(float) for k in names}
    run_infer_gtr("gtrinf_nuc_masked", nwk, aln, "gtr", prm, masks=masks)

    rng = np.random.default_rng(32)
    tree = synth.coalescent_tree(18, 0.05, rng)
    pi = rng.dirichlet(np.ones(5))
    W = np.triu(rng.uniform(0.5, 2.0, size=(5, 5)), 1)
    W = W + W.T
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc")
    states = synth.evolve(tree, g, 250, rng, invariant_frac=0.4)
    aln = synth._to_text(states, g.alphabet, 0.0, rng)
    for k in list(aln):
        s = np.array(list(aln[k]))
        r = rng.random(len(s))
        s[r < 0.04] = "N"
        s[(r > 0.04) & (r < 0.06)] = rng.choice(list("RYKM"))
        if rng.random() < 0.3:
            s[: rng.integers(1, 8)] = "-"
        aln[k] = "".join(s)
    run_infer_gtr("gtrinf_nuc5", to_newick(tree), aln, "gtr", {"pi": pi, "W": W, "alphabet": "nuc", "mu": 1.0})

    rng = np.random.default_rng(33)
    L = 60
    tree = synth.yule_tree(12, 0.08, rng)
    from treetime_gb300.gtr import GTR_site_specific
    pi_s = rng.dirichlet(np.full(21, 0.5), size=L).T
    W_s = np.triu(rng.uniform(0.1, 5.0, size=(21, 21)), 1)
    W_s = W_s + W_s.T
    gs = GTR_site_specific(seq_len=L, approximate=False, alphabet=synth.AA21)
    gs.assign_rates(mu=1.0, pi=pi_s, W=W_s)
    states = synth.evolve_site_specific(tree, gs, L, rng)
    aln = synth._to_text(states, gs.alphabet, 0.0, rng)
    pi0 = rng.dirichlet(np.ones(21))
    W0 = rng.uniform(0.5, 2.0, size=(21, 21))
    W0 = W0 + W0.T
    run_infer_gtr("gtrinf_aa_ss", to_newick(tree), aln, "gtr",
                  {"pi": pi0, "W": W0, "alphabet": synth.AA21, "mu": 1.0}, compress=False, site_specific=True)


def infer_gtr_ss_current_cases():
    """Marginal GTR inference of a site-specific model whose counts come from a
    site-specific current model (TreeTime's interpolated P(t))."""
    from treetime_gb300 import synth
    from treetime_gb300.gtr import GTR_site_specific
    from treetime_gb300.tree import to_newick
    rng = np.random.default_rng(34)
    L = 60
    tree = synth.yule_tree(14, 0.08, rng)
    pi_s = rng.dirichlet(np.full(21, 0.5), size=L).T
    W_s = np.triu(rng.uniform(0.1, 5.0, size=(21, 21)), 1)
    W_s = W_s + W_s.T
    gs = GTR_site_specific(seq_len=L, approximate=True, alphabet=synth.AA21)
    gs.assign_rates(mu=1.0, pi=pi_s, W=W_s)
    states = synth.evolve_site_specific(tree, gs, L, rng)
    aln = synth._to_text(states, gs.alphabet, 0.02, rng)
    run_infer_gtr("gtrinf_ss_current", to_newick(tree), aln, "ss",
                  {"pi": pi_s, "W": W_s, "alphabet": synth.AA21, "mu": 1.0, "approximate": True}, compress=False,
                  site_specific=True)


def run_fitch(name, newick, aln, kind, params, rng_seed=7):
    """TreeAnc.infer_ancestral_sequences(method='fitch'): the characters of
    every internal node and N_diff, then a second call (N_diff against the
    first) and a marginal reconstruction followed by Fitch (N_diff against
    the marginal sequences)."""
    from treetime import TreeAnc
    out = {"case": name, "newick": newick, "kind": kind, "rng_seed": rng_seed,
           "aln_names": np.array(list(aln.keys())), "aln_seqs": np.array(list(aln.values()))}
    for k, v in params.items():
        out["param_" + k] = np.asarray(v)
    tree, recs = _bio_inputs(newick, aln)
    t = TreeAnc(tree=tree, aln=recs, gtr=_ref_gtr(kind, params), compress=True, verbose=0, rng_seed=rng_seed)
    out["fitch_N_diff"] = t.infer_ancestral_sequences(method="fitch")
    inner = [n for n in t.tree.find_clades() if not n.is_terminal()]
    out["fitch_names"] = np.array([n.name for n in inner])
    out["fitch_cseq"] = np.stack([_codes(n._cseq) for n in inner])
    out["fitch_N_diff_again"] = t.infer_ancestral_sequences(method="fitch")
    out["fitch_cseq_again"] = np.stack([_codes(n._cseq) for n in inner])
    tree, recs = _bio_inputs(newick, aln)
    t = TreeAnc(tree=tree, aln=recs, gtr=_ref_gtr(kind, params), compress=True, verbose=0, rng_seed=rng_seed)
    t.infer_ancestral_sequences(marginal=True)
    out["fitch_after_marginal_N_diff"] = t.infer_ancestral_sequences(method="fitch")
    out["fitch_after_marginal_cseq"] = np.stack([_codes(n._cseq) for n in t.tree.find_clades()
                                                 if not n.is_terminal()])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return out


def fitch_cases():
    """Binary nucleotide tree; polytomies with ambiguity codes, N and gaps
    (characters outside the alphabet, repeated union entries); amino acids."""
    from treetime_gb300 import synth
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import to_newick
    rng = np.random.default_rng(41)
    tree = synth.coalescent_tree(30, 0.05, rng)
    g = GTR.custom(mu=1.0, pi=np.ones(4), W=np.ones((4, 4)), alphabet="nuc_nogap")
    states = synth.evolve(tree, g, 200, rng)
    aln = synth._to_text(states, g.alphabet, 0.0, rng)
    run_fitch("fitch_nuc", to_newick(tree), aln, "gtr", {"pi": np.ones(4), "W": np.ones((4, 4)),
                                                          "alphabet": "nuc_nogap", "mu": 1.0})
    rng = np.random.default_rng(42)
    tree = synth.coalescent_tree(22, 0.08, rng)
    inner = [c for c in tree.find_clades(order="postorder") if c.clades and c is not tree.root]
    for c in inner[:4]:
        for par in tree.find_clades():
            if c in par.clades:
                i = par.clades.index(c)
                par.clades[i:i + 1] = c.clades
                break
    pi = rng.dirichlet(np.ones(5))
    W = np.triu(rng.uniform(0.5, 2.0, size=(5, 5)), 1)
    W = W + W.T
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc")
    states = synth.evolve(tree, g, 150, rng)
    aln = synth._to_text(states, g.alphabet, 0.0, rng)
    for k in list(aln):
        s = np.array(list(aln[k]))
        r = rng.random(len(s))
        s[r < 0.05] = "N"
        s[(r > 0.05) & (r < 0.08)] = rng.choice(list("RYKMSW"))
        aln[k] = "".join(s)
    run_fitch("fitch_poly", to_newick(tree), aln, "gtr", {"pi": pi, "W": W, "alphabet": "nuc", "mu": 1.0})
    rng = np.random.default_rng(43)
    tree = synth.coalescent_tree(16, 0.2, rng)
    pi = rng.random(20)
    W = rng.random((20, 20))
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="aa_nogap")
    states = synth.evolve(tree, g, 100, rng)
    aln = synth._to_text(states, g.alphabet, 0.0, rng)
    run_fitch("fitch_aa", to_newick(tree), aln, "gtr", {"pi": pi, "W": W, "alphabet": "aa_nogap", "mu": 1.0})


def _vcf_haploid(path, ref, aln, rng):
    """A haploid VCF of an alignment's differences from `ref`: one line per
    variable column, ALT alleles in order of appearance, deletions of runs of
    gaps after a reference base written as REF/ALT indels, N as no-calls."""
    names = list(aln)
    L = len(ref)
    lines = ["##fileformat=VCFv4.2", "##source=synthetic",
             "#CHROM\tPOS\tID\tREF\tALT\tQUAL\tFILTER\tINFO\tFORMAT\t" + "\t".join(names)]
    pos = 0
    while pos < L:
        col = [aln[k][pos] for k in names]
        dels = [k for k in names if aln[k][pos] == "-"]
        if dels and pos > 0 and pos + 1 < L and all(aln[k][pos - 1] == ref[pos - 1] for k in dels) \
                and rng.random() < 0.5:
            # a one-base deletion written against the previous reference base
            r = ref[pos - 1:pos + 1]
            calls = ["1" if aln[k][pos] == "-" else "0" for k in names]
            lines.append("chr1\t%d\t.\t%s\t%s\t.\tPASS\t.\tGT\t%s" % (pos, r, r[0], "\t".join(calls)))
            pos += 1
            continue
        alts = []
        calls = []
        for c in col:
            if c == ref[pos]:
                calls.append("0")
            elif c == "N":
                calls.append(".")
            else:
                a = "*" if c == "-" else c
                if a not in alts:
                    alts.append(a)
                calls.append(str(alts.index(a) + 1))
        if alts or "." in calls:
            lines.append("chr1\t%d\t.\t%s\t%s\t.\tPASS\t.\tGT\t%s" % (pos + 1, ref[pos], ",".join(alts) or ".",
                                                                        "\t".join(calls)))
        pos += 1
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def _vcf_diploid(path):
    """A diploid VCF with every kind of call TreeTime's reader distinguishes:
    homozygous and heterozygous substitutions, no-calls, deletions,
    insertions (with and without a first-base change), insertion plus
    deletion, '*' and '.' alleles, an invalid allele and a non-GT line."""
    samples = ["s1", "s2", "s3", "s4"]
    rows = [
        (3, "A", "G", ["1/1", "0/1", "./.", "0/0"]),
        (6, "C", "T,G", ["2/2", "1|1", "0/2", "./."]),
        (10, "GTA", "G", ["1/1", "0/1", "./.", "0/0"]),
        (15, "T", "TAC", ["1/1", "0/1", "0/0", "./."]),
        (18, "A", "GCC", ["1/1", "0/0", "0/0", "0/0"]),
        (22, "GC", "GCC,G", ["1/1", "2/2", "0/1", "0/0"]),
        (25, "T", "*", ["1/1", "0/0", "0/0", "0/0"]),
        (27, "C", ".", ["1/1", "0/0", "0/0", "0/0"]),
        (29, "A", "<DEL>", ["1/1", "0/0", "0/0", "0/0"]),
        (31, "G", "a", ["1/1", "0/0", "1/1", "0/0"]),
        (33, "T", "C", ["0/0", "0/0", "1/1", "1/1"]),
        (35, "CA", "C,CTT", ["./.", "0/2", "2/2", "1/1"]),
    ]
    lines = ["##fileformat=VCFv4.2", "#CHROM\tPOS\tID\tREF\tALT\tQUAL\tFILTER\tINFO\tFORMAT\t" +
             "\t".join(samples)]
    for pos, r, a, calls in rows:
        lines.append("chr1\t%d\t.\t%s\t%s\t.\tPASS\t.\tGT:DP\t%s" % (pos, r, a,
                                                                       "\t".join(c + ":7" for c in calls)))
    lines.append("chr1\t37\t.\tA\tT\t.\tPASS\t.\tDP\t3\t3\t3\t3")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def vcf_cases(ref_path):
    """read_vcf on a diploid file exercising every call type and on a haploid
    file derived from a simulated alignment; for the latter also the sparse
    compression of SequenceData and a marginal reconstruction by TreeAnc."""
    import tempfile
    from treetime import TreeAnc
    from treetime.vcf_utils import read_vcf
    from treetime_gb300 import synth
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import to_newick

    def flat(d):
        keys = sorted((k, p) for k, v in d.items() for p in v)
        return (np.array([k for k, _ in keys]), np.array([p for _, p in keys], dtype=np.int64),
                np.array([d[k][p] for k, p in keys]))

    tmp = tempfile.mkdtemp()
    out = {}
    # diploid
    vcf = os.path.join(tmp, "d.vcf")
    _vcf_diploid(vcf)
    res = read_vcf(vcf)
    out["d_vcf_text"] = np.array(open(vcf).read())
    out["d_seq_name"], out["d_seq_pos"], out["d_seq_chr"] = flat(res["sequences"])
    out["d_ins_name"], out["d_ins_pos"], out["d_ins_str"] = flat(res["insertions"])
    out["d_ins_keys"] = np.array(sorted(res["insertions"].keys()))
    out["d_positions"] = np.array(res["positions"], dtype=np.int64)
    out["d_ploidy"] = res["metadata"]["ploidy"]
    out["d_chrom"] = res["metadata"]["chrom"]
    # haploid, from a simulated alignment
    rng = np.random.default_rng(51)
    tree = synth.coalescent_tree(20, 0.02, rng)
    g = GTR.custom(mu=1.0, pi=np.ones(5), W=np.ones((5, 5)), alphabet="nuc")
    L = 400
    states = synth.evolve(tree, g, L, rng)
    aln = synth._to_text(states, g.alphabet, 0.0, rng)
    ref = "".join(rng.choice(list("ACGT"), size=L))
    ref = "".join(max("ACGT", key=lambda c: sum(aln[k][i] == c for k in aln)) if rng.random() < 0.9 else ref[i]
                  for i in range(L))
    ref = ref[:100] + "NN" + ref[102:]
    for k in list(aln):
        s = np.array(list(aln[k]))
        r = rng.random(L)
        s[r < 0.02] = "N"
        aln[k] = "".join(s)
    vcf = os.path.join(tmp, "h.vcf")
    _vcf_haploid(vcf, ref, aln, rng)
    fa = os.path.join(tmp, "ref.fasta")
    with open(fa, "w") as fh:
        fh.write(">ref\n" + ref + "\n")
    res = read_vcf(vcf, fa)
    out["h_vcf_text"] = np.array(open(vcf).read())
    out["h_ref"] = np.array(res["reference"])
    out["h_seq_name"], out["h_seq_pos"], out["h_seq_chr"] = flat(res["sequences"])
    out["h_names"] = np.array(list(res["sequences"].keys()))
    out["h_positions"] = np.array(res["positions"], dtype=np.int64)
    nwk = to_newick(tree)
    out["h_newick"] = np.array(nwk)
    from Bio import Phylo
    gtr_nuc = _ref_gtr("gtr", {"pi": np.ones(5), "W": np.ones((5, 5)), "alphabet": "nuc", "mu": 1.0})
    t = TreeAnc(tree=Phylo.read(io.StringIO(nwk), "newick"), aln=res["sequences"], ref=res["reference"],
                gtr=gtr_nuc, verbose=0)
    d = t.data
    out["h_comp_names"] = np.array(list(d.compressed_alignment.keys()))
    out["h_comp_codes"] = np.stack([_codes(d.compressed_alignment[k]) for k in d.compressed_alignment])
    out["h_mult"] = d.multiplicity()
    out["h_f2c"] = d.full_to_compressed_sequence_map
    out["h_const_amb"] = np.array(sorted(d.inferred_const_sites), dtype=np.int64)
    t.infer_ancestral_sequences(marginal=True)
    out["h_marg_total_LH"] = t.tree.total_sequence_LH
    out["h_marg_sequence_LH"] = t.tree.sequence_LH
    np.savez_compressed(os.path.join(HERE, "vcf_cases.npz"), **out)


def run_sample(name, newick, aln, kind, params, rng_seed=5):
    """Marginal reconstruction with sample_from_profile=True (every node's
    state drawn from its profile with TreeTime's generator), without and with
    tip states, and a second call (N_diff against the first)."""
    from treetime import TreeAnc
    out = {"case": name, "newick": newick, "kind": kind, "rng_seed": rng_seed,
           "aln_names": np.array(list(aln.keys())), "aln_seqs": np.array(list(aln.values()))}
    for k, v in params.items():
        out["param_" + k] = np.asarray(v)
    for tips in (False, True):
        tree, recs = _bio_inputs(newick, aln)
        t = TreeAnc(tree=tree, aln=recs, gtr=_ref_gtr(kind, params), compress=True, verbose=0, rng_seed=rng_seed)
        tag = "tips" if tips else "inner"
        out[tag + "_N_diff"] = t.infer_ancestral_sequences(marginal=True, sample_from_profile=True,
                                                            reconstruct_tip_states=tips)
        nodes = [n for n in t.tree.find_clades() if hasattr(n, "_cseq") and n._cseq is not None]
        out[tag + "_names"] = np.array([n.name for n in nodes])
        out[tag + "_cseq"] = np.stack([_codes(n._cseq) for n in nodes])
        out[tag + "_N_diff_again"] = t.infer_ancestral_sequences(marginal=True, sample_from_profile=True,
                                                                  reconstruct_tip_states=tips)
        out[tag + "_cseq_again"] = np.stack([_codes(n._cseq) for n in nodes])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def sample_cases():
    from treetime_gb300 import synth
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import to_newick
    rng = np.random.default_rng(61)
    tree = synth.coalescent_tree(24, 0.08, rng)
    pi = rng.dirichlet(np.ones(5))
    W = np.triu(rng.uniform(0.5, 2.0, size=(5, 5)), 1)
    W = W + W.T
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc")
    states = synth.evolve(tree, g, 150, rng)
    aln = synth._to_text(states, g.alphabet, 0.02, rng)
    run_sample("sample_nuc5", to_newick(tree), aln, "gtr", {"pi": pi, "W": W, "alphabet": "nuc", "mu": 1.0})


def extra_sites_cases():
    """seq_len beyond the alignment (additional constant sites): TreeTime's
    compressed alignment and marginal log-likelihood, nucleotides and amino
    acids."""
    from treetime import TreeAnc
    from treetime_gb300 import synth
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import to_newick
    out = {}
    for tag, alphabet, q, seed, extra in (("nuc", "nuc", 5, 71, 1234), ("aa", "aa", 21, 72, 77)):
        rng = np.random.default_rng(seed)
        tree = synth.coalescent_tree(14, 0.05, rng)
        pi = rng.dirichlet(np.ones(q))
        W = np.triu(rng.uniform(0.5, 2.0, size=(q, q)), 1)
        W = W + W.T
        g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet=alphabet)
        aln = synth._to_text(synth.evolve(tree, g, 90, rng), g.alphabet, 0.03, rng)
        nwk = to_newick(tree)
        params = {"pi": pi, "W": W, "alphabet": alphabet, "mu": 1.0}
        tr, recs = _bio_inputs(nwk, aln)
        t = TreeAnc(tree=tr, aln=recs, gtr=_ref_gtr("gtr", params), verbose=0, seq_len=90 + extra)
        d = t.data
        out[tag + "_newick"] = np.array(nwk)
        out[tag + "_aln_names"] = np.array(list(aln.keys()))
        out[tag + "_aln_seqs"] = np.array(list(aln.values()))
        for k, v in params.items():
            out[tag + "_param_" + k] = np.asarray(v)
        out[tag + "_seq_len"] = 90 + extra
        out[tag + "_comp_names"] = np.array(list(d.compressed_alignment.keys()))
        out[tag + "_comp_codes"] = np.stack([_codes(d.compressed_alignment[k]) for k in d.compressed_alignment])
        out[tag + "_mult"] = d.multiplicity()
        out[tag + "_f2c"] = d.full_to_compressed_sequence_map
        t.infer_ancestral_sequences(marginal=True)
        out[tag + "_marg_total_LH"] = t.tree.total_sequence_LH
    np.savez_compressed(os.path.join(HERE, "extra_sites.npz"), **out)


def optimize_cases():
    """TreeAnc.optimize_tree_marginal: the branch lengths, log-likelihood and
    sequences after TreeTime's damped marginal iterations, on a tree with a
    bifurcating root (its two children optimised as one branch) and on one
    with a trifurcating root."""
    from treetime import TreeAnc
    from treetime_gb300 import synth
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import to_newick
    out = {}
    for tag, seed, collapse in (("bif", 81, False), ("tri", 82, True)):
        rng = np.random.default_rng(seed)
        tree = synth.coalescent_tree(20, 0.05, rng)
        if collapse:  # merge the root's first internal child into the root
            first = next(c for c in tree.root.clades if c.clades)
            tree.root.clades = [c for c in tree.root.clades if c is not first] + first.clades
        pi = rng.dirichlet(np.ones(4))
        W = np.triu(rng.uniform(0.5, 2.0, size=(4, 4)), 1)
        W = W + W.T
        g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc_nogap")
        aln = synth._to_text(synth.evolve(tree, g, 300, rng), g.alphabet, 0.0, rng)
        nwk = to_newick(tree)
        params = {"pi": pi, "W": W, "alphabet": "nuc_nogap", "mu": 1.0}
        tr, recs = _bio_inputs(nwk, aln)
        t = TreeAnc(tree=tr, aln=recs, gtr=_ref_gtr("gtr", params), verbose=0)
        t.optimize_tree_marginal(max_iter=4)
        nodes = list(t.tree.find_clades())
        out[tag + "_newick"] = np.array(nwk)
        out[tag + "_aln_names"] = np.array(list(aln.keys()))
        out[tag + "_aln_seqs"] = np.array(list(aln.values()))
        for k, v in params.items():
            out[tag + "_param_" + k] = np.asarray(v)
        out[tag + "_root_children"] = len(t.tree.root.clades)
        out[tag + "_node_names"] = np.array([n.name for n in nodes])
        out[tag + "_node_bl"] = np.array([n.branch_length for n in nodes], dtype=float)
        out[tag + "_total_LH"] = t.tree.total_sequence_LH
        inner = [n for n in nodes if n.clades]
        out[tag + "_cseq_names"] = np.array([n.name for n in inner])
        out[tag + "_cseq"] = np.stack([_codes(n._cseq) for n in inner])
    np.savez_compressed(os.path.join(HERE, "optimize_marginal.npz"), **out)


def prune_cases():
    """TreeAnc.prune_short_branches on a tree with two consecutive short
    internal branches (P -> X -> G) whose reconstructed sequences are set so
    that X equals P except for a gap, and G equals X except where X has the
    gap: X is collapsed (the gap is ignored), after which TreeTime compares G
    with its new parent P, where they differ, and keeps G."""
    from treetime import TreeAnc, GTR
    nwk = "((((t1:0.1,t2:0.1)G:0.0001,t3:0.1)X:0.0001,t4:0.1)P:0.1,(t5:0.1,t6:0.1)Q:0.1)R;"
    rng = np.random.default_rng(91)
    L = 40
    base = rng.choice(list("ACGT"), size=L)
    aln = {}
    for k in range(1, 7):
        seq = base.copy()
        seq[rng.integers(L, size=2)] = rng.choice(list("ACGT"), size=2)
        aln["t%d" % k] = "".join(seq)
    tr, recs = _bio_inputs(nwk, aln)
    t = TreeAnc(tree=tr, aln=recs, gtr=GTR.standard("JC69", alphabet="nuc"), verbose=0)
    t.infer_ancestral_sequences(marginal=False)
    nodes = {n.name: n for n in t.tree.find_clades()}
    p_seq = np.array(list("A" * t.data.compressed_length))
    x_seq = p_seq.copy()
    x_seq[0] = "-"
    g_seq = x_seq.copy()
    g_seq[0] = "C"
    nodes["P"]._cseq, nodes["X"]._cseq, nodes["G"]._cseq = p_seq, x_seq, g_seq
    inner = [n for n in t.tree.find_clades() if n.clades]
    out = {"newick": np.array(nwk), "aln_names": np.array(list(aln.keys())),
           "aln_seqs": np.array(list(aln.values())), "one_mutation": t.one_mutation,
           "multiplicity": t.data.multiplicity(),
           "cseq_names": np.array([n.name for n in inner]),
           "cseq": np.stack([_codes(n._cseq) for n in inner])}
    t.prune_short_branches()
    after = list(t.tree.find_clades())
    out["node_names"] = np.array([n.name for n in after])
    out["parent_names"] = np.array([n.up.name if n.up is not None else "" for n in after])
    np.savez_compressed(os.path.join(HERE, "prune_gaps.npz"), **out)


def optimize_joint_cases():
    """TreeAnc.optimize_tree(branch_length_mode='joint', prune_short=True): the
    topology, branch lengths, sequences and unconstrained log-likelihood after
    TreeTime's joint iterations, on a tree with many branches without
    mutations (pruned to polytomies)."""
    from treetime import TreeAnc
    from treetime_gb300 import synth
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import to_newick
    rng = np.random.default_rng(95)
    tree = synth.coalescent_tree(30, 0.004, rng)
    pi = rng.dirichlet(np.ones(4))
    W = np.triu(rng.uniform(0.5, 2.0, size=(4, 4)), 1)
    W = W + W.T
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc_nogap")
    aln = synth._to_text(synth.evolve(tree, g, 250, rng), g.alphabet, 0.0, rng)
    nwk = to_newick(tree)
    params = {"pi": pi, "W": W, "alphabet": "nuc_nogap", "mu": 1.0}
    tr, recs = _bio_inputs(nwk, aln)
    t = TreeAnc(tree=tr, aln=recs, gtr=_ref_gtr("gtr", params), verbose=0)
    n_before = sum(1 for _ in t.tree.find_clades())
    t.optimize_tree(branch_length_mode="joint", max_iter=3, prune_short=True)
    nodes = list(t.tree.find_clades())
    out = {"newick": np.array(nwk), "aln_names": np.array(list(aln.keys())),
           "aln_seqs": np.array(list(aln.values())), "kind": np.array("gtr"),
           "one_mutation": t.one_mutation, "n_nodes_before": n_before}
    for k, v in params.items():
        out["param_" + k] = np.asarray(v)
    out["node_names"] = np.array([n.name for n in nodes])
    out["parent_names"] = np.array([n.up.name if n.up is not None else "" for n in nodes])
    out["node_bl"] = np.array([n.branch_length for n in nodes], dtype=float)
    out["unconstrained_LH"] = t.tree.unconstrained_sequence_LH
    inner = [n for n in nodes if n.clades]
    out["cseq_names"] = np.array([n.name for n in inner])
    out["cseq"] = np.stack([_codes(n._cseq) for n in inner])
    np.savez_compressed(os.path.join(HERE, "optimize_joint.npz"), **out)


def main(ref_path):
    _setup(ref_path)
    from treetime_gb300 import synth
    from treetime_gb300.tree import to_newick

    def gtr_params(g, raw_pi, raw_W, alphabet, mu=1.0, approximate=None):
        d = {"pi": raw_pi, "W": raw_W, "alphabet": alphabet if isinstance(alphabet, str) else np.asarray(alphabet),
             "mu": mu}
        if approximate is not None:
            d["approximate"] = approximate
        return d

    # c0-shaped, small
    rng = np.random.default_rng(11)
    tree = synth.coalescent_tree(24, 0.02, rng)
    pi = rng.dirichlet(np.ones(4))
    W = np.triu(rng.uniform(0.5, 2.0, size=(4, 4)), 1)
    W = W + W.T
    from treetime_gb300.gtr import GTR
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc_nogap")
    states = synth.evolve(tree, g, 120, rng)
    aln = synth._to_text(states, g.alphabet, 0.05, rng)
    nwk = to_newick(tree)
    run_case("c0_small", nwk, aln, "gtr", gtr_params(g, pi, W, "nuc_nogap"))
    run_case("c0_small_tips", nwk, aln, "gtr", gtr_params(g, pi, W, "nuc_nogap"), reconstruct_tip_states=True)
    run_case("c0_small_sample", nwk, aln, "gtr", gtr_params(g, pi, W, "nuc_nogap"), sample_root=True,
             marginal_bl=False)

    # 5-state alphabet with gaps, ambiguity codes and invariant columns
    rng = np.random.default_rng(12)
    tree = synth.coalescent_tree(20, 0.05, rng)
    pi = rng.dirichlet(np.ones(5))
    W = np.triu(rng.uniform(0.5, 2.0, size=(5, 5)), 1)
    W = W + W.T
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc")
    states = synth.evolve(tree, g, 200, rng, invariant_frac=0.5)
    aln = synth._to_text(states, g.alphabet, 0.0, rng)
    names = list(aln)
    for k in names:
        s = np.array(list(aln[k]))
        r = rng.random(len(s))
        s[r < 0.03] = "N"
        s[(r > 0.03) & (r < 0.05)] = rng.choice(list("RYKMSW"))
        if rng.random() < 0.3:
            s[: rng.integers(1, 10)] = "-"
        aln[k] = "".join(s)
    run_case("nuc5", to_newick(tree), aln, "gtr", gtr_params(g, pi, W, "nuc"))

    # masks on a few branches
    rng = np.random.default_rng(13)
    tree = synth.coalescent_tree(16, 0.03, rng)
    pi = rng.dirichlet(np.ones(4))
    W = np.triu(rng.uniform(0.5, 2.0, size=(4, 4)), 1)
    W = W + W.T
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc_nogap")
    states = synth.evolve(tree, g, 120, rng)
    aln = synth._to_text(states, g.alphabet, 0.0, rng)
    tree_names = [c.name for c in tree.find_clades() if c.name]
    masks = {}
    for k in tree_names[:6]:
        masks[k] = None
    # the compressed length is only known after compression: run once to get it
    from treetime_gb300.seqdata import SequenceData
    P = SequenceData(aln, compress=True, ambiguous="N").compressed_length
    masks = {k: (rng.random(P) < 0.7).astype(float) for k in tree_names[:6]}
    run_case("masked", to_newick(tree), aln, "gtr", gtr_params(g, pi, W, "nuc_nogap"), masks=masks,
             marginal_bl=False)

    # polytomies, a tip without sequence, an unknown character
    rng = np.random.default_rng(14)
    tree = synth.coalescent_tree(18, 0.04, rng)
    inner = [c for c in tree.find_clades(order="postorder") if c.clades and c is not tree.root]
    for c in inner[:3]:
        # collapse: splice the clade's children into its parent
        for par in tree.find_clades():
            if c in par.clades:
                i = par.clades.index(c)
                par.clades[i:i + 1] = c.clades
                break
    g = GTR.custom(mu=1.0, pi=np.ones(4), W=np.ones((4, 4)), alphabet="nuc_nogap")
    states = synth.evolve(tree, g, 100, rng)
    aln = synth._to_text(states, g.alphabet, 0.02, rng)
    first = list(aln)[0]
    del aln[first]
    k2 = list(aln)[1]
    s = list(aln[k2])
    s[5] = "?"
    aln[k2] = "".join(s)
    run_case("polytomy", to_newick(tree), aln, "gtr", gtr_params(g, np.ones(4), np.ones((4, 4)), "nuc_nogap"),
             reconstruct_tip_states=True)

    # 22-state amino-acid alphabet, standard GTR (large-alphabet state_pair branch)
    rng = np.random.default_rng(15)
    tree = synth.coalescent_tree(12, 0.1, rng)
    pi = rng.random(22)
    W = rng.random((22, 22))
    g = GTR.custom(mu=1.0, pi=pi, W=W, alphabet="aa")
    states = synth.evolve(tree, g, 80, rng)
    aln = synth._to_text(states, g.alphabet, 0.0, rng)
    k = list(aln)[2]
    s = list(aln[k])
    s[3] = "X"
    s[4] = "B"
    aln[k] = "".join(s)
    run_case("aa22", to_newick(tree), aln, "gtr", gtr_params(g, pi, W, "aa"))

    # site-specific protein model, both P(t) paths
    rng = np.random.default_rng(16)
    L = 40
    tree = synth.yule_tree(14, 0.05, rng)
    pi = rng.dirichlet(np.full(21, 0.5), size=L).T
    W = np.triu(rng.uniform(0.1, 5.0, size=(21, 21)), 1)
    W = W + W.T
    from treetime_gb300.gtr import GTR_site_specific
    g = GTR_site_specific(seq_len=L, approximate=True, alphabet=synth.AA21)
    g.assign_rates(mu=1.0, pi=pi, W=W)
    states = synth.evolve_site_specific(tree, g, L, rng)
    aln = synth._to_text(states, g.alphabet, 0.0, rng)
    for approx in (True, False):
        run_case("aa_site_specific_%s" % ("interp" if approx else "exact"), to_newick(tree), aln, "ss",
                 gtr_params(g, pi, W, synth.AA21, approximate=approx), compress=False, marginal_bl=False)

    # full-size C0 workload: sequences, likelihoods and branch lengths only
    wl = synth.make_workload("c0", seed=0)
    g = wl["gtr"]
    rng = np.random.default_rng(0)
    # make_workload's model draws: recover the raw parameters by re-drawing
    tree = synth.coalescent_tree(100, 0.01, rng)
    pi = rng.dirichlet(np.ones(4))
    W = rng.uniform(0.5, 2.0, size=(4, 4))
    W = np.triu(W, 1)
    W = W + W.T
    assert np.allclose(GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc_nogap").W, g.W)
    run_case("c0_full", to_newick(wl["tree"]), wl["aln"], "gtr", gtr_params(g, pi, W, "nuc_nogap"),
             keep_profiles=False, marginal_bl=False)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref = args[0] if args else os.environ.get("TREETIME_SOURCE")
    if not ref:
        sys.exit("usage: make_golden.py <path of the TreeTime sources> [--case flag] "
                 "(or set TREETIME_SOURCE)")
    if "--blgrid" in sys.argv:
        _setup(ref)
        blgrid_cases()
    elif "--infer-gtr-ss" in sys.argv:
        _setup(ref)
        infer_gtr_ss_current_cases()
    elif "--infer-gtr" in sys.argv:
        _setup(ref)
        infer_gtr_cases()
    elif "--fitch" in sys.argv:
        _setup(ref)
        fitch_cases()
    elif "--vcf" in sys.argv:
        _setup(ref)
        vcf_cases(ref)
    elif "--sample" in sys.argv:
        _setup(ref)
        sample_cases()
    elif "--extra-sites" in sys.argv:
        _setup(ref)
        extra_sites_cases()
    elif "--optimize" in sys.argv and "--optimize-joint" not in sys.argv:
        _setup(ref)
        optimize_cases()
    elif "--prune" in sys.argv:
        _setup(ref)
        prune_cases()
    elif "--optimize-joint" in sys.argv:
        _setup(ref)
        optimize_joint_cases()
    else:
        main(ref)
