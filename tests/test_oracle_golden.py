"""Pin the CPU oracle (``oracle/anc.py``) and the host-side set-up code
against golden vectors produced by running TreeTime itself
(``tests/golden/make_golden.py``).  CPU only."""

import numpy as np
import pytest

import golden_cases as gc
from oracle import anc
from treetime_gb300.seqdata import SequenceData
from treetime_gb300.alphabets import extend_profile

CASES = gc.case_names()


def _names_map(names, arr):
    return {str(k): arr[i] for i, k in enumerate(names)}


def _prepared(g):
    tree, aln, model, masks = gc.inputs_from(g)
    anc.prepare_tree(tree)
    if masks:
        for n in anc.preorder(tree.root):
            if n.name in masks:
                n.mask = masks[n.name]
    return tree, aln, model, masks


@pytest.mark.parametrize("case", CASES)
def test_tree_preparation_names_and_order(case):
    g = gc.load(case)
    tree, _, _, _ = _prepared(g)
    nodes = list(anc.preorder(tree.root))
    assert [n.name for n in nodes] == g["node_names"].tolist()
    parent = [nodes.index(n.up) if n.up is not None else -1 for n in nodes]
    assert parent == g["node_parent"].tolist()


@pytest.mark.parametrize("case", CASES)
def test_model_eigendecomposition(case):
    g = gc.load(case)
    m = gc.model_from(g)
    np.testing.assert_allclose(m.W, g["W_norm"], rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(m.Pi, g["Pi"], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(m.mu, g["mu"], rtol=1e-14)
    np.testing.assert_allclose(m.eigenvals, g["eigenvals"], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(m.v, g["v"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(m.v_inv, g["v_inv"], rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("case", CASES)
def test_host_compression_bit_exact(case):
    g = gc.load(case)
    _, aln, model, _ = gc.inputs_from(g)
    sd = SequenceData(aln, compress=bool(g["compress"]), ambiguous=model.ambiguous)
    assert sd.sequence_names == g["compressed_names"].tolist()
    np.testing.assert_array_equal(sd.compressed_codes, g["compressed_codes"])
    np.testing.assert_array_equal(sd.multiplicity(), g["multiplicity"])
    np.testing.assert_array_equal(sd.full_to_compressed_sequence_map, g["full_to_compressed"])


@pytest.mark.parametrize("case", [c for c in CASES if not c.startswith("aa_site")])
def test_oracle_compression_restatement(case):
    g = gc.load(case)
    _, aln, model, _ = gc.inputs_from(g)
    arrays = {k: anc.seq2array(v, fill_overhangs=True, ambiguous=model.ambiguous) for k, v in aln.items()}
    comp, mult, f2c, _ = anc.compress_alignment(list(arrays), arrays, model.ambiguous)
    chars = g["compressed_codes"].view("S1").astype("U1")
    for i, k in enumerate(g["compressed_names"].tolist()):
        np.testing.assert_array_equal(comp[k], chars[i])
    np.testing.assert_array_equal(mult, g["multiplicity"])
    np.testing.assert_array_equal(f2c, g["full_to_compressed"])


@pytest.mark.parametrize("case", CASES)
def test_oracle_marginal_matches_treetime(case):
    g = gc.load(case)
    tree, _, model, _ = _prepared(g)
    aln = gc.compressed_from(g, model)
    rng = np.random.default_rng(int(g["rng_seed"]))
    res = anc.marginal(tree, aln, g["multiplicity"], model, len(g["full_to_compressed"]),
                       sample_from_profile="root" if bool(g["sample_root"]) else False,
                       reconstruct_tip_states=bool(g["reconstruct_tip_states"]), rng=rng)
    np.testing.assert_allclose(res["sequence_LH"], g["marg_sequence_LH"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(res["total_sequence_LH"], g["marg_total_LH"], rtol=1e-13)
    assert res["N_diff"] == int(g["marg_N_diff"])
    want = _names_map(g["marg_cseq_names"], g["marg_cseq"])
    assert set(want) == set(res["cseq"])
    for k, v in want.items():
        np.testing.assert_array_equal(gc.codes_of(res["cseq"][k]), v, err_msg=k)
    if "marg_profile" in g:
        for key, gk in (("profile", "marg_profile"), ("subtree_LH", "marg_subtree"), ("outgroup_LH", "marg_outgroup")):
            want = _names_map(g[gk + "_names"], g[gk])
            for k, v in want.items():
                np.testing.assert_allclose(res[key][k], v, rtol=1e-10, atol=1e-13, err_msg="%s %s" % (key, k))


@pytest.mark.parametrize("case", CASES)
def test_oracle_joint_matches_treetime(case):
    g = gc.load(case)
    tree, _, model, _ = _prepared(g)
    aln = gc.compressed_from(g, model)
    rng = np.random.default_rng(int(g["rng_seed"]))
    res = anc.joint(tree, aln, g["multiplicity"], model, len(g["full_to_compressed"]),
                    sample_from_profile="root" if bool(g["sample_root"]) else False,
                    reconstruct_tip_states=bool(g["reconstruct_tip_states"]), rng=rng)
    np.testing.assert_allclose(res["sequence_LH"], g["joint_sequence_LH"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(res["sequence_joint_LH"], g["joint_total_LH"], rtol=1e-13)
    assert res["N_diff"] == int(g["joint_N_diff"])
    want = _names_map(g["joint_cseq_names"], g["joint_cseq"])
    for k, v in want.items():
        np.testing.assert_array_equal(gc.codes_of(res["cseq"][k]), v, err_msg=k)


@pytest.mark.parametrize("case", [c for c in CASES if "jbl" in gc.load(c)])
def test_oracle_joint_branch_lengths_match_treetime(case):
    g = gc.load(case)
    tree, _, model, _ = _prepared(g)
    aln = gc.compressed_from(g, model)
    res = anc.joint(tree, aln, g["multiplicity"], model, len(g["full_to_compressed"]),
                    reconstruct_tip_states=bool(g["reconstruct_tip_states"]))
    cseq = dict(res["cseq"])
    if not bool(g["reconstruct_tip_states"]):
        cseq.update({k: v for k, v in aln.items()})
    bl = anc.optimize_branch_lengths_joint(tree, lambda n: cseq[n.name], g["multiplicity"], model,
                                           ignore_gaps=bool(g["ignore_gaps"]))
    want = _names_map(g["jbl_names"], g["jbl"])
    # the argmin of a smooth objective is only defined to ~sqrt(machine eps)
    # relative; 1e-6 relative (+1e-10 absolute) is the branch-length bar
    for k, v in want.items():
        assert abs(bl[k] - v) <= 1e-6 * abs(v) + 1e-10, (k, bl[k], v)


@pytest.mark.parametrize("case", [c for c in CASES if "mbl" in gc.load(c)])
def test_oracle_marginal_branch_lengths_match_treetime(case):
    g = gc.load(case)
    tree, _, model, _ = _prepared(g)
    aln = gc.compressed_from(g, model)
    res = anc.marginal(tree, aln, g["multiplicity"], model, len(g["full_to_compressed"]),
                       reconstruct_tip_states=bool(g["reconstruct_tip_states"]))
    want = _names_map(g["mbl_names"], g["mbl"])
    for n in anc.preorder(tree.root):
        if n.up is None:
            continue
        m = g["multiplicity"] if n.mask is None else g["multiplicity"] * n.mask
        t, _ = anc.optimal_t_compressed(model, (res["outgroup_LH"][n.name], res["subtree_LH"][n.name]), m,
                                        profiles=True)
        v = want[n.name]
        assert abs(t - v) <= 1e-6 * abs(v) + 1e-10, (n.name, t, v)


# ------------------------------------------------ branch-length interpolator grids
BLGRID = gc.blgrid_names()


@pytest.mark.parametrize("case", BLGRID)
def test_branch_len_grids_match_treetime(case):
    """The oracle's and the product's grid builders give TreeTime's grids
    bit for bit (both shapes: zero-length and finite branches)."""
    from treetime_gb300 import engine
    g = gc.load(case)
    n, om = int(g["n_grid_points"]), float(g["one_mutation"])
    for mode in ("marginal", "joint"):
        grids, lengths = engine.branch_len_grids(g[mode + "_mutation_length"], om, n)
        np.testing.assert_array_equal(lengths, g[mode + "_len"])
        for i, ml in enumerate(g[mode + "_mutation_length"]):
            want = g[mode + "_x"][i, :int(g[mode + "_len"][i])]
            np.testing.assert_array_equal(anc.branch_len_grid(float(ml), om, n), want)
            np.testing.assert_array_equal(engine.branch_len_grid(float(ml), om, n), want)
            np.testing.assert_array_equal(grids[i, :lengths[i]], want)
            assert (grids[i, lengths[i]:] == -1.0).all()


@pytest.mark.parametrize("mode", ["marginal", "joint"])
@pytest.mark.parametrize("case", BLGRID)
def test_oracle_branch_len_values_match_treetime(case, mode):
    g = gc.load(case)
    got = gc.blgrid_oracle(g, mode)
    got_e = gc.blgrid_oracle(g, mode, expm1_form=True)
    n_noise = 0
    for i, name in enumerate(g[mode + "_names"].tolist()):
        L = int(g[mode + "_len"][i])
        want = g[mode + "_y"][i, :L] + g[mode + "_peak"][i]
        np.testing.assert_allclose(got[name][0], want, rtol=1e-11, atol=1e-9, err_msg=name)
        # the expm1 form agrees wherever the observed pairs' P(t) is resolved
        ok = got_e[name][1] >= 1e-6
        n_noise += int((~ok).sum())
        np.testing.assert_allclose(got_e[name][0][ok], want[ok], rtol=1e-9, atol=1e-8, err_msg=name)
    if mode == "marginal":
        assert n_noise == 0
    elif case == "blgrid_nuc":
        assert n_noise > 0  # the fixture does reach the rounding-dominated points


# ------------------------------------------------------------------ GTR inference
GTRINF = gc.gtrinf_names()


def _gtrinf_modes(g):
    return [m for m in ("marginal", "joint") if m + "_nij" in g]


@pytest.mark.parametrize("case", GTRINF)
def test_host_gtr_infer_matches_treetime(case):
    """The host fit (GTR.infer / GTR_site_specific.infer) on TreeTime's own
    counts gives TreeTime's model."""
    from treetime_gb300.gtr import GTR, GTR_site_specific
    g = gc.load(case)
    model = gc.model_from(g)
    for mode in _gtrinf_modes(g):
        if bool(g["site_specific"]):
            m = GTR_site_specific.infer(np.copy(g[mode + "_nij"]), np.copy(g[mode + "_Ti"]),
                                        root_state=np.copy(g[mode + "_root_state"]), pc=float(g["pc"]),
                                        alphabet=model.alphabet, prof_map=model.profile_map)
            m.mu /= m.average_rate().mean()
        else:
            m = GTR.infer(np.copy(g[mode + "_nij"]), np.copy(g[mode + "_Ti"]), np.copy(g[mode + "_root_state"]),
                          pc=float(g["pc"]), alphabet=model.alphabet, prof_map=model.profile_map)
            m.mu = 1.0
        np.testing.assert_allclose(m.W, g[mode + "_W"], rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(m.Pi, g[mode + "_Pi"], rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose(m.mu, g[mode + "_mu"], rtol=1e-12)


@pytest.mark.parametrize("case", GTRINF)
def test_oracle_substitution_counts_match_treetime(case):
    g = gc.load(case)
    for mode in _gtrinf_modes(g):
        n_ija, T_ia, _ = gc.gtrinf_oracle(g, mode)
        if bool(g["site_specific"]):
            np.testing.assert_allclose(n_ija, g[mode + "_nij"], rtol=1e-11, atol=1e-11)
            np.testing.assert_allclose(T_ia, g[mode + "_Ti"], rtol=1e-11, atol=1e-11)
        else:
            np.testing.assert_allclose(n_ija.sum(axis=-1), g[mode + "_nij"], rtol=1e-11, atol=1e-11)
            np.testing.assert_allclose(T_ia.sum(axis=-1), g[mode + "_Ti"], rtol=1e-11, atol=1e-11)


# ------------------------------------------------------------------ Fitch parsimony
FITCH = gc.fitch_names()


@pytest.mark.parametrize("case", FITCH)
def test_oracle_fitch_matches_treetime(case):
    g = gc.load(case)
    tree, aln, model, _ = gc.inputs_from(g)
    anc.prepare_tree(tree)
    caln, mult, full = gc.compress_inputs(aln, model)
    rng = np.random.default_rng(int(g["rng_seed"]))
    cseq, nd = anc.fitch(tree, caln, len(mult), rng)
    assert nd == int(g["fitch_N_diff"])
    for i, k in enumerate(g["fitch_names"].tolist()):
        np.testing.assert_array_equal(gc.codes_of(cseq[k]), g["fitch_cseq"][i], err_msg=k)
    cseq2, nd2 = anc.fitch(tree, caln, len(mult), rng, prev_cseq=cseq)
    assert nd2 == int(g["fitch_N_diff_again"])
    for i, k in enumerate(g["fitch_names"].tolist()):
        np.testing.assert_array_equal(gc.codes_of(cseq2[k]), g["fitch_cseq_again"][i], err_msg=k)
    res = anc.marginal(tree, caln, mult, model, full)
    cseq3, nd3 = anc.fitch(tree, caln, len(mult), np.random.default_rng(int(g["rng_seed"])),
                           prev_cseq=res["cseq"])
    assert nd3 == int(g["fitch_after_marginal_N_diff"])
    for i, k in enumerate(g["fitch_names"].tolist()):
        np.testing.assert_array_equal(gc.codes_of(cseq3[k]), g["fitch_after_marginal_cseq"][i], err_msg=k)


# ------------------------------------------------------- states drawn at every node
@pytest.mark.parametrize("tips", [False, True])
def test_oracle_sampling_at_every_node_matches_treetime(tips):
    g = gc.load("sample_nuc5")
    tree, aln, model, _ = gc.inputs_from(g)
    anc.prepare_tree(tree)
    caln, mult, full = gc.compress_inputs(aln, model)
    rng = np.random.default_rng(int(g["rng_seed"]))
    tag = "tips" if tips else "inner"
    res = anc.marginal(tree, caln, mult, model, full, sample_from_profile=True, reconstruct_tip_states=tips, rng=rng)
    assert res["N_diff"] == int(g[tag + "_N_diff"])
    for i, k in enumerate(g[tag + "_names"].tolist()):
        np.testing.assert_array_equal(gc.codes_of(res["cseq"][k]), g[tag + "_cseq"][i], err_msg=k)
    res2 = anc.marginal(tree, caln, mult, model, full, sample_from_profile=True, reconstruct_tip_states=tips,
                        rng=rng, prev_cseq=res["cseq"])
    assert res2["N_diff"] == int(g[tag + "_N_diff_again"])


# ------------------------------------------------ optimize_tree_marginal iterations
@pytest.mark.parametrize("tag,g", gc.optimize_cases(), ids=lambda x: x if isinstance(x, str) else "")
def test_oracle_optimize_tree_marginal_matches_treetime(tag, g):
    """The oracle's restatement of TreeTime's damped marginal branch-length
    iterations (bifurcating root: the two children as one branch, updated at
    the visit of each child; trifurcating root: every branch on its own)
    against TreeTime's own run: branch lengths, log-likelihood, sequences."""
    tree, aln, model, _ = gc.inputs_from(g)
    anc.prepare_tree(tree)
    assert len(tree.root.clades) == int(g["root_children"])
    caln, mult, L = gc.compress_inputs(aln, model)
    res, history = anc.optimize_tree_marginal(tree, caln, mult, model, L, max_iter=4)
    want = _names_map(g["node_names"], g["node_bl"])
    for n in anc.preorder(tree.root):
        v = want[n.name]
        assert abs(n.branch_length - v) <= 1e-9 * abs(v) + 1e-12, (tag, n.name, n.branch_length, v)
    assert abs(res["total_sequence_LH"] - float(g["total_LH"])) <= 1e-9 * abs(float(g["total_LH"]))
    cseq = _names_map(g["cseq_names"], g["cseq"])
    for name, codes in cseq.items():
        np.testing.assert_array_equal(np.frombuffer(np.asarray(res["cseq"][name]).astype("S1").tobytes(), np.uint8),
                                      codes)


def test_oracle_prune_short_branches_matches_treetime():
    """Short-branch pruning with a collapsed parent: TreeTime compares the
    next node with its new parent (where a gap no longer hides a mismatch)
    and keeps it; the oracle's restatement gives TreeTime's topology."""
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import parse_newick
    g = gc.load("prune_gaps")
    tree = parse_newick(str(g["newick"]))
    anc.prepare_tree(tree)
    model = GTR.standard("JC69", alphabet="nuc")
    chars = g["cseq"].view("S1").astype("U1")
    cseq = {str(k): chars[i] for i, k in enumerate(g["cseq_names"])}
    collapsed = anc.prune_short_branches(tree, lambda n: cseq[n.name], g["multiplicity"], model,
                                         float(g["one_mutation"]))
    assert collapsed == ["X"]
    got = {n.name: (n.up.name if n.up is not None else "") for n in anc.preorder(tree.root)}
    assert got == dict(zip(g["node_names"].tolist(), g["parent_names"].tolist()))


def test_oracle_optimize_tree_joint_matches_treetime():
    """TreeTime's joint optimize_tree loop (reconstruction, branch lengths,
    pruning of branches without mutations, until no character changes): the
    oracle's restatement gives the same topology, branch lengths, sequences
    and unconstrained log-likelihood."""
    g = gc.load("optimize_joint")
    tree, aln, model, _ = gc.inputs_from(g)
    anc.prepare_tree(tree)
    assert sum(1 for _ in anc.preorder(tree.root)) == int(g["n_nodes_before"])
    caln, mult, L = gc.compress_inputs(aln, model)
    res, lh = anc.optimize_tree_joint(tree, caln, mult, model, L, float(g["one_mutation"]), max_iter=3)
    got = {n.name: (n.up.name if n.up is not None else "") for n in anc.preorder(tree.root)}
    assert got == dict(zip(g["node_names"].tolist(), g["parent_names"].tolist()))
    want = _names_map(g["node_names"], g["node_bl"])
    for n in anc.preorder(tree.root):
        v = want[n.name]
        assert abs(n.branch_length - v) <= 1e-9 * abs(v) + 1e-12, (n.name, n.branch_length, v)
    assert abs(lh - float(g["unconstrained_LH"])) <= 1e-9 * abs(float(g["unconstrained_LH"]))
    for name, codes in _names_map(g["cseq_names"], g["cseq"]).items():
        np.testing.assert_array_equal(np.frombuffer(np.asarray(res["cseq"][name]).astype("S1").tobytes(), np.uint8),
                                      codes)


def test_mixin_prune_logic_matches_treetime(monkeypatch):
    """GPUAncMixin.prune_short_branches' host logic (preorder visit, collapse,
    the re-parented node compared with its new parent) on the pruning
    fixture, with the device pieces (pair histograms of the layout's
    branches, log P at distance zero) stood in for by the oracle on the CPU."""
    import torch
    from types import SimpleNamespace
    from treetime_gb300 import engine
    from treetime_gb300.anc_gpu import GPUAncMixin, pair_counts
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import parse_newick
    g = gc.load("prune_gaps")
    tree = parse_newick(str(g["newick"]))
    anc.prepare_tree(tree)
    layout = engine.TreeLayout(tree.root)
    model = GTR.standard("JC69", alphabet="nuc")
    q, mult = model.n_states, g["multiplicity"]
    P = len(mult)
    index = {c: i for i, c in enumerate(model.alphabet)}
    chars = g["cseq"].view("S1").astype("U1")
    states = np.zeros((layout.n_nodes, P), np.uint8)
    for name, row in zip(g["cseq_names"].tolist(), chars):
        k = next(i for i, n in enumerate(layout.nodes) if n.name == name)
        states[k] = [index[c] for c in row]
    hist = np.zeros((layout.n_nodes, q, q))
    for k in range(layout.n_nodes):
        if layout.parent[k] >= 0 and k < layout.n_int:
            hist[k] = pair_counts(states[layout.parent[k]], states[k], mult, q, model.gap_index, True)
    sess = {"layout": layout, "model": model, "forest": SimpleNamespace(device="cpu"),
            "bufs": SimpleNamespace(cache={("states", torch.uint8): torch.from_numpy(states.reshape(-1))})}

    def log_p0(q_, counts, model_, t):
        out = []
        for c in counts.cpu().numpy():
            nz = np.argwhere(c > 0)
            out.append(anc.prob_t_compressed(model_, nz, c[nz[:, 0], nz[:, 1]], t, return_log=True) if len(nz)
                       else 0.0)
        return np.array(out)

    monkeypatch.setattr(engine, "prob_t_pairs_batch", log_p0)

    class Host(GPUAncMixin):
        def logger(self, *args, **kwargs):
            pass

    host = Host()
    host.tree, host.gtr = SimpleNamespace(find_clades=tree.find_clades, root=tree.root), model
    host.data = SimpleNamespace(multiplicity=lambda mask=None: mult if mask is None else mult * mask,
                                compressed_length=P)
    host.one_mutation = float(g["one_mutation"])
    host._pair_histograms = lambda ignore_gaps=None: (sess, torch.from_numpy(hist))
    host.prune_short_branches()
    got = {n.name: (n.up.name if n.up is not None else "") for n in anc.preorder(tree.root)}
    assert got == dict(zip(g["node_names"].tolist(), g["parent_names"].tolist()))


@pytest.mark.parametrize("tag,g", gc.optimize_cases(), ids=lambda x: x if isinstance(x, str) else "")
def test_mixin_optimize_tree_marginal_logic_matches_treetime(tag, g, monkeypatch):
    """GPUAncMixin.optimize_tree_marginal's host logic (damping, tolerances,
    the bifurcating root's pair updated at both children's visits, the stop
    rule) on TreeTime's fixture, with the device pieces (reconstruction,
    profile Brent) stood in for by the oracle on the CPU."""
    from types import SimpleNamespace
    from treetime_gb300 import engine
    from treetime_gb300.anc_gpu import GPUAncMixin
    tree, aln, model, _ = gc.inputs_from(g)
    anc.prepare_tree(tree)
    caln, mult, L = gc.compress_inputs(aln, model)
    monkeypatch.setattr(engine, "optimal_t_compressed",
                        lambda gtr, pair, m, profiles=False, tol=1e-10:
                        anc.optimal_t_compressed(model, pair, m, profiles=profiles, tol=tol)[0])

    class Host(GPUAncMixin):
        def logger(self, *args, **kwargs):
            pass

        def infer_ancestral_sequences(self, marginal=True, **kwargs):
            self.res = anc.marginal(tree, caln, mult, model, L)
            for n in anc.preorder(tree.root):
                n.marginal_subtree_LH = self.res["subtree_LH"][n.name]
                n.marginal_outgroup_LH = self.res["outgroup_LH"][n.name]

        def sequence_LH(self):
            return self.res["total_sequence_LH"]

        def _marginal_branch_lengths(self, nodes, tol):
            return np.array([anc.optimal_t_compressed(model, (n.marginal_outgroup_LH, n.marginal_subtree_LH), mult,
                                                      profiles=True, tol=tol)[0] for n in nodes])

    host = Host()
    host.tree, host.gtr = tree, model
    host.data = SimpleNamespace(multiplicity=lambda mask=None: mult if mask is None else mult * mask)
    host.optimize_tree_marginal(max_iter=4)
    want = _names_map(g["node_names"], g["node_bl"])
    for n in anc.preorder(tree.root):
        v = want[n.name]
        assert abs(n.branch_length - v) <= 1e-9 * abs(v) + 1e-12, (tag, n.name, n.branch_length, v)
    assert abs(host.sequence_LH() - float(g["total_LH"])) <= 1e-9 * abs(float(g["total_LH"]))


def test_treeanc_optimize_tree_joint_logic_matches_treetime(monkeypatch):
    """treetime_gb300.TreeAnc.optimize_tree in joint mode (the loop, the
    mixin's joint branch lengths and pruning, node preparation) on TreeTime's
    fixture, with the device pieces (joint reconstruction, pair histograms,
    Brent on pair counts, log P at distance zero) stood in for by the oracle
    on the CPU."""
    import torch
    from types import SimpleNamespace
    from treetime_gb300 import TreeAnc, engine
    from treetime_gb300.tree import parse_newick
    g = gc.load("optimize_joint")
    _, aln, model, _ = gc.inputs_from(g)
    q = model.n_states

    def counts_of(c):
        nz = np.argwhere(c > 0)
        return nz, c[nz[:, 0], nz[:, 1]]

    def log_p0(q_, counts, model_, t):
        out = []
        for c in counts.cpu().numpy():
            nz, m = counts_of(c)
            out.append(anc.prob_t_compressed(model, nz, m, t, return_log=True) if len(nz) else 0.0)
        return np.array(out)

    def brent_pairs(q_, counts, model_, model_of=None, tol=1e-10):
        ts = []
        for c in counts.cpu().numpy():
            nz, m = counts_of(c)
            ts.append(anc.optimal_t_compressed(model, nz, m, tol=tol)[0] if len(nz) else 0.0)
        return torch.tensor(ts, dtype=torch.float64), torch.zeros(len(ts), dtype=torch.int32)

    monkeypatch.setattr(engine, "prob_t_pairs_batch", log_p0)
    monkeypatch.setattr(engine, "optimal_t_pairs", brent_pairs)

    class Host(TreeAnc):
        def _compressed(self):
            chars = {k: np.array(list(v)) for k, v in self.data.compressed_alignment.items()}
            return chars, self.data.multiplicity(), self.data.full_length

        def _ml_anc_joint(self, reconstruct_tip_states=False, **kwargs):
            caln, mult, L = self._compressed()
            inner = [n for n in self.tree.find_clades() if n.clades]
            prev = {n.name: n._cseq for n in inner} if self.sequence_reconstruction else None
            res = anc.joint(self.tree, caln, mult, model, L, prev_cseq=prev)
            for n in inner:
                n._cseq = res["cseq"][n.name]
            self.tree.sequence_LH = res["sequence_LH"]
            self.sequence_reconstruction = "joint"
            self.reconstructed_tip_sequences = False
            return res["N_diff"]

        def _pair_histograms(self, ignore_gaps=None):
            ig = self.ignore_gaps if ignore_gaps is None else ignore_gaps
            caln, mult, _ = self._compressed()
            layout = engine.TreeLayout(self.tree.root)
            seq = lambda n: n._cseq if n.clades else caln[n.name]
            hist = np.zeros((layout.n_nodes, q, q))
            states = np.zeros((layout.n_nodes, len(mult)), np.uint8)
            idx = {c: i for i, c in enumerate(model.alphabet)}
            for k, n in enumerate(layout.nodes):
                if n.clades:
                    states[k] = [idx[c] for c in n._cseq]
                if layout.parent[k] >= 0:
                    m = mult if getattr(n, "mask", None) is None else mult * n.mask
                    nz, cnt = anc.state_pair(model, seq(layout.nodes[layout.parent[k]]), seq(n),
                                             pattern_multiplicity=m, ignore_gaps=ig)
                    for (i, j), c in zip(nz, cnt):
                        hist[k, i, j] = c
            sess = {"layout": layout, "model": model, "forest": SimpleNamespace(device="cpu"),
                    "bufs": SimpleNamespace(cache={("states", torch.uint8): torch.from_numpy(states.reshape(-1))})}
            return sess, torch.from_numpy(hist)

    tree = parse_newick(str(g["newick"]))
    t = Host(tree=tree, aln=aln, gtr=model, verbose=0)
    assert sum(1 for _ in t.tree.find_clades()) == int(g["n_nodes_before"])
    t.optimize_tree(branch_length_mode="joint", max_iter=3, prune_short=True)
    got = {n.name: (n.up.name if n.up is not None else "") for n in t.tree.find_clades()}
    assert got == dict(zip(g["node_names"].tolist(), g["parent_names"].tolist()))
    want = _names_map(g["node_names"], g["node_bl"])
    for n in t.tree.find_clades():
        v = want[n.name]
        assert abs(n.branch_length - v) <= 1e-9 * abs(v) + 1e-12, (n.name, n.branch_length, v)
    lh = float(g["unconstrained_LH"])
    assert abs(t.tree.unconstrained_sequence_LH - lh) <= 1e-9 * abs(lh)
