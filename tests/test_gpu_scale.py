"""Parity at the sizes of the benchmark configurations, against the oracle
(TreeTime's algorithms restated in numpy, run over a spawn-started process
pool with the patterns split between the processes: patterns are
independent, so the pooled result is the result of one call).

Workloads (seeded, ``treetime_gb300.synth``):
  * the 2,000-tip x 30,000-site nucleotide tree (90% invariant sites, 2,748
    patterns) through the public TreeAnc API: marginal in FP64 and FP32, joint,
    optimize_branch_lengths_joint on all 3,998 branches, and the profile-mode
    (marginal) branch lengths of all branches from FP64 and FP32 profiles;
  * the 500-tip x 1,500-site protein tree under a site-specific model (TreeTime's
    default interpolated P(t)) through TreeAnc: marginal in FP64 and FP32, and
    joint;
  * the three largest trees of the 256-tree batch (by tips x sites), as one
    forest through the engine's batch path, FP64 and FP32; one of them is the
    batch's least divergent large tree (3,116 tips, mean branch 1.2e-4).

Tolerances (the contract of this port):
  * FP64 kernels: per-tree log-likelihood 1e-10 relative, per-pattern 1e-10
    relative, profiles 1e-10 absolute, argmax states exact except where the
    oracle's posterior has a top-two margin below 1e-9;
  * FP32 kernels: per-tree log-likelihood 1e-6 relative, per-pattern 1e-6
    relative + 1e-5 absolute (a protein site's log-likelihood is ~-500, where
    FP32 rounding alone is ~1e-5), profiles 1e-5 absolute, states exact except
    where the oracle's top-two margin is below 1e-5;
  * joint: state indices exact except patterns where the oracle's top-two
    margin at some node of the chosen path is below 1e-9 (counted and
    printed), log-likelihood 1e-12 relative;
  * joint branch lengths: 1e-6 relative + 1e-10 absolute, or, where the
    objective is flat enough that its argmin is rounding noise, equal
    objective values at both lengths (1e-9 relative).
"""

import numpy as np
import pytest

from oracle import anc, parallel

pytestmark = pytest.mark.gpu


def _alpha_index(gtr):
    idx = np.full(256, 255, dtype=np.uint8)
    for i, c in enumerate(gtr.alphabet):
        idx[ord(str(c))] = i
    return idx


def _states(t, names, gtr):
    """State indices [len(names), P] of TreeAnc's reconstruction."""
    nodes = {n.name: n for n in t.tree.find_clades()}
    idx = _alpha_index(gtr)
    return np.stack([idx[np.frombuffer(np.asarray(nodes[k]._cseq).astype("S1").tobytes(), dtype=np.uint8)]
                     for k in names])


def _check_states(got, ora, near, level, what):
    bad = (got != ora) & (near < level)
    assert not bad.any(), (what, int(bad.sum()), np.argwhere(bad)[:5])
    return int(((got != ora) & (near >= level)).sum())


# ------------------------------------------------------------------ 2,000 x 30,000
@pytest.fixture(scope="module")
def c1():
    from treetime_gb300 import synth
    from treetime_gb300.tree import to_newick
    wl = synth.make_workload("c1", seed=1)  # the benchmark's instance
    return wl, to_newick(wl["tree"])


def _treeanc(wl, nwk, precision):
    from treetime_gb300 import TreeAnc
    from treetime_gb300.tree import parse_newick
    return TreeAnc(tree=parse_newick(nwk), aln=wl["aln"], gtr=wl["gtr"], compress=wl["compress"], verbose=0,
                   precision=precision)


@pytest.fixture(scope="module")
def c1_oracle(c1):
    wl, nwk = c1
    t = _treeanc(wl, nwk, "f64")
    d = t.data
    names = [n.name for n in t.tree.find_clades() if n.clades]
    mar = parallel.marginal(nwk, d.sequence_names, d.compressed_codes, d.multiplicity(), wl["gtr"], d.full_length,
                            keep=names)
    jnt = parallel.joint(nwk, d.sequence_names, d.compressed_codes, d.multiplicity(), wl["gtr"], d.full_length)
    return mar, jnt


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_c1_marginal_matches_oracle(c1, c1_oracle, precision):
    wl, nwk = c1
    mar, _ = c1_oracle
    t = _treeanc(wl, nwk, precision)
    t.infer_ancestral_sequences(marginal=True)
    f32 = precision == "f32"
    assert t.data.compressed_length == 2748
    tot = mar["total"]
    assert abs(t.tree.total_sequence_LH - tot) <= (1e-6 if f32 else 1e-10) * abs(tot), (t.tree.total_sequence_LH, tot)
    if f32:
        np.testing.assert_allclose(t.tree.sequence_LH, mar["site_lh"], rtol=1e-6, atol=1e-5)
    else:
        np.testing.assert_allclose(t.tree.sequence_LH, mar["site_lh"], rtol=1e-10, atol=0)
    nodes = {n.name: n for n in t.tree.find_clades()}
    tol = 1e-5 if f32 else 1e-10
    worst = 0.0
    for k, want in mar["profiles"].items():
        worst = max(worst, float(np.abs(nodes[k].marginal_profile - want).max()))
    assert worst <= tol, worst
    ties = _check_states(_states(t, mar["names"], wl["gtr"]), mar["states"], mar["near"], 2 if f32 else 1,
                         "marginal " + precision)
    print("c1 marginal %s: max profile difference %.2e, relative log-LH error %.2e, %d near-tie states"
          % (precision, worst, abs(t.tree.total_sequence_LH - tot) / abs(tot), ties))


def test_c1_joint_and_branch_lengths_match_oracle(c1, c1_oracle):
    wl, nwk = c1
    _, jnt = c1_oracle
    t = _treeanc(wl, nwk, "f64")
    t.infer_ancestral_sequences(marginal=False)
    assert abs(t.tree.sequence_joint_LH - jnt["total"]) <= 1e-12 * abs(jnt["total"])
    got = _states(t, jnt["names"], wl["gtr"])
    tie = jnt["tie"][None, :]
    bad = (got != jnt["states"]) & ~tie
    assert not bad.any(), (int(bad.sum()), np.argwhere(bad)[:5])
    print("c1 joint: %d of %d patterns have a near-tie on their path" % (int(jnt["tie"].sum()), tie.size))
    # branch lengths of every branch from the reconstructed sequences (GPU) and from the oracle's
    # Brent over TreeTime's objective on the same sequences
    seqs = {n.name: np.asarray(n._cseq) for n in t.tree.find_clades() if n.clades}
    d = t.data
    for i, k in enumerate(d.sequence_names):
        seqs[k] = d.compressed_codes[i].view("S1").astype("U1")
    from treetime_gb300.tree import parse_newick
    tree_o = anc.prepare_tree(parse_newick(nwk))
    want = anc.optimize_branch_lengths_joint(tree_o, lambda n: seqs[n.name], d.multiplicity(), wl["gtr"],
                                             ignore_gaps=t.ignore_gaps)
    t.optimize_branch_lengths_joint()
    nodes = {n.name: n for n in t.tree.find_clades()}
    flat = 0
    assert len(want) == 3998
    for k, v in want.items():
        x = nodes[k].branch_length
        if abs(x - v) <= 1e-6 * abs(v) + 1e-10:
            continue
        n = nodes[k]
        pairs, cnt = n.branch_state["pair"], n.branch_state["multiplicity"]
        f = lambda tt: -anc.prob_t_compressed(wl["gtr"], pairs, cnt, tt, return_log=True)
        assert abs(f(x) - f(v)) <= 1e-9 * abs(f(v)) + 1e-12, (k, x, v, f(x), f(v))
        flat += 1
    print("c1 joint branch lengths: %d of 3998 differ beyond 1e-6 with equal objective values" % flat)


@pytest.fixture(scope="module")
def c1_marginal_lengths(c1):
    wl, nwk = c1
    t = _treeanc(wl, nwk, "f64")
    d = t.data
    return parallel.marginal_branch_lengths(nwk, d.sequence_names, d.compressed_codes, d.multiplicity(), wl["gtr"],
                                            d.full_length)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_c1_marginal_branch_lengths_match_oracle(c1, c1_marginal_lengths, precision):
    """Profile-mode branch lengths (optimal_marginal_branch_length, tol 1e-10) of
    all 3,998 branches after a marginal reconstruction: 1e-6 relative + 1e-10
    absolute, or equal objective values (1e-9 relative, with the oracle's FP64
    profiles) where the objective is flat enough that its argmin is rounding
    noise.  The FP32 path searches on its FP32 objective and then polishes the
    root of the objective's derivative."""
    wl, nwk = c1
    want = c1_marginal_lengths
    t = _treeanc(wl, nwk, precision)
    t.infer_ancestral_sequences(marginal=True)
    nodes = {n.name: n for n in t.tree.find_clades()}
    names = sorted(want)
    got = dict(zip(names, t._marginal_branch_lengths([nodes[k] for k in names], 1e-10)))
    far = [k for k in names if abs(got[k] - want[k]) > 1e-6 * abs(want[k]) + 1e-10]
    if far:
        from treetime_gb300.tree import parse_newick
        d = t.data
        tree_o = anc.prepare_tree(parse_newick(nwk))
        aln = {k: d.compressed_codes[i].view("S1").astype("U1") for i, k in enumerate(d.sequence_names)}
        ores = anc.marginal(tree_o, aln, d.multiplicity(), wl["gtr"], d.full_length)
        for k in far:
            pp, pc = ores["outgroup_LH"][k], ores["subtree_LH"][k]
            f = lambda tt: -anc.prob_t_profiles(wl["gtr"], (pp, pc), d.multiplicity(), tt, return_log=True) \
                + np.exp(tt * tt / 1e4)
            assert abs(f(got[k]) - f(want[k])) <= 1e-9 * abs(f(want[k])) + 1e-12, (k, got[k], want[k])
    rel = np.array([abs(got[k] - want[k]) / max(abs(want[k]), 1e-300) for k in names])
    print("c1 marginal branch lengths %s: median relative difference %.2e, 99th percentile %.2e, %d of %d beyond "
          "1e-6 with equal objective values" % (precision, np.median(rel), np.percentile(rel, 99), len(far),
                                                len(names)))


# ------------------------------------------------------------------ protein, site-specific
@pytest.fixture(scope="module")
def c2():
    from treetime_gb300 import synth
    from treetime_gb300.tree import to_newick
    wl = synth.make_workload("c2")
    assert wl["gtr"].approximate
    return wl, to_newick(wl["tree"])


@pytest.fixture(scope="module")
def c2_oracle(c2):
    wl, nwk = c2
    t = _treeanc(wl, nwk, "f64")
    d = t.data
    names = [n.name for n in t.tree.find_clades() if n.clades]
    return parallel.marginal(nwk, d.sequence_names, d.compressed_codes, d.multiplicity(), wl["gtr"], d.full_length,
                             keep=names)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_c2_site_specific_marginal_matches_oracle(c2, c2_oracle, precision):
    wl, nwk = c2
    mar = c2_oracle
    t = _treeanc(wl, nwk, precision)
    t.infer_ancestral_sequences(marginal=True)
    f32 = precision == "f32"
    assert t.data.compressed_length == 1500 and t.tree.count_terminals() == 500
    tot = mar["total"]
    assert abs(t.tree.total_sequence_LH - tot) <= (1e-6 if f32 else 1e-10) * abs(tot)
    if f32:
        np.testing.assert_allclose(t.tree.sequence_LH, mar["site_lh"], rtol=1e-6, atol=1e-5)
    else:
        np.testing.assert_allclose(t.tree.sequence_LH, mar["site_lh"], rtol=1e-10, atol=0)
    nodes = {n.name: n for n in t.tree.find_clades()}
    tol = 1e-5 if f32 else 1e-10
    worst = max(float(np.abs(nodes[k].marginal_profile - want).max()) for k, want in mar["profiles"].items())
    assert worst <= tol, worst
    ties = _check_states(_states(t, mar["names"], wl["gtr"]), mar["states"], mar["near"], 2 if f32 else 1,
                         "site-specific " + precision)
    print("c2 marginal %s: max profile difference %.2e, relative log-LH error %.2e, %d near-tie states"
          % (precision, worst, abs(t.tree.total_sequence_LH - tot) / abs(tot), ties))


def test_c2_site_specific_joint_matches_oracle(c2):
    """Joint reconstruction under the site-specific model (TreeTime's
    interpolated P(t)) at full size: states exact except near-ties, per-site
    and total log-likelihoods 1e-10 relative (FP64)."""
    wl, nwk = c2
    t = _treeanc(wl, nwk, "f64")
    d = t.data
    jnt = parallel.joint(nwk, d.sequence_names, d.compressed_codes, d.multiplicity(), wl["gtr"], d.full_length)
    t.infer_ancestral_sequences(marginal=False)
    assert abs(t.tree.sequence_joint_LH - jnt["total"]) <= 1e-10 * abs(jnt["total"])
    np.testing.assert_allclose(t.tree.sequence_LH, jnt["site_lh"], rtol=1e-10, atol=0)
    got = _states(t, jnt["names"], wl["gtr"])
    bad = (got != jnt["states"]) & ~jnt["tie"][None, :]
    assert not bad.any(), (int(bad.sum()), np.argwhere(bad)[:5])
    print("c2 joint: %d of %d sites have a near-tie on their path" % (int(jnt["tie"].sum()), jnt["tie"].size))


# ------------------------------------------------------------------ batch: the largest trees
@pytest.fixture(scope="module")
def c3_top():
    """The three largest trees of the 256-tree batch (tips x sites) with
    their trees prepared as TreeTime prepares them (ladderised, internal nodes
    named in preorder), as one forest."""
    from treetime_gb300 import engine, synth
    from treetime_gb300.tree import parse_newick, to_newick
    sizes = synth.c3_sizes()
    top = sorted(range(len(sizes)), key=lambda k: -sizes[k][0] * sizes[k][1])[:3]
    raw, gtrs = synth.forest_c3(only=top)
    inputs, jobs = [], []
    for m, ti in enumerate(raw):
        tips = ti.layout.nodes[ti.layout.n_int:]
        names = [tp.name for tp in tips]
        codes = ti.tip_codes[ti.tip_row]                     # rows in the order of `names`
        row = {k: i for i, k in enumerate(names)}
        prep = anc.prepare_tree(parse_newick(to_newick(ti.tree)))
        lay = engine.TreeLayout(prep.root)
        tip_row = np.array([row[n.name] for n in lay.nodes[lay.n_int:]], dtype=np.int32)
        inputs.append(engine.TreeInput(lay, codes, tip_row, ti.mult, engine.branch_lengths(lay, ti.full_length),
                                       model=m))
        jobs.append((to_newick(prep), names, codes, ti.mult, ti.full_length))
    oracle = [parallel.marginal(nwk, names, codes, mult, gtrs[m], L) for m, (nwk, names, codes, mult, L)
              in enumerate(jobs)]
    return inputs, gtrs, oracle


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_c3_largest_trees_match_oracle(c3_top, precision):
    from treetime_gb300 import engine
    inputs, gtrs, oracle = c3_top
    f32 = precision == "f32"
    forest = engine.Forest(inputs, 4)
    model = engine.DeviceModel(gtrs)
    out = engine.marginal(forest, model, engine.Buffers(forest), precision=precision)
    tree_lh = out["tree_lh"].cpu().numpy()
    site_lh = out["site_lh"].cpu().numpy()
    states = out["states"].cpu().numpy()
    for m, (ti, ora) in enumerate(zip(inputs, oracle)):
        tr = forest.trees_host[m]
        P = ti.n_patterns
        rel = abs(tree_lh[m] - ora["total"]) / abs(ora["total"])
        assert rel <= (1e-6 if f32 else 1e-10), (m, rel)
        s = site_lh[tr["pat_base"]:tr["pat_base"] + P]
        if f32:
            np.testing.assert_allclose(s, ora["site_lh"], rtol=1e-6, atol=1e-5)
        else:
            np.testing.assert_allclose(s, ora["site_lh"], rtol=1e-10, atol=0)
        lay = ti.layout
        k_of = {n.name: k for k, n in enumerate(lay.nodes[:lay.n_int])}
        got = np.stack([states[tr["state_base"] + k_of[k] * P:tr["state_base"] + (k_of[k] + 1) * P]
                        for k in ora["names"]])
        ties = _check_states(got, ora["states"], ora["near"], 2 if f32 else 1, "tree %d %s" % (m, precision))
        print("batch tree of %d tips x %d patterns (mean branch %.2g), %s: relative log-LH error %.2e, "
              "%d near-tie states" % (lay.n_tip, P, float(np.mean(ti.bl)), precision, rel, ties))
