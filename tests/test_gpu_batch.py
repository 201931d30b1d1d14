"""GPU: the batched path.  A marginal pass captured as a CUDA graph replays to
the same numbers as a direct call (also after the branch lengths are changed
in place), and a small batch built like the 256-tree workload (random trees,
sizes and models, alignments from the sparse sampler) matches the oracle tree
by tree."""

import numpy as np
import pytest

from oracle import anc

pytestmark = pytest.mark.gpu


def _internal_state_rows(forest):
    """Indices of the state bytes the pass writes without tip reconstruction
    (internal nodes; tip rows are left as they were)."""
    idx = []
    for tr in forest.trees_host:
        P = int(tr["n_patterns"])
        idx.append(np.arange(int(tr["state_base"]), int(tr["state_base"]) + int(tr["n_int"]) * P))
    return np.concatenate(idx)


def _small_batch(n_trees=5, seed=11):
    from treetime_gb300 import synth
    return synth.forest_c3(n_trees=n_trees, seed=seed, n_range=(8, 60), L_range=(80, 400), bl_range=(1e-3, 0.1))


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_captured_marginal_equals_direct(precision):
    from treetime_gb300 import engine
    inputs, gtrs = _small_batch()
    forest = engine.Forest(inputs, 4)
    model = engine.DeviceModel(gtrs)
    direct = engine.marginal(forest, model, engine.Buffers(forest), precision=precision)
    rows = _internal_state_rows(forest)
    pick = lambda d: {"posterior": d["posterior"].cpu().numpy().copy(), "states": d["states"].cpu().numpy()[rows],
                      "site_lh": d["site_lh"].cpu().numpy().copy(), "tree_lh": d["tree_lh"].cpu().numpy().copy()}
    ref = pick(direct)
    cap = engine.CapturedMarginal(forest, model, engine.Buffers(forest), precision=precision)
    for _ in range(3):
        got = pick(cap.replay(sync=True))
        for k, v in ref.items():
            np.testing.assert_array_equal(got[k], v)
    # new branch lengths written in place: the replay follows them
    rng = np.random.default_rng(5)
    new_bl = [ti.bl * rng.uniform(0.5, 2.0, size=ti.bl.shape) for ti in inputs]
    forest.set_branch_lengths(new_bl)
    again = cap.replay(sync=True)
    direct2 = engine.marginal(forest, model, engine.Buffers(forest), precision=precision)
    np.testing.assert_array_equal(again["tree_lh"].cpu().numpy(), direct2["tree_lh"].cpu().numpy())
    assert not np.array_equal(again["tree_lh"].cpu().numpy(), ref["tree_lh"])


def test_batch_matches_oracle_per_tree():
    from treetime_gb300 import engine
    from treetime_gb300.tree import Tree
    inputs, gtrs = _small_batch(n_trees=6, seed=12)
    forest = engine.Forest(inputs, 4)
    model = engine.DeviceModel(gtrs)
    out = engine.marginal(forest, model, engine.Buffers(forest), precision="f32")
    tree_lh = out["tree_lh"].cpu().numpy()
    post = out["posterior"].cpu().numpy()
    for k, ti in enumerate(inputs):
        lay = ti.layout
        tips = lay.nodes[lay.n_int:]
        chars = ti.tip_codes.view("S1").astype("U1")
        aln = {t.name: chars[r] for t, r in zip(tips, ti.tip_row)}
        # the oracle ladderizes and renames in place: compare through the clade objects
        internal = lay.nodes[:lay.n_int]
        tree = anc.prepare_tree(Tree(root=lay.nodes[lay.n_int - 1]))
        ref = anc.marginal(tree, aln, ti.mult, gtrs[k], int(round(ti.mult.sum())))
        assert abs(tree_lh[k] - ref["total_sequence_LH"]) <= 1e-6 * abs(ref["total_sequence_LH"])
        tr = forest.trees_host[k]
        P = ti.n_patterns
        for j, n in enumerate(internal):
            rows = post[tr["prof_base"] + j * P: tr["prof_base"] + (j + 1) * P, :4]
            np.testing.assert_allclose(rows, ref["profile"][n.name], atol=1e-5)
