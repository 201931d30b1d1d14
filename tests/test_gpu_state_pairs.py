"""GPU: the (parent state, child state) histograms of every branch against the
oracle's restatement of GTR.state_pair (treetime/gtr.py:631-712) on the same
sequences: whole-number multiplicities summed as integers (bit for bit the
float sums), masked branches and fractional weights in FP64, for alphabets of
4, 5 and 20 states (the integer warp reductions below 33 bins, per-warp
integer bins above), with and without ignore_gaps.  state_pair casts its sums
to int (gtr.py:709-712); the device keeps them and the callers truncate."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle_hist(t, mult, ignore_gaps):
    from oracle import anc
    sess = t._get_session()
    layout = sess["layout"]
    q = t.gtr.n_states
    caln = t.data.compressed_alignment
    seq = lambda n: n._cseq if n.clades else caln[n.name]
    hist = np.zeros((layout.n_nodes, q, q))
    for k, n in enumerate(layout.nodes):
        if layout.parent[k] < 0:
            continue
        m = mult if getattr(n, "mask", None) is None else mult * n.mask
        nz, cnt = anc.state_pair(t.gtr, seq(layout.nodes[layout.parent[k]]), seq(n), pattern_multiplicity=m,
                                 ignore_gaps=ignore_gaps)
        for (i, j), c in zip(nz, cnt):
            hist[k, i, j] = c
    return hist


@pytest.mark.parametrize("alphabet", ["nuc_nogap", "nuc", "aa_nogap"])
@pytest.mark.parametrize("weights", ["whole", "masked", "fractional"])
def test_pair_histograms_match_the_oracle(alphabet, weights):
    from treetime_gb300 import TreeAnc, engine, synth
    wl = synth.make_workload("c0", seed=21, n=70, L=900, alphabet=alphabet, gap_frac=0.08)
    t = TreeAnc(tree=wl["tree"], aln=wl["aln"], gtr=wl["gtr"], verbose=0)
    t.infer_ancestral_sequences(marginal=False)
    P = t.data.compressed_length
    rng = np.random.default_rng(5)
    mult = np.asarray(t.data.multiplicity(), dtype=np.float64)
    if weights == "masked":
        for n in list(t.tree.find_clades())[3:40:3]:
            n.mask = rng.choice([0.0, 0.5, 1.0], size=P)
        t.infer_ancestral_sequences(marginal=False)
    sess = t._get_session()
    if weights == "fractional":
        mult = mult * rng.choice([1.0, 0.25, 1.5], size=P)
        sess["forest"].d_mult.copy_(engine.torch().from_numpy(mult))
    for ig in (False, True):
        _, hist = t._pair_histograms(ignore_gaps=ig)
        got = hist.cpu().numpy()
        want = _oracle_hist(t, mult, ig)
        # TreeTime's state_pair returns its sums cast to int; the device histograms keep the sums
        # and the branch-length step truncates them.  The weights here are whole numbers or
        # multiples of 1/4, so every order of summation gives the same FP64 sums.
        assert np.array_equal(np.trunc(got), want)
        if weights == "whole":
            assert np.array_equal(got, want)
        else:
            assert (got != np.trunc(got)).any()  # the fractional sums reached the device histograms
