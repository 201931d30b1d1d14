"""GPU: the FP32 drop-in reconstruction runs the pass without its outgroup rows
and changed-site count, and forms them afterwards (engine.marginal_lean,
engine.outgroups, tt_outgroups_f32, tt_count_changes).  The rows must equal,
bit for bit, the ones the pass itself stores (marginal(keep_outgroup=True,
tip_outgroup=True) on the same forest and lengths), for 4 and 5 states, with
masks and polytomies, after the branch lengths changed since the
reconstruction (the rows belong to the lengths the pass used), and through
the session's CUDA-graph replays; N_diff must equal the count of changed
states between consecutive reconstructions (treetime/treeanc.py:880-932)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _treeanc(alphabet, masks, polytomy, seed=7):
    from treetime_gb300 import TreeAnc, synth
    wl = synth.make_workload("c0", seed=seed, n=90, L=700, alphabet=alphabet, gap_frac=0.06)
    tree = wl["tree"]
    if polytomy:
        inner = [c for c in tree.find_clades(order="postorder") if c.clades and c is not tree.root]
        c = inner[len(inner) // 2]
        for par in tree.find_clades():
            if c in par.clades:
                i = par.clades.index(c)
                par.clades[i:i + 1] = c.clades
                break
    t = TreeAnc(tree=tree, aln=wl["aln"], gtr=wl["gtr"], verbose=0, precision="f32")
    if masks:
        rng = np.random.default_rng(seed)
        P = t.data.compressed_length
        for n in list(t.tree.find_clades())[2:60:4]:
            n.mask = rng.choice([0.0, 0.3, 1.0], size=P)
    return t


def _reference_rows(t):
    """The outgroup rows the pass stores itself, on the session's forest and current lengths."""
    from treetime_gb300 import engine
    s = t._get_session()
    ref = engine.marginal(s["forest"], s["model"], engine.Buffers(s["forest"]), precision="f32",
                          keep_outgroup=True, tip_outgroup=True)
    return ref["outgroup"].cpu().numpy().copy(), ref["tip_outgroup"].cpu().numpy().copy()


def _deferred_rows(t):
    out = t._last[1]
    out["_outgroups"]()
    return out["outgroup"].cpu().numpy().copy(), out["tip_outgroup"].cpu().numpy().copy()


def _internal_rows(t, a):
    lay = t._get_session()["layout"]
    P = t.data.compressed_length
    return a[: lay.n_int * P]  # the internal nodes' rows (the root's: pi)


@pytest.mark.parametrize("alphabet", ["nuc_nogap", "nuc"])
@pytest.mark.parametrize("masks,polytomy", [(False, False), (True, False), (False, True)])
def test_deferred_outgroups_equal_the_pass(alphabet, masks, polytomy):
    t = _treeanc(alphabet, masks, polytomy)
    want_og, want_tip = _reference_rows(t)
    for call in range(4):  # eager, captured, replayed, replayed
        t.infer_ancestral_sequences(marginal=True)
        got_og, got_tip = _deferred_rows(t)
        assert np.array_equal(_internal_rows(t, got_og), _internal_rows(t, want_og)), call
        assert np.array_equal(got_tip, want_tip), call
    # the node attributes read the same rows
    lay = t._get_session()["layout"]
    P = t.data.compressed_length
    for k in (0, lay.n_int // 2, lay.n_int + 3):
        n = lay.nodes[k]
        rows = want_tip[(k - lay.n_int) * P:(k - lay.n_int + 1) * P] if k >= lay.n_int else want_og[k * P:(k + 1) * P]
        np.testing.assert_array_equal(n.marginal_outgroup_LH, rows[:, :t.gtr.n_states].astype(np.float64))


def test_deferred_outgroups_belong_to_the_lengths_of_the_pass():
    t = _treeanc("nuc_nogap", False, False)
    for _ in range(3):
        t.infer_ancestral_sequences(marginal=True)
    want_og, want_tip = _reference_rows(t)
    t.infer_ancestral_sequences(marginal=True)
    for n in list(t.tree.find_clades())[1:30]:  # new lengths after the reconstruction
        n.branch_length = n.branch_length * 1.7 + 1e-3
    got_og, got_tip = _deferred_rows(t)
    assert np.array_equal(_internal_rows(t, got_og), _internal_rows(t, want_og))
    assert np.array_equal(got_tip, want_tip)


def test_changed_site_count_between_reconstructions():
    t = _treeanc("nuc", True, False)
    lay = t._get_session()["layout"]
    t.infer_ancestral_sequences(marginal=True)
    for step in range(4):
        before = {id(n): np.array(n._cseq) for n in lay.nodes[:lay.n_int - 1]}
        for n in list(t.tree.find_clades())[1::7]:
            n.branch_length = n.branch_length * (0.2 if step % 2 else 5.0) + 1e-4
        n_diff = t.infer_ancestral_sequences(marginal=True)
        want = sum(int((np.array(n._cseq) != before[id(n)]).sum()) for n in lay.nodes[:lay.n_int - 1])
        assert n_diff == want, step


def test_changed_site_count_with_tip_states():
    """With tip states reconstructed the pass counts the tips' rows too (the second range of
    tt_count_changes); the first such call counts against the alignment's states."""
    t = _treeanc("nuc_nogap", False, False, seed=12)
    lay = t._get_session()["layout"]
    rows = lay.nodes[:lay.n_int - 1] + lay.nodes[lay.n_int:]
    t.infer_ancestral_sequences(marginal=True, reconstruct_tip_states=True)
    for step in range(3):
        before = {id(n): np.array(n._cseq) for n in rows}
        for n in list(t.tree.find_clades())[1::5]:
            n.branch_length = n.branch_length * (0.3 if step % 2 else 4.0) + 1e-4
        n_diff = t.infer_ancestral_sequences(marginal=True, reconstruct_tip_states=True)
        want = sum(int((np.array(n._cseq) != before[id(n)]).sum()) for n in rows)
        assert n_diff == want, step
