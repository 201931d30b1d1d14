"""The allocation-free joint entry point (tt_joint_noalloc).

Callers that cannot allocate device memory -- hosts that hand out only their
own pre-sized buffers, pools that reserve all device memory at start-up,
paths that cannot afford an allocation's implicit synchronisation -- call
tt_joint_noalloc, whose scratch is a fixed array inside the library.  These
tests call it through the C ABI and compare it with the allocating entry point
(tt_branch_pmats + tt_joint) on the same inputs, on two calls in a row (the
shared scratch keeps the first call's contents), and check that a wrong row
count is refused instead of overrunning the scratch.  The file is named so
that pytest collects it last.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _forest(n=40, L=300, seed=21, trees=1):
    """A forest of `trees` trees (different sizes, one model each) and its
    internal-node pattern rows."""
    from oracle import anc
    from treetime_gb300 import engine, synth
    from treetime_gb300.seqdata import SequenceData
    inputs, gtrs = [], []
    for k in range(trees):
        wl = synth.make_workload("c0", seed=seed + k, n=n + 7 * k, L=L + 53 * k)
        tree = anc.prepare_tree(wl["tree"])
        sd = SequenceData(wl["aln"], ambiguous="N")
        layout = engine.TreeLayout(tree.root)
        tip_row = np.array([sd.name_to_row[x.name] for x in layout.nodes[layout.n_int:]], dtype=np.int32)
        inputs.append(engine.TreeInput(layout, sd.compressed_codes, tip_row, sd.multiplicity(),
                                       engine.branch_lengths(layout, sd.full_length), model=k))
        gtrs.append(wl["gtr"])
    forest = engine.Forest(inputs, 4)
    model = engine.DeviceModel(gtrs)
    return forest, model, sum(ti.layout.n_int * ti.n_patterns for ti in inputs)


def _noalloc(forest, model, rows, expect_status=0):
    import torch
    from treetime_gb300 import _lib, engine
    lib = _lib.load()
    states = torch.zeros(forest.state_rows, dtype=torch.uint8, device=forest.device)
    site = torch.zeros(forest.n_patterns, dtype=torch.float64, device=forest.device)
    tree = torch.zeros(len(forest.inputs), dtype=torch.float64, device=forest.device)
    status = torch.zeros(1, dtype=torch.int32, device=forest.device)
    st = lib.tt_joint_noalloc(C.byref(forest.struct), C.byref(model.struct), rows, engine._p(states), engine._p(site),
                              engine._p(tree), None, None, 0, 0, engine._p(status), engine._stream())
    _lib.check(st, "tt_joint_noalloc")
    torch.cuda.synchronize()
    assert int(status.item()) == expect_status
    return states.cpu().numpy(), site.cpu().numpy(), tree.cpu().numpy()


def _reference(forest, model):
    from treetime_gb300 import engine
    ref = engine.joint(forest, model, engine.Buffers(forest))
    return ref["states"].cpu().numpy(), ref["site_lh"].cpu().numpy(), ref["tree_lh"].cpu().numpy()


def _internal_rows_equal(forest, got, want):
    for t, ti in enumerate(forest.inputs):
        tr = forest.trees_host[t]
        a = int(tr["state_base"])
        b = a + ti.layout.n_int * ti.n_patterns
        # internal nodes carry the reconstruction; tip rows are not written without tip reconstruction
        np.testing.assert_array_equal(got[a:b], want[a:b])


def test_noalloc_joint_equals_allocating_entry_point_twice():
    """Two calls in a row: a larger two-tree forest, then a smaller one-tree
    forest of other data (its rows lie over the first call's leftovers in the
    shared scratch); each equals the allocating entry point on its own
    inputs."""
    big, big_model, big_rows = _forest(n=60, L=500, seed=31, trees=2)
    small, small_model, small_rows = _forest(n=25, L=180, seed=7, trees=1)
    for forest, model, rows in ((big, big_model, big_rows), (small, small_model, small_rows)):
        want_states, want_site, want_tree = _reference(forest, model)
        states, site, tree = _noalloc(forest, model, rows)
        _internal_rows_equal(forest, states, want_states)
        np.testing.assert_allclose(site, want_site, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(tree, want_tree, rtol=1e-12, atol=0)


def test_noalloc_undercounted_rows_are_refused_not_overrun():
    """internal_rows below what the forest needs: the kernel skips the trees
    whose rows do not fit (TT_ERR_OOM in the status word) instead of writing
    past the scratch rows; the trees that fit are still reconstructed."""
    from treetime_gb300 import _lib
    forest, model, rows = _forest(n=30, L=200, seed=3, trees=2)
    first = forest.inputs[0].layout.n_int * forest.inputs[0].n_patterns
    want_states, want_site, _ = _reference(forest, model)
    states, site, _ = _noalloc(forest, model, first, expect_status=_lib.TT_ERR_OOM)
    tr0 = forest.trees_host[0]
    a, b = int(tr0["state_base"]), int(tr0["state_base"]) + first
    np.testing.assert_array_equal(states[a:b], want_states[a:b])
    P0 = forest.inputs[0].n_patterns
    np.testing.assert_allclose(site[:P0], want_site[:P0], rtol=1e-12, atol=1e-12)


def test_noalloc_rejects_problems_beyond_the_fixed_scratch():
    from treetime_gb300 import _lib, engine
    forest, model, rows = _forest(n=8, L=50)
    lib = _lib.load()
    st = lib.tt_joint_noalloc(C.byref(forest.struct), C.byref(model.struct), 1 << 40, None, None, None, None, None,
                              0, 0, None, engine._stream())
    assert st == _lib.TT_ERR_INVALID
    import torch
    d = lambda n, t: torch.zeros(n, dtype=t, device=forest.device)
    states, site, tree = d(forest.state_rows, torch.uint8), d(forest.n_patterns, torch.float64), d(1, torch.float64)
    st = lib.tt_joint_noalloc(C.byref(forest.struct), C.byref(model.struct), 1 << 40, engine._p(states),
                              engine._p(site), engine._p(tree), None, None, 0, 0, None, engine._stream())
    assert st == _lib.TT_ERR_OOM
    assert "fixed scratch" in _lib.last_error()
