"""The allocation-free joint entry point (tt_joint_noalloc).

Callers that cannot allocate device memory -- hosts that hand out only their
own pre-sized buffers, pools that reserve all device memory at start-up,
paths that cannot afford an allocation's implicit synchronisation -- call
tt_joint_noalloc, whose scratch is a fixed array inside the library.  These
tests call it through the C ABI and compare it with the allocating entry point
(tt_branch_pmats + tt_joint) on the same inputs, on two calls in a row (the
shared scratch keeps the first call's contents).  The file is named so that
pytest collects it last.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _forest(n=40, L=300, seed=21):
    from oracle import anc
    from treetime_gb300 import engine, synth
    from treetime_gb300.seqdata import SequenceData
    wl = synth.make_workload("c0", seed=seed, n=n, L=L)
    tree = anc.prepare_tree(wl["tree"])
    sd = SequenceData(wl["aln"], ambiguous="N")
    layout = engine.TreeLayout(tree.root)
    tip_row = np.array([sd.name_to_row[x.name] for x in layout.nodes[layout.n_int:]], dtype=np.int32)
    ti = engine.TreeInput(layout, sd.compressed_codes, tip_row, sd.multiplicity(),
                          engine.branch_lengths(layout, sd.full_length))
    forest = engine.Forest([ti], 4)
    model = engine.DeviceModel([wl["gtr"]])
    return forest, model, layout.n_int * ti.n_patterns


def _noalloc(forest, model, rows):
    import torch
    from treetime_gb300 import _lib, engine
    lib = _lib.load()
    states = torch.zeros(forest.state_rows, dtype=torch.uint8, device=forest.device)
    site = torch.zeros(forest.n_patterns, dtype=torch.float64, device=forest.device)
    tree = torch.zeros(1, dtype=torch.float64, device=forest.device)
    status = torch.zeros(1, dtype=torch.int32, device=forest.device)
    st = lib.tt_joint_noalloc(C.byref(forest.struct), C.byref(model.struct), rows, engine._p(states), engine._p(site),
                              engine._p(tree), None, None, 0, 0, engine._p(status), engine._stream())
    _lib.check(st, "tt_joint_noalloc")
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    return states.cpu().numpy(), site.cpu().numpy(), float(tree.item())


def test_noalloc_joint_equals_allocating_entry_point_twice():
    from treetime_gb300 import engine
    forest, model, rows = _forest()
    ref = engine.joint(forest, model, engine.Buffers(forest))
    ref_states = ref["states"].cpu().numpy()
    ref_site = ref["site_lh"].cpu().numpy()
    ref_tree = float(ref["tree_lh"][0].item())
    n_int = forest.inputs[0].layout.n_int
    P = forest.inputs[0].n_patterns
    for _ in range(2):
        states, site, tree = _noalloc(forest, model, rows)
        # internal nodes carry the reconstruction; tip rows are not written without tip reconstruction
        np.testing.assert_array_equal(states[: n_int * P], ref_states[: n_int * P])
        np.testing.assert_allclose(site, ref_site, rtol=1e-12, atol=1e-12)
        assert abs(tree - ref_tree) <= 1e-12 * abs(ref_tree)


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
