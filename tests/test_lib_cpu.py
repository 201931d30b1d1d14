"""CPU-only checks of the C-ABI library and the host-side schedule: the shared
library loads, exports every entry point the public header declares, and the
tree flattening produces a valid height-levelled CSR schedule."""

import ctypes
import os
import re

import numpy as np
import pytest

from treetime_gb300 import _lib, synth
from treetime_gb300.engine import TreeLayout

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "treetime_gb300.h")


def _declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tt_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from treetime_gb300 import build
    build.build()
    return _lib.load()


def test_header_declares_the_bound_entry_points():
    assert _declared() == _lib.exported_names()


def test_library_exports_every_declared_symbol(lib):
    raw = ctypes.CDLL(_lib.LIB_PATH)
    for name in _declared():
        assert hasattr(raw, name), name
    assert lib.tt_abi_version() == 1
    assert lib.tt_status_string(7).decode().startswith("Brent")


def _check_layout(tree):
    L = TreeLayout(tree.root)
    n = L.n_nodes
    assert L.nodes[L.n_int - 1] is tree.root
    assert L.parent[L.n_int - 1] == -1
    assert (L.parent[:L.n_int - 1] >= 0).all() and (L.parent[L.n_int:] >= 0).all()
    # children are listed in clade order and always come before the parent level
    lev = L.level_off
    height = np.zeros(n, dtype=int)
    for h in range(L.n_levels):
        height[lev[h]:lev[h + 1]] = h + 1
    for k in range(L.n_int):
        ch = L.child_idx[L.child_off[k]:L.child_off[k + 1]]
        assert [L.nodes[c] for c in ch] == list(L.nodes[k].clades)
        assert all(height[c] < height[k] for c in ch)
        assert all(L.parent[c] == k for c in ch)
    assert lev[0] == 0 and lev[-1] == L.n_int
    # tips in preorder
    assert [t.name for t in L.nodes[L.n_int:]] == [t.name for t in tree.get_terminals()]
    return L


@pytest.mark.parametrize("n", [3, 17, 200])
def test_tree_layout_coalescent(n):
    tree = synth.coalescent_tree(n, 0.01, np.random.default_rng(n))
    _check_layout(tree)


def test_tree_layout_caterpillar_and_polytomy():
    from treetime_gb300.tree import parse_newick
    cat = "(" * 300 + "a:1,b:1)" + "".join(",t%d:1)" % i for i in range(299)) + ";"
    L = _check_layout(parse_newick(cat))
    assert L.n_levels == 300
    L = _check_layout(parse_newick("((a,b,c,d)x,(e,f)y,g,h)r;"))
    assert L.n_levels == 2


def test_uncompiled_alphabet_size_fails_before_launch():
    """A custom alphabet whose size the tree kernels were not compiled for
    raises NotImplementedError at the public call, before any device work; the
    serving front end refuses such a job when it is created."""
    from treetime_gb300 import GTR, TreeAnc
    from treetime_gb300.engine import check_alphabet
    from treetime_gb300.serving import Job
    g = GTR.custom(pi=np.ones(7) / 7, W=np.ones((7, 7)), alphabet=np.array(list("ABCDEFG")))
    aln = {"a": "ABCDEFG", "b": "ABCDEFF", "c": "ABCDEGG", "d": "GBCDEFG"}
    t = TreeAnc(tree="((a:0.1,b:0.2):0.05,c:0.3,d:0.1);", aln=aln, gtr=g, verbose=0)
    for marginal in (False, True):
        with pytest.raises(NotImplementedError, match="alphabet size 7"):
            t.infer_ancestral_sequences(marginal=marginal)
    with pytest.raises(NotImplementedError, match="alphabet size 7"):
        Job(None, g)
    for q in (4, 5, 20, 21, 22):
        check_alphabet(q)
    with pytest.raises(NotImplementedError):
        check_alphabet(5, site_specific=True)


def test_profile_branch_groups_rows():
    """The branch lists of the profile-mode calls (host logic): internal
    branches read their child rows from the partials, tips from their codes
    (child row -1, parent row in the tip outgroup buffer); positions refer to
    the caller's node order."""
    from types import SimpleNamespace
    from treetime_gb300.anc_gpu import GPUAncMixin
    tree = synth.coalescent_tree(40, 0.01, np.random.default_rng(3))
    L = TreeLayout(tree.root)
    P = 17
    out = {"outgroup": "OUT", "tip_outgroup": "TIPOUT", "partial": "PART"}
    host = SimpleNamespace(_last=("marginal", out), data=SimpleNamespace(compressed_length=P))
    root = L.nodes[L.n_int - 1]
    nodes = [n for n in L.nodes if n is not root]
    order = np.random.default_rng(4).permutation(len(nodes))
    nodes = [nodes[i] for i in order]
    seen = np.zeros(len(nodes), bool)
    groups = list(GPUAncMixin._profile_branch_groups(host, nodes, {"layout": L}))
    assert [g[2] for g in groups] == ["OUT", "TIPOUT"]
    for idx, kk, pp, pp_row, pc_row, pc in groups:
        assert pc == "PART" and kk.dtype == np.int32 and pp_row.dtype == np.int64 and pc_row.dtype == np.int64
        for i, k, r, c in zip(idx, kk, pp_row, pc_row):
            assert L.local[id(nodes[i])] == k
            seen[i] = True
            if k < L.n_int:
                assert pp == "OUT" and r == k * P and c == k * P
            else:
                assert pp == "TIPOUT" and r == (k - L.n_int) * P and c == -1
    assert seen.all()


@pytest.mark.parametrize("alphabet,ignore_gaps", [("nuc", True), ("nuc", False), ("nuc_nogap", True), ("aa", True)])
def test_pair_counts_equal_state_pair(alphabet, ignore_gaps):
    """The host pair counts used for a re-parented node when pruning equal
    TreeTime's GTR.state_pair (the oracle's restatement, both alphabet-size
    branches) after its cast to integers, with masked multiplicities."""
    from oracle import anc
    from treetime_gb300.anc_gpu import pair_counts
    from treetime_gb300.gtr import GTR
    g = GTR.standard("JC69", alphabet=alphabet)
    q = g.n_states
    rng = np.random.default_rng(q + ignore_gaps)
    L = 500
    a = rng.integers(q, size=L)
    b = np.where(rng.random(L) < 0.2, rng.integers(q, size=L), a)
    mult = rng.integers(1, 5, size=L) * np.where(rng.random(L) < 0.3, 0.5, 1.0)
    got = np.trunc(pair_counts(a, b, mult, q, g.gap_index, ignore_gaps))
    pairs, cnt = anc.state_pair(g, g.alphabet[a], g.alphabet[b], pattern_multiplicity=mult, ignore_gaps=ignore_gaps)
    want = np.zeros((q, q))
    for (i, j), c in zip(pairs, cnt):
        want[i, j] = c
    np.testing.assert_array_equal(got, want)


def test_model_cache_is_a_bounded_lru(monkeypatch):
    """engine.model_for keeps the DeviceModels of the most recently used GTR
    objects (bounded), rebuilds one when the model's numbers change, and an
    entry keeps its GTR alive (so its id cannot be taken by another object)."""
    from treetime_gb300 import engine
    from treetime_gb300.gtr import GTR

    class FakeModel:
        def __init__(self, gtrs, device=None):
            self.gtrs = [gtrs]

    monkeypatch.setattr(engine, "DeviceModel", FakeModel)
    monkeypatch.setattr(engine, "require_device", lambda device=None: "cpu")
    monkeypatch.setattr(engine, "_MODEL_CACHE", engine.collections.OrderedDict())
    monkeypatch.setattr(engine, "MODEL_CACHE_SIZE", 3)
    gs = [GTR.standard("JC69", alphabet="nuc_nogap") for _ in range(5)]
    first = engine.model_for(gs[0])
    assert engine.model_for(gs[0]) is first                      # cached
    for g in gs[1:4]:
        engine.model_for(g)
    assert len(engine._MODEL_CACHE) == 3 and id(gs[0]) not in engine._MODEL_CACHE  # least recent evicted
    engine.model_for(gs[1])                                       # gs[1] becomes the most recent
    engine.model_for(gs[4])
    assert id(gs[2]) not in engine._MODEL_CACHE and id(gs[1]) in engine._MODEL_CACHE
    m1 = engine.model_for(gs[1])
    gs[1].assign_rates(mu=2.0)                                    # new numbers: rebuilt
    assert engine.model_for(gs[1]) is not m1
    assert all(e[1].gtrs[0] is not None for e in engine._MODEL_CACHE.values())
