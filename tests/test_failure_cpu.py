"""Host-side failure detection (no GPU): the conditions under which TreeTime
raises, or silently repairs its input, are caught or repaired the same way
before anything is launched.

* exp(Q t) with mu*lambda*t > 10 -- a model with a positive eigenvalue --
  raises TreeTime's ValueError (treetime/gtr.py:1042-1047), both in the
  pre-launch check of the engine and in the GTR object's own check;
* a NaN branch length becomes the branch-length floor, as Python's
  max(floor, nan) does in TreeAnc._branch_length_to_gtr
  (treetime/treeanc.py:752-760);
* an oversize branch length of a standard model (all eigenvalues <= 0) does
  not raise in TreeTime and does not raise here either.
"""

import copy

import numpy as np
import pytest

from oracle import anc
from treetime_gb300 import engine, synth
from treetime_gb300.gtr import GTR


def _positive_model():
    g = GTR.standard("JC69", alphabet="nuc_nogap")
    bad = copy.deepcopy(g)
    bad.eigenvals = np.array(bad.eigenvals, dtype=float)
    bad.eigenvals[-1] = 0.5  # a rate matrix with a positive eigenvalue
    return g, bad


def test_positive_eigenvalue_raises_treetimes_value_error():
    g, bad = _positive_model()
    t = np.array([1e-3, 0.1, 25.0])
    # TreeTime's own expression raises at t = 25 (mu * 0.5 * 25 > 10) ...
    with pytest.raises(ValueError):
        anc.expQt(bad, 25.0)
    # ... and so do the engine's pre-launch check and the model's check, with TreeTime's message
    with pytest.raises(ValueError, match="Q has positive eigenvalues or the branch length t is too large"):
        engine.check_exp(bad, t)
    with pytest.raises(ValueError, match="Q has positive eigenvalues"):
        bad.check_branch_lengths(t)
    # below the limit both accept it
    anc.expQt(bad, 1.0)
    engine.check_exp(bad, np.array([1.0, 19.9]))


def test_oversize_branch_of_a_standard_model_does_not_raise():
    g, _ = _positive_model()
    t = np.array([1e-6, 4.0, 1e6])
    anc.expQt(g, 1e6)          # TreeTime: all mu*lambda*t <= 0, no error
    engine.check_exp(g, t)
    g.check_branch_lengths(t)


def test_nan_branch_length_takes_the_floor_like_treetime():
    wl = synth.make_workload("c0", seed=5, n=10, L=50)
    tree = anc.prepare_tree(wl["tree"])
    layout = engine.TreeLayout(tree.root)
    nodes = layout.nodes
    nodes[3].branch_length = float("nan")
    nodes[-1].branch_length = float("nan")
    L = 50
    got = engine.branch_lengths(layout, L)
    want = np.array([anc.branch_length_to_gtr(n, L) for n in nodes])
    np.testing.assert_array_equal(got, want)
    assert np.isfinite(got).all() and got[3] == got[-1] == 1e-3 / L
