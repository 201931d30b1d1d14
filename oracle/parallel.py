"""The oracle over a process pool (TEST INFRASTRUCTURE ONLY -- see
``oracle/__init__.py``).

Patterns (sites) are independent through every pass of TreeTime's marginal
and joint reconstructions, so the oracle's restatement (``oracle.anc``) runs
on column slices of the compressed alignment in a spawn-started pool and the
slices' results are put back together: the same numbers as one call on the
whole alignment, in a fraction of the time, for workloads of thousands of
tips and tens of thousands of patterns.

Every worker returns compact per-pattern results instead of whole profiles:
site log-likelihoods, the argmax state of every internal node with its
near-tie class, and the full profiles of the nodes asked for.
"""

import multiprocessing as mp
import os
import types

import numpy as np


def model_state(gtr, cols=None):
    """Picklable copy of the model attributes the oracle reads; for a
    site-specific model, restricted to the site columns ``cols`` (the
    interpolation grid stays that of the whole model, as in TreeTime)."""
    ss = bool(getattr(gtr, "is_site_specific", False))
    st = types.SimpleNamespace(alphabet=np.asarray(gtr.alphabet), profile_map=dict(gtr.profile_map),
                               gap_index=gtr.gap_index, is_site_specific=ss)
    if not ss:
        st.v, st.v_inv, st.eigenvals, st.mu, st.Pi = gtr.v, gtr.v_inv, gtr.eigenvals, gtr.mu, gtr.Pi
        return st
    c = slice(None) if cols is None else cols
    st.v = np.ascontiguousarray(gtr.v[:, :, c])
    st.v_inv = np.ascontiguousarray(gtr.v_inv[:, :, c])
    st.eigenvals = np.ascontiguousarray(gtr.eigenvals[:, c])
    st.mu = np.ascontiguousarray(np.asarray(gtr.mu)[c])
    st.Pi = np.ascontiguousarray(gtr.Pi[:, c])
    st.approximate = bool(gtr.approximate)
    st.rate_scale = float(gtr.rate_scale)
    st.t_grid = np.asarray(gtr.t_grid, dtype=float)
    return st


def _setup(newick, names, codes):
    from oracle import anc
    from treetime_gb300.tree import parse_newick
    tree = anc.prepare_tree(parse_newick(newick))
    chars = np.ascontiguousarray(codes).view("S1").astype("U1")
    aln = {k: chars[i] for i, k in enumerate(names)}
    internal = [n for n in anc.preorder(tree.root) if n.clades]
    return anc, tree, aln, internal


def _top2(p):
    s = np.sort(p, axis=1)
    return s[:, -1] - s[:, -2]


def _marginal_worker(args):
    newick, names, codes, mult, model, full_length, keep, tie_tols = args
    anc, tree, aln, internal = _setup(newick, names, codes)
    res = anc.marginal(tree, aln, mult, model, full_length)
    prof = res["profile"]
    states = np.empty((len(internal), len(mult)), dtype=np.uint8)
    near = np.zeros((len(internal), len(mult)), dtype=np.uint8)
    for k, n in enumerate(internal):
        p = prof[n.name]
        states[k] = p.argmax(axis=1).astype(np.uint8)
        m = _top2(p)
        for tol in tie_tols:
            near[k] += m < tol
    return dict(site_lh=res["sequence_LH"], states=states, near=near,
                profiles={k: prof[k] for k in keep if k in prof},
                subtree={k: res["subtree_LH"][k] for k in keep if k in res["subtree_LH"]},
                names=[n.name for n in internal])


def _joint_worker(args):
    newick, names, codes, mult, model, full_length, tie_tol = args
    anc, tree, aln, internal = _setup(newick, names, codes)
    res = anc.joint(tree, aln, mult, model, full_length)
    tie = res["root_margin"] < tie_tol
    for n in anc.preorder(tree.root):
        if n.up is None or n.name not in res["margin"]:
            continue
        ps = res["seq_idx"].get(n.up.name)
        if ps is None:
            continue
        tie |= res["margin"][n.name][np.arange(len(ps)), ps] < tie_tol
    states = np.stack([np.asarray(res["seq_idx"][n.name], dtype=np.uint8) for n in internal])
    return dict(site_lh=res["sequence_LH"], states=states, tie=tie, names=[n.name for n in internal])


def _chunks(P, workers):
    n = max(1, min(workers, P))
    return [slice(i * P // n, (i + 1) * P // n) for i in range(n)]


def _run(fn, jobs, workers):
    if len(jobs) == 1:
        return [fn(jobs[0])]
    with mp.get_context("spawn").Pool(min(workers, len(jobs))) as pool:
        return pool.map(fn, jobs)


def _merge(parts, keys=("site_lh",), cat1=("states",)):
    out = {k: np.concatenate([p[k] for p in parts]) for k in keys}
    for k in cat1:
        out[k] = np.concatenate([p[k] for p in parts], axis=1)
    out["names"] = parts[0]["names"]
    return out


def marginal(newick, names, codes, mult, gtr, full_length, keep=(), tie_tols=(1e-9, 1e-5), workers=None):
    """TreeTime's marginal reconstruction (oracle.anc.marginal) of the tree
    ``newick`` and the compressed alignment ``codes`` ([tips][patterns] bytes,
    rows named by ``names``) split over a pool.  Returns site_lh [P],
    total (sum of site_lh * mult), states [n_internal, P] (argmax index of the
    posterior), near [n_internal, P] (how many of ``tie_tols`` the posterior's
    top-two margin is below), names (internal nodes, preorder), and profiles /
    subtree {name: [P, q]} of the nodes in ``keep``."""
    P = len(mult)
    workers = workers or os.cpu_count() or 1
    sl = _chunks(P, workers)
    ss = bool(getattr(gtr, "is_site_specific", False))
    jobs = [(newick, list(names), np.ascontiguousarray(codes[:, s]), np.asarray(mult)[s],
             model_state(gtr, s if ss else None), full_length, tuple(keep), tuple(tie_tols)) for s in sl]
    parts = _run(_marginal_worker, jobs, workers)
    out = _merge(parts, cat1=("states", "near"))
    for key in ("profiles", "subtree"):
        out[key] = {k: np.concatenate([p[key][k] for p in parts]) for k in parts[0][key]}
    out["total"] = float((out["site_lh"] * np.asarray(mult)).sum())
    return out


def joint(newick, names, codes, mult, gtr, full_length, tie_tol=1e-9, workers=None):
    """TreeTime's joint reconstruction (oracle.anc.joint) split over a pool.
    Returns site_lh [P], total, states [n_internal, P] (state indices), tie
    [P] (patterns where the reference's top-two margin at some node of the
    chosen path is below ``tie_tol``) and names (internal nodes, preorder)."""
    P = len(mult)
    workers = workers or os.cpu_count() or 1
    ss = bool(getattr(gtr, "is_site_specific", False))
    jobs = [(newick, list(names), np.ascontiguousarray(codes[:, s]), np.asarray(mult)[s],
             model_state(gtr, s if ss else None), full_length, tie_tol) for s in _chunks(P, workers)]
    out = _merge(_run(_joint_worker, jobs, workers), keys=("site_lh", "tie"))
    out["total"] = float((out["site_lh"] * np.asarray(mult)).sum())
    return out


def _marginal_bl_worker(args):
    newick, names, codes, mult, model, full_length, branch_names, tol = args
    anc, tree, aln, internal = _setup(newick, names, codes)
    res = anc.marginal(tree, aln, mult, model, full_length)
    out = {}
    for k in branch_names:
        pp, pc = res["outgroup_LH"][k], res["subtree_LH"][k]
        out[k] = anc.optimal_t_compressed(model, (pp, pc), mult, profiles=True, tol=tol)[0]
    return out


def marginal_branch_lengths(newick, names, codes, mult, gtr, full_length, tol=1e-10, workers=None):
    """TreeTime's optimal_marginal_branch_length (oracle.anc.optimal_t_compressed
    with profiles, scipy's Brent) for every non-root branch after a marginal
    reconstruction, the branches split over a pool (each process reconstructs
    the whole tree once).  Returns {node name: t}."""
    from oracle import anc
    from treetime_gb300.tree import parse_newick
    tree = anc.prepare_tree(parse_newick(newick))
    branches = [n.name for n in anc.preorder(tree.root) if n.up is not None]
    workers = workers or os.cpu_count() or 1
    n = max(1, min(workers, len(branches)))
    jobs = [(newick, list(names), np.ascontiguousarray(codes), np.asarray(mult), model_state(gtr), full_length,
             branches[i::n], tol) for i in range(n)]
    out = {}
    for part in _run(_marginal_bl_worker, jobs, workers):
        out.update(part)
    return out
