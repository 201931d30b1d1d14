"""GPU: the serving loop.  Every job's results (per-iteration log-likelihood,
reconstructed states, final branch lengths) are the same whether the job runs
alone or in a mix of jobs that overlap on the device (continuous batching,
one stream per admitted job), for reconstruction, marginal and joint
branch-length jobs, nucleotide and site-specific protein models; a tight
memory budget queues jobs without changing their results; and each kind of
served job gives the results of the same work through TreeAnc."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jobs(seed=21):
    from treetime_gb300 import TreeAnc, serving, synth
    inputs, gtrs = synth.forest_c3(n_trees=8, seed=seed, n_range=(20, 300), L_range=(200, 3000),
                                   bl_range=(1e-3, 0.05))
    jobs = []
    for k, (ti, g) in enumerate(zip(inputs, gtrs)):
        jobs.append(serving.Job(ti, g, kind=("marginal", "optimize", "joint")[k % 3], iterations=3))
    # two protein jobs with a site-specific model
    for s in (1, 2):
        wl = synth.make_workload("c2", seed=30 + s, n=25, L=60)
        t = TreeAnc(tree=wl["tree"], aln=wl["aln"], gtr=wl["gtr"], compress=False, verbose=0)
        sess = t._get_session()
        jobs.append(serving.Job(sess["forest"].inputs[0], t.gtr, kind="marginal", iterations=3))
    return jobs


def _run(jobs, arrivals, **kw):
    from treetime_gb300 import serving
    srv = serving.Server(**kw)
    done, wall = srv.serve(jobs, arrivals)
    assert all(j.result is not None for j in done)
    assert all(np.isfinite(j.result["tree_lh"]).all() for j in done)
    return {j.id: j.result for j in done}, srv


def test_alone_equals_mix():
    jobs = _jobs()
    alone = {}
    for j in jobs:
        res, _ = _run([j], [0.0], max_slots=1)
        alone.update(res)
    mix_jobs = _jobs()  # the same jobs again (new objects, same data), all arriving together
    for a, b in zip(jobs, mix_jobs):
        b.id = a.id
    mixed, srv = _run(mix_jobs, np.zeros(len(mix_jobs)), max_slots=8)
    assert srv.peak_active > 1
    for jid, ra in alone.items():
        rb = mixed[jid]
        np.testing.assert_array_equal(ra["tree_lh"], rb["tree_lh"])
        np.testing.assert_array_equal(ra["states"], rb["states"])
        np.testing.assert_array_equal(ra["branch_lengths"], rb["branch_lengths"])


def test_branch_length_jobs_raise_the_likelihood():
    jobs = [j for j in _jobs(seed=22) if j.kind != "marginal"]
    res, _ = _run(jobs, np.zeros(len(jobs)), max_slots=4)
    for j in jobs:
        lh = res[j.id]["tree_lh"]
        assert lh[-1] >= lh[0] - 1e-6 * abs(lh[0])


def test_memory_budget_queues_without_changing_results():
    jobs = _jobs(seed=23)
    base, _ = _run(jobs, np.zeros(len(jobs)), max_slots=8)
    tight_jobs = _jobs(seed=23)
    for a, b in zip(jobs, tight_jobs):
        b.id = a.id
    budget = max(j.footprint for j in tight_jobs) + 1
    tight, srv = _run(tight_jobs, np.zeros(len(tight_jobs)), max_slots=8, hbm_bytes=budget)
    assert srv.peak_bytes <= budget
    assert srv.peak_active < len(tight_jobs)
    for jid in base:
        np.testing.assert_array_equal(base[jid]["tree_lh"], tight[jid]["tree_lh"])


def _served_and_treeanc(kind, seed, iterations=3, n=40, L=400):
    """A job served in a mix, and the same tree, alignment and model through
    treetime_gb300.TreeAnc (FP32 profiles, as the serving loop uses)."""
    from treetime_gb300 import TreeAnc, serving, synth
    from treetime_gb300.tree import parse_newick, to_newick
    wl = synth.make_workload("c0", seed=seed, n=n, L=L, gap_frac=0.02)
    nwk = to_newick(wl["tree"])
    make = lambda: TreeAnc(tree=parse_newick(nwk), aln=wl["aln"], gtr=wl["gtr"], verbose=0, precision="f32")
    t1 = make()
    job = serving.Job(t1._get_session()["forest"].inputs[0], t1.gtr, kind=kind, iterations=iterations)
    return job, make()


def _states_of(t):
    lay = t._get_session()["layout"]
    idx = {c: i for i, c in enumerate(t.gtr.alphabet)}
    return np.stack([[idx[c] for c in n._cseq] for n in lay.nodes[:lay.n_int]]), lay


def test_served_results_equal_treeanc():
    """Each kind of served job against the same job through TreeAnc:
      * "marginal": the last iteration's log-likelihood and states equal
        infer_ancestral_sequences(marginal=True);
      * "optimize": the branch lengths after three damped updates equal
        optimize_tree_marginal(max_iter=3) with its log-likelihood stop
        disabled, the root's two children updated as one branch at both visits
        (the tree has a bifurcating root);
      * "joint": states, log-likelihood and branch lengths equal
        optimize_tree(branch_length_mode="joint", max_iter=2, prune_short=False)
        (three rounds of reconstruction and branch lengths).
    Served in a mix of jobs (1e-10 relative: the same kernels on the same inputs)."""
    jm, tm = _served_and_treeanc("marginal", 61)
    jo, to = _served_and_treeanc("optimize", 62)
    jj, tj = _served_and_treeanc("joint", 63)
    assert len(to.tree.root.clades) == 2
    others = [j for j in _jobs(seed=24)]
    res, srv = _run([jm, jo, jj] + others, np.zeros(3 + len(others)), max_slots=8)
    assert srv.peak_active > 1
    floor = lambda t, bl: np.fmax(1e-3 / t.data.full_length, bl)

    tm.infer_ancestral_sequences(marginal=True)
    r = res[jm.id]
    assert abs(r["tree_lh"][-1] - tm.tree.total_sequence_LH) <= 1e-10 * abs(tm.tree.total_sequence_LH)
    states, lay = _states_of(tm)
    np.testing.assert_array_equal(r["states"], states)

    to.optimize_tree_marginal(max_iter=3, LHtol=-np.inf)
    lay = to._get_session()["layout"]
    want = floor(to, np.array([n.branch_length for n in lay.nodes]))
    got = res[jo.id]["branch_lengths"]
    root = lay.n_int - 1
    keep = np.arange(lay.n_nodes) != root
    np.testing.assert_allclose(got[keep], want[keep], rtol=1e-10, atol=0)

    tj.optimize_tree(branch_length_mode="joint", max_iter=2, prune_short=False)
    r = res[jj.id]
    lay = tj._get_session()["layout"]
    want = floor(tj, np.array([n.branch_length for n in lay.nodes]))
    keep = np.arange(lay.n_nodes) != lay.n_int - 1
    np.testing.assert_allclose(r["branch_lengths"][keep], want[keep], rtol=1e-10, atol=0)
    assert abs(r["tree_lh"][-1] - tj.tree.unconstrained_sequence_LH) <= 1e-10 * abs(tj.tree.unconstrained_sequence_LH)
    states, _ = _states_of(tj)
    np.testing.assert_array_equal(r["states"], states)
