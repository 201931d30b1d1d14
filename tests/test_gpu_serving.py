"""GPU: the serving loop.  Every job's results (per-iteration log-likelihood,
reconstructed states, final branch lengths) are the same whether the job runs
alone or in a mix of jobs that overlap on the device (continuous batching,
one stream per admitted job), for reconstruction and branch-length jobs,
nucleotide and site-specific protein models; a tight memory budget queues
jobs without changing their results."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jobs(seed=21):
    from treetime_gb300 import TreeAnc, serving, synth
    inputs, gtrs = synth.forest_c3(n_trees=8, seed=seed, n_range=(20, 300), L_range=(200, 3000),
                                   bl_range=(1e-3, 0.05))
    jobs = []
    for k, (ti, g) in enumerate(zip(inputs, gtrs)):
        jobs.append(serving.Job(ti, g, kind="optimize" if k % 2 else "marginal", iterations=3))
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
    jobs = [j for j in _jobs(seed=22) if j.kind == "optimize"]
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
