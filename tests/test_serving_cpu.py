"""Host logic of the serving loop (no GPU): the admission policy (arrival
order while a slot is free and the device footprint fits; a job that does not
fit holds the head of the queue), the staging of tip codes at submission, and
the scheduler loop with its device work stood in for (admission order, slots,
collection, error reporting)."""

from types import SimpleNamespace

import numpy as np
import pytest

from treetime_gb300.serving import footprint, plan_admissions


def _job(fp, name):
    return SimpleNamespace(footprint=fp, name=name)


def test_admits_in_order_within_slots_and_bytes():
    q = [_job(10, "a"), _job(20, "b"), _job(30, "c"), _job(5, "d")]
    assert [j.name for j in plan_admissions(q, 2, 1000)] == ["a", "b"]
    assert [j.name for j in plan_admissions(q, 10, 60)] == ["a", "b", "c"]
    assert [j.name for j in plan_admissions(q, 10, 1000)] == ["a", "b", "c", "d"]


def test_head_of_queue_blocks_smaller_later_jobs():
    q = [_job(100, "big"), _job(1, "small")]
    assert plan_admissions(q, 4, 50) == []
    assert plan_admissions([], 4, 50) == []
    assert plan_admissions(q, 0, 10 ** 9) == []


def test_footprint_grows_with_size_and_kind():
    from treetime_gb300 import engine, synth
    (small,), _ = synth.forest_c3(n_trees=1, seed=1, n_range=(20, 21), L_range=(100, 101))
    (big,), _ = synth.forest_c3(n_trees=1, seed=1, n_range=(400, 401), L_range=(2000, 2001))
    assert small.layout.n_nodes * small.n_patterns < big.layout.n_nodes * big.n_patterns
    assert footprint(small, 4, "marginal") < footprint(big, 4, "marginal")
    assert footprint(big, 4, "marginal") < footprint(big, 4, "optimize")
    rows = big.layout.n_int * big.n_patterns * 4 * 4
    assert footprint(big, 4, "marginal") >= 2 * rows


def test_submit_stages_codes_for_a_bounded_number_of_waiting_jobs():
    """Submitting copies a job's tip codes into a (here: ordinary) host buffer
    of the pool while fewer than 2 x max_slots waiting jobs hold one; later
    jobs are packed at admission instead."""
    import collections
    import threading
    import torch
    from treetime_gb300 import engine, synth
    from treetime_gb300.gtr import GTR
    from treetime_gb300.serving import Job, Server

    class Pool:
        def take(self, n):
            return torch.zeros(max(n, 1), dtype=torch.uint8)

    tree = synth.coalescent_tree(12, 0.01, np.random.default_rng(0))
    lay = engine.TreeLayout(tree.root)
    rng = np.random.default_rng(1)
    codes = rng.choice(np.frombuffer(b"ACGT", np.uint8), size=(lay.n_tip, 50))
    ti = engine.TreeInput(lay, codes, np.arange(lay.n_tip, dtype=np.int32), np.ones(50), np.full(lay.n_nodes, 0.01))
    g = GTR.standard("JC69", alphabet="nuc_nogap")
    srv = object.__new__(Server)  # the queueing half of the server, without a device
    srv.max_slots, srv._lock, srv._queue = 2, threading.Lock(), collections.deque()
    srv._staged_waiting, srv._pinned, srv.hbm_bytes = 0, Pool(), 1 << 40
    jobs = [Job(ti, g) for _ in range(6)]
    for j in jobs:
        srv.submit(j)
    staged = [j._codes_buf is not None for j in jobs]
    assert staged == [True] * 4 + [False] * 2 and srv._staged_waiting == 4 and len(srv._queue) == 6
    np.testing.assert_array_equal(jobs[0]._codes_buf[:codes.size].numpy(), codes.reshape(-1))


def _small_job_inputs():
    from treetime_gb300 import engine, synth
    from treetime_gb300.gtr import GTR
    tree = synth.coalescent_tree(8, 0.01, np.random.default_rng(2))
    lay = engine.TreeLayout(tree.root)
    codes = np.random.default_rng(3).choice(np.frombuffer(b"ACGT", np.uint8), size=(lay.n_tip, 20))
    ti = engine.TreeInput(lay, codes, np.arange(lay.n_tip, dtype=np.int32), np.ones(20), np.full(lay.n_nodes, 0.01))
    return ti, GTR.standard("JC69", alphabet="nuc_nogap")


def _fake_server(monkeypatch, max_slots, polls_until_done=3):
    """A Server whose device work is replaced by a stand-in that finishes a
    job after a few scheduler polls (host logic only)."""
    import torch
    from types import SimpleNamespace
    from treetime_gb300 import engine, serving

    class Pool:
        def take(self, n):
            return torch.zeros(max(n, 1), dtype=torch.uint8)

        def give(self, buf):
            pass

    class FakeActive:
        def __init__(self, job, server):
            if getattr(job, "oom", False):
                raise MemoryError("CUDA out of memory (stand-in)")
            self.job, self.stream, self.it, self.done_event, self.phase_events = job, object(), 0, None, None
            self.admitted_with = len(server._active)

        def enqueue_iteration(self):
            self.it += 1

        def enqueue_results(self):
            left = [polls_until_done]

            def query():
                left[0] -= 1
                return left[0] <= 0
            self.done_event = SimpleNamespace(query=query)

        def collect(self):
            if getattr(self.job, "fail", False):
                self.job.error = RuntimeError("device status of job %d" % self.job.id)
            else:
                self.job.result = {"iterations": self.it}

    monkeypatch.setattr(engine, "require_device", lambda device=None: "cpu")
    monkeypatch.setattr(serving, "pinned_pool", lambda: Pool())
    monkeypatch.setattr(serving, "_Active", FakeActive)
    return serving.Server(device="cpu", max_slots=max_slots, hbm_bytes=1 << 40, poll_s=1e-4)


def test_scheduler_admits_in_order_and_collects_every_job(monkeypatch):
    """The scheduler loop with its device work stood in for: every job is
    admitted in arrival order, never more than max_slots at once, runs all its
    iterations and is collected (on the collector thread) with its times in
    order."""
    from treetime_gb300.serving import Job
    ti, g = _small_job_inputs()
    srv = _fake_server(monkeypatch, max_slots=3)
    jobs = [Job(ti, g, iterations=2 + (k % 3)) for k in range(20)]
    arrivals = np.linspace(0.0, 0.05, len(jobs))
    done, wall = srv.serve(jobs, arrivals)
    assert len(srv.done) == len(jobs) and srv.peak_active <= 3
    assert all(j.result == {"iterations": j.iterations} and j.error is None for j in jobs)
    admit_order = sorted(jobs, key=lambda j: j.t_admit)
    assert [j.id for j in admit_order] == [j.id for j in jobs]
    assert all(j.t_submit <= j.t_admit <= j.t_done for j in jobs)
    assert srv._staged_waiting == 0 and srv.pending() == 0


def test_scheduler_raises_a_device_error_after_the_other_jobs_finish(monkeypatch):
    """A job whose device status reports an error does not stop the others:
    run() raises it once every job has finished."""
    from treetime_gb300.serving import Job
    ti, g = _small_job_inputs()
    srv = _fake_server(monkeypatch, max_slots=2)
    jobs = [Job(ti, g) for _ in range(6)]
    jobs[1].fail = True
    with pytest.raises(RuntimeError, match="device status of job %d" % jobs[1].id):
        srv.serve(jobs, np.zeros(len(jobs)))
    assert len(srv.done) == len(jobs)
    assert all(j.result is not None for j in jobs if j is not jobs[1])


def test_submit_rejects_a_job_larger_than_the_whole_budget(monkeypatch):
    """A job whose device footprint exceeds the server's whole memory budget
    could never be admitted and would hold the head of the queue for good:
    submit raises MemoryError instead, and the queue stays usable."""
    from treetime_gb300.serving import Job
    ti, g = _small_job_inputs()
    srv = _fake_server(monkeypatch, max_slots=2)
    big = Job(ti, g)
    srv.hbm_bytes = big.footprint - 1
    with pytest.raises(MemoryError, match="budget"):
        srv.submit(big)
    assert srv.pending() == 0
    srv.hbm_bytes = 1 << 40
    jobs = [Job(ti, g) for _ in range(3)]
    srv.serve(jobs, np.zeros(3))
    assert all(j.result is not None for j in jobs)


def test_failed_admission_fails_only_that_job(monkeypatch):
    """A device allocation that fails while a job is admitted (stood in for by
    a MemoryError from the admission) makes that job fail alone: its slot is
    given back, the other jobs run to completion, and run() raises the error
    once they have finished."""
    from treetime_gb300.serving import Job
    ti, g = _small_job_inputs()
    srv = _fake_server(monkeypatch, max_slots=2)
    jobs = [Job(ti, g) for _ in range(6)]
    jobs[2].oom = True
    with pytest.raises(MemoryError, match="out of memory"):
        srv.serve(jobs, np.zeros(len(jobs)))
    assert len(srv.done) == len(jobs) and srv.pending() == 0
    assert jobs[2].result is None and isinstance(jobs[2].error, MemoryError)
    assert all(j.result is not None and j.error is None for j in jobs if j is not jobs[2])
