"""Admission policy of the serving loop (host logic, no GPU): jobs are
admitted in arrival order while a slot is free and their device footprint
fits; a job that does not fit holds the head of the queue."""

from types import SimpleNamespace

import numpy as np

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
    (a, b), _ = synth.forest_c3(n_trees=2, seed=1, n_range=(20, 200), L_range=(100, 1000))
    small, big = sorted((a, b), key=lambda ti: ti.layout.n_nodes * ti.n_patterns)
    assert footprint(small, 4, "marginal") < footprint(big, 4, "marginal")
    assert footprint(big, 4, "marginal") < footprint(big, 4, "optimize")
    rows = big.layout.n_int * big.n_patterns * 4 * 4
    assert footprint(big, 4, "marginal") >= 2 * rows
