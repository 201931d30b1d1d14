"""Autotuner for the FP32 marginal kernel's launch shape.

The best shape depends on the workload: the CTA size and residency (1024
threads, one CTA per SM; 512 threads, two CTAs per SM; 512 threads, one CTA
per SM with two nodes per group at a time) and how many pattern ranges the
forest is cut into per SM (one wide range per SM, or two narrower ones).  ``tune`` times every candidate on the actual forest
with CUDA events and returns the fastest; results are cached in memory and in
a JSON file keyed by a coarse workload signature (alphabet size, number of
trees, node and pattern counts rounded to powers of two).
"""

import json
import math
import os
import statistics

from . import engine

CANDIDATES = [(threads, ctas, rps) for threads, ctas in ((1024, 1), (512, 2), (512, 1)) for rps in (1, 2)]
_CACHE = {}
CACHE_PATH = os.environ.get("TREETIME_GB300_TUNE_CACHE",
                            os.path.join(os.path.expanduser("~"), ".cache", "treetime_gb300", "autotune.json"))


def signature(inputs, q):
    nodes = sum(ti.layout.n_nodes for ti in inputs)
    pats = sum(ti.n_patterns for ti in inputs)
    b = lambda x: int(round(math.log2(max(1, x))))
    return "q%d_t%d_n%d_p%d" % (q, b(len(inputs)), b(nodes), b(pats))


def _load_file():
    try:
        with open(CACHE_PATH) as fh:
            return json.load(fh)
    except Exception:
        return {}


def _save_file(d):
    try:
        os.makedirs(os.path.dirname(CACHE_PATH), exist_ok=True)
        with open(CACHE_PATH, "w") as fh:
            json.dump(d, fh, indent=1, sort_keys=True)
    except Exception:
        pass


def tune(inputs, q, model, device=None, candidates=None, reps=7, use_cache=True):
    """Fastest (threads, ctas_per_sm, ranges_per_sm) for this forest and the
    table of median times (ms) of all candidates."""
    key = signature(inputs, q)
    if use_cache:
        if key in _CACHE:
            return _CACHE[key]
        disk = _load_file()
        if key in disk:
            _CACHE[key] = (tuple(disk[key]["best"]), disk[key]["table"])
            return _CACHE[key]
    t = engine.torch()
    cands = candidates or CANDIDATES
    if q != 4:
        cands = [c for c in cands if c[:2] == (512, 1)]
    table = {}
    for threads, ctas, rps in cands:
        try:
            f = engine.Forest(inputs, q, device=device, threads=threads, ctas_per_sm=ctas, ranges_per_sm=rps)
            bufs = engine.Buffers(f)
            for _ in range(2):
                engine.marginal(f, model, bufs, precision="f32", sync=False)
            t.cuda.synchronize()
            times = []
            for _ in range(reps):
                a, b = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
                a.record()
                engine.marginal(f, model, bufs, precision="f32", sync=False)
                b.record()
                b.synchronize()
                times.append(a.elapsed_time(b))
            table["%d/%d/%d" % (threads, ctas, rps)] = statistics.median(times)
        except Exception as e:  # a shape that cannot launch (e.g. too much shared memory) is skipped
            table["%d/%d/%d" % (threads, ctas, rps)] = None
    ok = {k: v for k, v in table.items() if v is not None}
    best = tuple(int(x) for x in min(ok, key=ok.get).split("/"))
    _CACHE[key] = (best, table)
    if use_cache:
        disk = _load_file()
        disk[key] = {"best": list(best), "table": table}
        _save_file(disk)
    return best, table
