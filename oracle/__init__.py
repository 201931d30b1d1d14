"""CPU oracle for the TreeTime Felsenstein-pruning hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` may import this package, and only as the
checker or the timed CPU reference -- never as part of the product path.

``oracle.anc`` restates TreeTime's numpy algorithms (each function cites the
file:line it follows) on plain numpy arrays.  It is pinned against golden
vectors produced by running the unmodified TreeTime package
(``tests/golden/make_golden.py``, through the test-only ``oracle/bioshim``
stand-in for Biopython).
"""
