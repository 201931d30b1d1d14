"""GPU: pattern compression with the column classification on the device
(tt_compress_columns) gives exactly the host compression (which the CPU tests
pin to TreeTime's make_compressed_alignment): patterns, multiplicities and the
full -> compressed map, with gaps, ambiguity codes, {X, ambiguous} columns and
constant columns."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed,n,L", [(0, 37, 2000), (1, 37, 2003), (2, 5, 1001), (3, 3, 1000), (4, 211, 4096)])
def test_compress_columns_equals_host(seed, n, L):
    """Row lengths that are (tiled kernel) and are not (column kernel)
    multiples of 4, fewer rows than the tiled kernel's warps, ragged tiles."""
    from treetime_gb300 import engine
    from treetime_gb300.seqdata import compress_codes
    rng = np.random.default_rng(seed)
    alpha = np.frombuffer(b"ACGT", dtype=np.uint8)
    root = rng.integers(4, size=L)
    codes = alpha[np.where(rng.random((n, L)) < 0.08, rng.integers(4, size=(n, L)), root[None, :])]
    codes[rng.random((n, L)) < 0.03] = ord("N")            # ambiguous
    codes[rng.random((n, L)) < 0.02] = ord("-")            # gaps
    codes[:, :50] = alpha[root[:50]]                       # constant columns
    codes[rng.integers(n, size=40), rng.integers(50, size=40)] = ord("N")  # {X, ambiguous} columns
    codes[:, 60] = ord("N")                                # an all-ambiguous column
    h = compress_codes(codes, ord("N"))
    d = engine.compress_columns(codes, ord("N"))
    np.testing.assert_array_equal(d[0], h[0])
    np.testing.assert_array_equal(d[1], h[1])
    np.testing.assert_array_equal(d[2], h[2])
