"""Numerical floors and ceilings used by the reconstruction and branch-length
code.  The values are part of the numerical contract with TreeTime
(treetime/config.py:3-36) and must not change."""

BIG_NUMBER = 1e10
TINY_NUMBER = 1e-12
SUPERTINY_NUMBER = 1e-24
MIN_LOG = -1e8
MIN_BRANCH_LENGTH = 1e-3  # fraction of one mutation used as lower cut-off for branch lengths
MAX_BRANCH_LENGTH = 4.0
BRANCH_GRID_SIZE = 125  # grid points of a branch-length interpolator
VERBOSE = 3
SUCCESS = "success"
ERROR = "error"
