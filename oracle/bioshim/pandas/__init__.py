"""Empty pandas stand-in (test-only): TreeTime imports pandas at module load for
date parsing, which the ancestral-reconstruction path never calls."""
