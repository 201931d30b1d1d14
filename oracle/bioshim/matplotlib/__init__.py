"""Empty matplotlib stand-in (test-only): TreeTime imports plotting helpers at
module load; the ancestral-reconstruction path never plots."""
