"""Test-only stand-in for the few Biopython types that TreeTime's ancestral
reconstruction touches.  It exists so that the unmodified TreeTime package can
be imported in a container without Biopython, to generate golden vectors.

Written from Biopython's documented behaviour (Bio.Phylo traversal orders,
Tree.ladderize, SeqRecord/MultipleSeqAlignment attributes), not from its
source.  Never imported by the product package.
"""

__version__ = "1.85-shim"
