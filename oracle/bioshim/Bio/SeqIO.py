"""Minimal Bio.SeqIO stand-in (test-only)."""

from .AlignIO import _read_fasta


def read(handle, format):
    if format != "fasta":
        raise ValueError("bioshim SeqIO.read supports fasta only")
    if hasattr(handle, "read"):
        text = handle.read()
    else:
        with open(handle) as fh:
            text = fh.read()
    recs = _read_fasta(text)
    if len(recs) != 1:
        raise ValueError("expected one record")
    return recs[0]


def parse(handle, format):
    if hasattr(handle, "read"):
        text = handle.read()
    else:
        with open(handle) as fh:
            text = fh.read()
    return iter(_read_fasta(text))
