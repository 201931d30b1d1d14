"""Minimal Bio.AlignIO stand-in (test-only): FASTA reading."""

from .Align import MultipleSeqAlignment
from .Seq import Seq
from .SeqRecord import SeqRecord


def _read_fasta(text):
    records = []
    name, chunks = None, []
    for line in text.splitlines():
        line = line.strip()
        if not line:
            continue
        if line.startswith(">"):
            if name is not None:
                records.append((name, "".join(chunks)))
            name, chunks = line[1:].split()[0] if line[1:].split() else "", []
        else:
            chunks.append(line)
    if name is not None:
        records.append((name, "".join(chunks)))
    return [SeqRecord(Seq(s), id=n, name=n, description=n) for n, s in records]


def read(handle, format):
    if format != "fasta":
        raise ValueError("bioshim AlignIO.read supports fasta only")
    if hasattr(handle, "read"):
        text = handle.read()
    else:
        with open(handle) as fh:
            text = fh.read()
    return MultipleSeqAlignment(_read_fasta(text))


def write(aln, handle, format):
    text = "".join(">%s\n%s\n" % (r.id, str(r.seq)) for r in aln)
    if hasattr(handle, "write"):
        handle.write(text)
    else:
        with open(handle, "w") as fh:
            fh.write(text)
