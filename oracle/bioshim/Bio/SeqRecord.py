"""Minimal Bio.SeqRecord stand-in (test-only)."""


class SeqRecord:
    def __init__(self, seq, id="<unknown id>", name="<unknown name>", description="", **kwargs):
        self.seq = seq
        self.id = id
        self.name = name
        self.description = description

    def __len__(self):
        return len(self.seq)

    def upper(self):
        """A copy with the sequence in upper case (Biopython's SeqRecord.upper)."""
        return SeqRecord(self.seq.upper(), id=self.id, name=self.name, description=self.description)
