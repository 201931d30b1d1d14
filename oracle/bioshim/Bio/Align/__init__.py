"""Minimal Bio.Align stand-in (test-only)."""


class MultipleSeqAlignment:
    def __init__(self, records):
        self._records = list(records)

    def __iter__(self):
        return iter(self._records)

    def __len__(self):
        return len(self._records)

    def __getitem__(self, i):
        return self._records[i]

    def get_alignment_length(self):
        return max((len(r.seq) for r in self._records), default=0)
