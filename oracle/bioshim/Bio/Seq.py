"""Minimal Bio.Seq stand-in (test-only)."""


class Seq:
    def __init__(self, data):
        self._data = str(data)

    def __str__(self):
        return self._data

    def __len__(self):
        return len(self._data)

    def __iter__(self):
        return iter(self._data)

    def __getitem__(self, i):
        return self._data[i]

    def upper(self):
        return Seq(self._data.upper())
