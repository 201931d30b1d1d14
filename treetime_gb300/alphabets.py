"""Alphabets, ambiguity profiles and character-array helpers.

The alphabets and the IUPAC ambiguity tables are part of the data contract
with TreeTime (treetime/seq_utils.py:5-121): the same characters map to the
same state sets.  They are written here as state-set strings and expanded
into 0/1 profile rows.

Device-side, tip characters travel as raw bytes (uint8) and are expanded by a
256-row lookup table built from the profile map (``profile_lut``).
"""

import numpy as np

alphabet_synonyms = {
    "nuc": "nuc",
    "nucleotide": "nuc",
    "aa": "aa",
    "aminoacid": "aa",
    "nuc_nogap": "nuc_nogap",
    "nucleotide_nogap": "nuc_nogap",
    "aa_nogap": "aa_nogap",
    "aminoacid_nogap": "aa_nogap",
    "DNA": "nuc",
    "DNA_nogap": "nuc_nogap",
}

_AA20 = "ACDEFGHIKLMNPQRSTVWY"

alphabets = {
    "nuc": np.array(list("ACGT-")),
    "nuc_nogap": np.array(list("ACGT")),
    "aa": np.array(list(_AA20 + "*-")),
    "aa_nogap": np.array(list(_AA20)),
}

# IUPAC nucleotide codes as the set of bases each stands for.
_NUC_CODES = {
    "R": "AG", "Y": "CT", "S": "CG", "W": "AT", "K": "GT", "M": "AC",
    "D": "AGT", "H": "ACT", "B": "CGT", "V": "ACG",
}
# Amino-acid ambiguity codes.
_AA_CODES = {"B": "DN", "Z": "EQ"}


def _build_map(alphabet, codes, all_ones, extra=None):
    alphabet = list(alphabet)
    n = len(alphabet)
    index = {c: i for i, c in enumerate(alphabet)}
    pm = {}
    for c in alphabet:
        row = np.zeros(n, dtype=float)
        row[index[c]] = 1.0
        pm[c] = row
    for c in all_ones:
        pm[c] = np.ones(n, dtype=float)
    for c, states in codes.items():
        row = np.zeros(n, dtype=float)
        for s in states:
            row[index[s]] = 1.0
        pm[c] = row
    if extra:
        pm.update(extra)
    return pm


def _default_profile_maps():
    return {
        "nuc": _build_map("ACGT-", _NUC_CODES, "NX"),
        # without a gap state a gap carries no information: all-ones row
        "nuc_nogap": _build_map("ACGT", _NUC_CODES, "-NX"),
        "aa": _build_map(_AA20 + "*-", _AA_CODES, "X"),
        "aa_nogap": _build_map(_AA20, _AA_CODES, "X"),
    }


profile_maps = _default_profile_maps()


def fresh_profile_map(name):
    """A private copy of a named profile map (models extend their own copy)."""
    return {k: v.copy() for k, v in _default_profile_maps()[alphabet_synonyms[name]].items()}


def seq2array(seq, word_length=1, convert_upper=False, fill_overhangs=False, ambiguous="N"):
    """Character array of a sequence; with ``fill_overhangs`` the leading and
    trailing runs of '-' become ``ambiguous`` (an all-gap sequence becomes all
    ``ambiguous``).  Follows treetime/seq_utils.py:152-204."""
    if isinstance(seq, str):
        s = seq
    elif hasattr(seq, "seq"):
        s = str(seq.seq)
    elif isinstance(seq, np.ndarray):
        s = "".join(seq.astype("U").tolist())
    else:
        s = str(seq)
    if convert_upper:
        s = s.upper()
    if word_length != 1:
        raise ValueError("only word_length=1 is supported")
    arr = np.array(list(s))
    if fill_overhangs:
        non_gap = np.flatnonzero(arr != "-")
        if len(non_gap):
            arr[: non_gap[0]] = ambiguous
            arr[non_gap[-1] + 1:] = ambiguous
        else:
            arr[:] = ambiguous
    return arr


def guess_alphabet(seqs):
    """'nuc' when more than 90% of characters are in acgtACGT-N, else 'aa'
    (treetime/seq_utils.py:139-149)."""
    total = 0
    nuc = 0
    allowed = np.array(list("acgtACGT-N"))
    for s in seqs:
        total += len(s)
        nuc += int(np.isin(s, allowed).sum())
    return "nuc" if nuc > 0.9 * total else "aa"


def extend_profile(gtr, seqs, logger=None):
    """Characters present in the alignment but unknown to the model become
    missing data: an all-ones profile row (treetime/seq_utils.py:126-136)."""
    chars = set()
    for s in seqs:
        chars.update(np.unique(s).tolist())
    for c in sorted(chars):
        if c not in gtr.profile_map:
            gtr.profile_map[c] = np.ones(gtr.n_states)
            if logger:
                logger("WARNING: character %s is unknown. Treating it as missing information" % c, 1, warn=True)


def chars_to_codes(arr):
    """numpy '<U1' character array -> uint8 byte codes (ASCII)."""
    arr = np.asarray(arr)
    if arr.dtype.kind == "u" or arr.dtype == np.uint8:
        return arr.astype(np.uint8)
    return np.frombuffer(np.ascontiguousarray(arr.astype("S1")).tobytes(), dtype=np.uint8).reshape(arr.shape)


def codes_to_chars(codes):
    codes = np.ascontiguousarray(codes, dtype=np.uint8)
    return np.frombuffer(codes.tobytes(), dtype="S1").reshape(codes.shape).astype("U1")


# Code 0 never occurs in text; it marks a tip without a sequence (all-ones row).
MISSING_CODE = 0


def profile_lut(profile_map, n_states):
    """256 x n_states float64 table: byte code -> profile row.  Code 0 is the
    all-ones row used for tips absent from the alignment."""
    lut = np.zeros((256, n_states), dtype=np.float64)
    lut[MISSING_CODE] = 1.0
    for c, row in profile_map.items():
        if isinstance(c, str) and len(c) == 1 and ord(c) < 256:
            lut[ord(c)] = row
    return lut


def state_lut(alphabet):
    """256-entry table byte code -> state index, 255 for characters that are
    not states of the alphabet."""
    lut = np.full(256, 255, dtype=np.uint8)
    for i, c in enumerate(alphabet):
        lut[ord(str(c))] = i
    return lut
