"""Alignment ingest and column-pattern compression.

``SequenceData`` keeps the alignment as a uint8 byte matrix (tips × sites)
and compresses it into alignment patterns with the exact semantics of
treetime/sequence_data.py:325-464:

  * a column with exactly two letters, one of them the ambiguous character,
    is rewritten to the other letter first;
  * only constant columns merge: a column with two or more letters gets a
    private pattern (TreeTime keys it by '<column>_<position>');
  * patterns are numbered by first occurrence, ``multiplicity`` counts the
    merged columns, and the two maps full<->compressed are kept;
  * ``compress=False`` is the identity.

The compression is vectorised over columns (numpy on the host, or the
``tt_compress_columns`` CUDA entry point for large alignments); both give
bit-identical patterns, multiplicities and maps.
"""

import os
from collections import OrderedDict

import numpy as np

from . import config as ttconf
from .alphabets import seq2array, guess_alphabet, chars_to_codes, codes_to_chars
from .errors import MissingDataError


def read_fasta(path_or_handle):
    if hasattr(path_or_handle, "read"):
        text = path_or_handle.read()
    else:
        with open(path_or_handle) as fh:
            text = fh.read()
    out = OrderedDict()
    name, chunks = None, []
    for line in text.splitlines():
        line = line.strip()
        if not line:
            continue
        if line.startswith(">"):
            if name is not None:
                out[name] = "".join(chunks)
            parts = line[1:].split()
            name, chunks = (parts[0] if parts else ""), []
        else:
            chunks.append(line)
    if name is not None:
        out[name] = "".join(chunks)
    return out


def _record_name(rec):
    """Name of an alignment record as TreeTime picks it
    (treetime/sequence_data.py:161-173)."""
    rid, rname = getattr(rec, "id", None), getattr(rec, "name", None)
    if rid == rname:
        return rid
    if rid is not None and "<unknown" in str(rid):
        return rname
    if rname is not None and "<unknown" in str(rname):
        return rid
    return rname


def compress_codes(codes, ambiguous_code, compress=True):
    """Column-pattern compression of a tips × sites uint8 matrix.

    Returns (pattern_codes [tips × P] uint8, multiplicity [P] float64,
    full_to_compressed [L] int64, compressed_to_full dict p -> positions).
    """
    n, L = codes.shape
    if not compress:
        return (codes.copy(), np.ones(L, dtype=float), np.arange(L),
                {p: np.array([p]) for p in range(L)})
    if n == 0:
        raise MissingDataError("empty alignment")
    amb = -1 if ambiguous_code is None else int(ambiguous_code)
    c16 = codes.astype(np.int16)
    is_amb = c16 == amb
    big, small = np.int16(1000), np.int16(-1)
    non_amb_min = np.where(is_amb, big, c16).min(axis=0)
    non_amb_max = np.where(is_amb, small, c16).max(axis=0)
    any_non_amb = non_amb_max >= 0
    any_amb = is_amb.any(axis=0)
    all_same = codes.min(axis=0) == codes.max(axis=0)
    # {X, ambiguous} columns collapse to X
    amb_fix = any_non_amb & any_amb & (non_amb_min == non_amb_max)
    constant = all_same | amb_fix
    fixed = codes
    if amb_fix.any():
        fixed = codes.copy()
        cols = np.flatnonzero(amb_fix)
        sub = fixed[:, cols]
        sub[is_amb[:, cols]] = np.broadcast_to(non_amb_min[cols].astype(np.uint8), sub.shape)[is_amb[:, cols]]
        fixed[:, cols] = sub
    letter = np.where(amb_fix, non_amb_min, codes[0].astype(np.int16)).astype(np.int64)
    key = np.where(constant, letter, 256 + np.arange(L, dtype=np.int64))
    uniq, first, inverse, counts = np.unique(key, return_index=True, return_inverse=True, return_counts=True)
    order = np.argsort(first, kind="stable")          # pattern number by first occurrence
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    full_to_compressed = rank[inverse].astype(np.int64)
    multiplicity = counts[order].astype(float)
    pattern_codes = np.ascontiguousarray(fixed[:, first[order]])
    pos_sorted = np.argsort(full_to_compressed, kind="stable")
    bounds = np.concatenate(([0], np.cumsum(counts[order])))
    c2f = {p: pos_sorted[bounds[p]:bounds[p + 1]].astype(int) for p in range(len(order))}
    return pattern_codes, multiplicity, full_to_compressed, c2f


class _LazyCharRows(OrderedDict):
    """name -> character array of the alignment, built from the byte matrix on
    first access of each row."""

    def __init__(self, names, codes):
        super().__init__((k, None) for k in names)
        self._codes = codes
        self._row = {k: i for i, k in enumerate(names)}

    def __getitem__(self, k):
        v = super().__getitem__(k)
        if v is None:
            v = codes_to_chars(self._codes[self._row[k]])
            super().__setitem__(k, v)
        return v

    def values(self):
        return [self[k] for k in self.keys()]

    def items(self):
        return [(k, self[k]) for k in self.keys()]

    def get(self, k, default=None):
        return self[k] if k in self else default


class SequenceData:
    """Alignment container with TreeTime's SequenceData interface for dense
    alignments (dict name -> sequence, an iterable of records with id/name/seq,
    or a FASTA file)."""

    def __init__(self, aln, ref=None, logger=None, convert_upper=True, sequence_length=None, compress=True,
                 word_length=1, sequence_type=None, fill_overhangs=True, seq_multiplicity=None, ambiguous=None,
                 **kwargs):
        self.logger = logger if logger else (lambda *a, **k: None)
        self.convert_upper = convert_upper
        self.compress = compress
        self.word_length = word_length
        self.fill_overhangs = fill_overhangs
        self.ambiguous = ambiguous
        self.sequence_type = sequence_type
        self.seq_multiplicity = seq_multiplicity or {}
        self.additional_constant_sites = kwargs.get("additional_constant_sites", 0)
        self.is_sparse = False
        self.ref = ref
        self._full_length = int(sequence_length) if sequence_length else None
        self._aln = None
        self._compressed_alignment = None
        self.aln = aln

    # ------------------------------------------------------------ ingest
    @property
    def aln(self):
        return self._aln

    @aln.setter
    def aln(self, in_aln):
        self._aln = None
        self._compressed_alignment = None
        if in_aln is None:
            return
        if isinstance(in_aln, str) and os.path.isfile(in_aln):
            if in_aln.lower().endswith((".vcf", ".vcf.gz")) and self.ref is not None:
                from .vcf import read_vcf
                in_aln = read_vcf(in_aln)["sequences"]
            else:
                in_aln = read_fasta(in_aln)
        if isinstance(in_aln, dict) and in_aln and all(isinstance(v, dict) for v in in_aln.values()):
            return self._set_sparse(in_aln)
        if isinstance(in_aln, dict):
            raw = [(k, v) for k, v in in_aln.items()]
        else:
            try:
                raw = [(_record_name(r), r) for r in in_aln]
            except TypeError:
                raise MissingDataError("SequenceData: loading alignment failed... " + str(in_aln))
        if not raw:
            raise MissingDataError("SequenceData: loading alignment failed... empty alignment")
        rows = [self._to_codes(v) for _, v in raw]
        sample = np.concatenate([r[:20000] for r in rows[:50]])
        nucish = np.isin(sample, np.frombuffer(b"acgtACGT-N", dtype=np.uint8)).sum()
        self.likely_alphabet = "nuc" if nucish > 0.9 * len(sample) else "aa"
        if self.ambiguous is None:
            self.ambiguous = "N" if self.likely_alphabet == "nuc" else "X"
        lengths = {len(r) for r in rows}
        if len(lengths) != 1:
            raise MissingDataError("SequenceData: sequences have different lengths")
        L = lengths.pop()
        if self.fill_overhangs:
            amb = ord(self.ambiguous)
            gap = ord("-")
            for r in rows:
                ng = np.flatnonzero(r != gap)
                if len(ng):
                    r[: ng[0]] = amb
                    r[ng[-1] + 1:] = amb
                else:
                    r[:] = amb
        if self._full_length:
            if self._full_length < L:
                raise AttributeError("SequenceData.aln: specified sequence length is smaller than alignment length!")
            if self._full_length > L:
                self.logger("SequenceData.aln: specified sequence length doesn't match alignment length. Treating "
                            "difference as constant sites.", 2, warn=True)
            self.additional_constant_sites = max(0, self._full_length - L)
        else:
            self._full_length = L
        self.sequence_names = [k for k, _ in raw]
        self.codes = np.stack(rows) if rows else np.zeros((0, L), np.uint8)
        self._aln = _LazyCharRows(self.sequence_names, self.codes)
        self.make_compressed_alignment()

    def _set_sparse(self, in_aln):
        """A sparse alignment {name: {position: character}} of differences from
        the reference `ref` (e.g. from a VCF file), compressed as TreeTime does
        (treetime/sequence_data.py:325-464 with
        treetime/vcf_utils.py:653-749): positions that differ in no sequence,
        or are constant up to the ambiguous character, or carry one non-reference
        state in every sequence, become constant patterns, one per state in
        sorted order; the other positions are taken in the order in which they
        first appear in the sequences' dictionaries, a column with one state
        after replacing the ambiguous character joins that state's constant
        pattern, any other column gets a pattern of its own."""
        if self.ref is None:
            raise MissingDataError("SequenceData: a sparse alignment needs a reference sequence")
        if not self.compress:
            raise NotImplementedError("sparse alignments are always compressed")
        ref = self.ref
        if isinstance(ref, str) and os.path.isfile(ref):
            recs = read_fasta(ref)
            if len(recs) != 1:
                raise TypeError("SequenceData.ref: reference sequence file %s could not be parsed" % ref)
            ref = next(iter(recs.values()))
        if hasattr(ref, "seq"):
            ref = str(ref.seq)
        ref = ref if isinstance(ref, str) else "".join(np.asarray(ref).astype("U").tolist())
        ref = ref.upper() if self.convert_upper else ref
        ref_codes = np.frombuffer(ref.encode("latin-1"), dtype=np.uint8).copy()
        self.ref = ref_codes.view("S1").astype("U1")  # the reference as a character array, as TreeTime keeps it
        sample = ref_codes[:20000]
        nucish = np.isin(sample, np.frombuffer(b"acgtACGT-N", dtype=np.uint8)).sum()
        self.likely_alphabet = "nuc" if nucish > 0.9 * len(sample) else "aa"
        if self.ambiguous is None:
            self.ambiguous = "N" if self.likely_alphabet == "nuc" else "X"
        amb = ord(self.ambiguous)
        L = len(ref_codes)
        if self._full_length and self._full_length != L:
            self.logger("SequenceData.aln: specified sequence length doesn't match reference length, ignoring "
                        "sequence length.", 1, warn=True)
        self._full_length = L
        self.is_sparse = True
        self.codes = None
        self.sequence_names = list(in_aln.keys())
        names = self.sequence_names
        nseq = len(names)
        conv = (lambda c: c.upper()) if self.convert_upper else (lambda c: c)
        seqs = {k: {int(p): ord(conv(str(c))) for p, c in v.items()} for k, v in in_aln.items()}
        # positions with at least one difference, in order of first appearance
        inv = {}
        for k in names:
            for p, c in seqs[k].items():
                inv.setdefault(p, []).append(c)
        ref_mod = ref_codes.copy()
        variable, nonref_pos, nonref_allele, up_to_amb = [], [], [], []
        for p, bs in inv.items():
            bases = sorted(set(bs))
            if len(bs) == nseq:
                if len(bases) == 1 or (len(bases) <= 2 and amb in bases):
                    nonref_pos.append(p)
                    nonref_allele.append(bases[0] if len(bases) == 1 else [x for x in bases if x != amb][0])
                    if amb in bases:
                        up_to_amb.append(p)
                else:
                    variable.append(p)
            elif len(bases) == 1 and bases[0] == amb:
                up_to_amb.append(p)
            else:
                variable.append(p)
        if nonref_pos:
            ref_mod[np.asarray(nonref_pos)] = np.asarray(nonref_allele, dtype=np.uint8)
        states = np.unique(ref_mod)
        if variable:
            ref_mod[np.asarray(variable)] = ord(".")
        columns, patterns, positions = [], {}, []
        for base in states:
            if base == amb:
                continue
            pos = np.flatnonzero(ref_mod == base)
            if len(pos):
                patterns[bytes([base]) * nseq] = len(columns)
                columns.append(np.full(nseq, base, dtype=np.uint8))
                positions.append(list(pos))
        for p in variable:
            col = np.array([seqs[k].get(p, ref_codes[p]) for k in names], dtype=np.uint8)
            letters = np.unique(col)
            if len(letters) == 2 and amb in letters:
                col[col == amb] = letters[letters != amb][0]
                letters = letters[letters != amb]
            key = col.tobytes()
            if len(letters) > 1:
                key += b"_%d" % p
            if key not in patterns:
                patterns[key] = len(columns)
                columns.append(col)
                positions.append([p])
            else:
                positions[patterns[key]].append(p)
        mult = np.array([len(x) for x in positions], dtype=float)
        f2c = np.zeros(L, dtype=int)
        c2f = {}
        for i, pos in enumerate(positions):
            f2c[np.asarray(pos, dtype=int)] = i
            c2f[i] = np.asarray(pos, dtype=int)
        self.inferred_const_sites = up_to_amb
        self.nonref_positions = np.sort(np.asarray(list(inv.keys()), dtype=int))
        self._aln = in_aln
        self.compressed_codes = np.stack(columns, axis=1) if columns else np.zeros((nseq, 0), np.uint8)
        self._multiplicity = mult
        self.full_to_compressed_sequence_map = f2c
        self.compressed_to_full_sequence_map = c2f
        self._compressed_length = len(mult)
        self._compressed_alignment = None
        self.name_to_row = {k: i for i, k in enumerate(names)}

    def _to_codes(self, v):
        if isinstance(v, np.ndarray) and v.dtype == np.uint8:
            return v.copy()
        if isinstance(v, np.ndarray):
            v = "".join(v.astype("U").tolist())
        elif hasattr(v, "seq"):
            v = str(v.seq)
        elif not isinstance(v, str):
            v = str(v)
        if self.convert_upper:
            v = v.upper()
        return np.frombuffer(v.encode("latin-1"), dtype=np.uint8).copy()

    @property
    def full_length(self):
        return self._full_length

    @property
    def compressed_length(self):
        return self._compressed_length

    def make_compressed_alignment(self, device=None):
        if self.is_sparse:
            return ttconf.SUCCESS
        amb = ord(self.ambiguous) if self.ambiguous else None
        if device is not None and self.compress:
            from . import engine
            pc, mult, f2c, c2f = engine.compress_columns(self.codes, amb, device)
        else:
            pc, mult, f2c, c2f = compress_codes(self.codes, amb, self.compress)
        if self.additional_constant_sites and self.compress:
            pc, mult, f2c, c2f = self._add_constant_sites(pc, mult, f2c, c2f)
        self.compressed_codes = pc
        self._multiplicity = mult
        self.full_to_compressed_sequence_map = f2c
        self.compressed_to_full_sequence_map = c2f
        self._compressed_length = len(mult)
        self._compressed_alignment = None
        self.name_to_row = {k: i for i, k in enumerate(self.sequence_names)}
        return ttconf.SUCCESS

    def _add_constant_sites(self, pc, mult, f2c, c2f):
        """Constant columns for the sites beyond the alignment
        (treetime/sequence_data.py:418-441): shared among the alphabet's states
        (without gap and ambiguous character) in proportion to their counts in
        the alignment, rounded, the last state taking the remainder; each
        state's columns join its constant pattern or start one, at positions
        after the alignment."""
        from .alphabets import alphabets
        extra = int(self.additional_constant_sites)
        states = [c for c in alphabets[self.likely_alphabet + "_nogap"].tolist() if c not in (self.ambiguous, "-")]
        counts = [(c, int(np.sum(self.codes == ord(c)))) for c in states]
        total = np.sum([n for _, n in counts])
        shares = [(c, int(np.round(extra * n / total))) for c, n in counts]
        left = extra
        pi = self.codes.shape[1]
        nseq = pc.shape[0]
        cols = [pc[:, i] for i in range(pc.shape[1])]
        mult = list(mult)
        f2c = np.concatenate([f2c, np.zeros(extra, dtype=f2c.dtype)])
        const = {}
        for i, col in enumerate(cols):
            if (col == col[0]).all() and col[0] not in const:
                const[int(col[0])] = i
        c2f = dict(c2f)
        for c, n in shares:
            if c == shares[-1][0]:
                n = left
            if n:
                code = ord(c)
                if code in const:
                    p = const[code]
                    mult[p] += n
                    c2f[p] = np.concatenate([c2f[p], np.arange(pi, pi + n)])
                else:
                    p = len(cols)
                    cols.append(np.full(nseq, code, dtype=np.uint8))
                    mult.append(float(n))
                    const[code] = p
                    c2f[p] = np.arange(pi, pi + n)
                f2c[pi:pi + n] = p
                pi += n
                left -= n
        return np.ascontiguousarray(np.stack(cols, axis=1)), np.asarray(mult, dtype=float), f2c, c2f

    @property
    def compressed_alignment(self):
        if self._compressed_alignment is None:
            if not self.compress:
                self._compressed_alignment = self._aln
            else:
                chars = codes_to_chars(self.compressed_codes)
                self._compressed_alignment = OrderedDict(
                    (k, chars[i]) for i, k in enumerate(self.sequence_names))
        return self._compressed_alignment

    def multiplicity(self, mask=None):
        if mask is None:
            return self._multiplicity
        return self._multiplicity * mask

    # ------------------------------------------------------ sequence maps
    def compressed_to_full_sequence(self, sequence, include_additional_constant_sites=False, as_string=False):
        """treetime/sequence_data.py:513-539: the sites beyond the alignment only
        when asked for."""
        L = self.full_length if include_additional_constant_sites else \
            self.full_length - int(self.additional_constant_sites or 0)
        tmp = sequence[self.full_to_compressed_sequence_map[:L]]
        if as_string:
            return "".join(tmp.astype("U"))
        return tmp

    def differences(self, seq1, seq2, seq1_compressed=True, seq2_compressed=True, mask=None):
        """Sorted (anc, pos, der) list between two sequences, expanded to full
        length (treetime/sequence_data.py:541-568, dense alignments)."""
        if seq1_compressed:
            seq1 = self.compressed_to_full_sequence(seq1)
        if seq2_compressed:
            seq2 = self.compressed_to_full_sequence(seq2)
        if mask is None:
            pos = np.flatnonzero(seq1 != seq2)
        else:
            pos = np.flatnonzero((seq1 != seq2) & (mask > 0))
        return [(seq1[p], int(p), seq2[p]) for p in pos]
