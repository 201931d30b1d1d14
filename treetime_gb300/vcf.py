"""VCF input: sparse alignments as differences from a reference sequence.

``read_vcf`` follows TreeTime's reader (treetime/vcf_utils.py:10-362): one
chromosome, genotype (GT) calls only, VCF positions converted to 0-based.
Per sample it records the characters that differ from the reference:

  * a homozygous call (or a polyploid call whose alleles agree) applies the
    ALT allele: a substitution; a deletion ('-' at the deleted reference
    positions); an insertion (kept in ``insertions``, with a substitution at
    its first base when that differs from the reference); REF and ALT both
    longer than one base with ALT the longer one: substitutions where they
    differ and the rest of ALT as an insertion at the last REF base.  ALT
    '*' or '.' means N over the REF length.  Invalid ALT strings (outside
    [ACGTN]+, '*', '.') are skipped with a warning;
  * a haploid no-call ('.') writes N over the REF length;
  * a heterozygous or partial no-call writes N: at a single-base site (a
    heterozygous insertion, or a no-call with multi-base ALTs, is ignored),
    or, at a deletion site, N over the deleted part after the substitutions
    of the first allele.

The result is the dict TreeTime returns: ``reference`` (upper-case FASTA
string or None), ``sequences`` {sample: {position: character}},
``insertions`` {sample: {position: bases}}, ``positions`` (sorted positions
with a difference) and ``metadata`` (the '##' lines, chromosome, ploidy).
A ``SequenceData`` (and so a ``TreeAnc``) built from ``sequences`` and the
reference compresses the sparse alignment as TreeTime does.
"""

import gzip
import re

from .errors import TreeTimeError

_ALT_CHARS = re.compile(r"^([ACGTNacgtn]+|\*|\.)$")


def _valid_alt(alt):
    if _ALT_CHARS.match(alt):
        return alt.upper()
    print(f"WARNING: Encountered invalid allele base(s) {alt!r}. Skipping...")
    return None


def _homozygous(snps, ins, pos, ref, alt):
    if alt in ("*", "."):
        alt = "N" * len(ref)
    if len(ref) > 1 and len(alt) > len(ref):
        # insertion where there are also deletions / substitutions: compare base by base; the
        # rest of ALT from the last REF base on is the insertion
        for i in range(len(ref)):
            if ref[i] != alt[i]:
                snps[pos + i] = alt[i]
            if i + 1 >= len(ref):
                ins[pos + i] = alt[i:]
    elif len(ref) > 1:  # deletion (and possible substitutions before it)
        for i in range(len(ref)):
            if i + 1 > len(alt):
                snps[pos + i] = "-"
            elif ref[i] != alt[i]:
                snps[pos + i] = alt[i]
    elif len(alt) > 1:  # insertion after a single reference base
        ins[pos] = alt
        if ref[0] != alt[0]:
            snps[pos] = alt[0]
    else:
        snps[pos] = alt


def _heterozygous(gt, snps, pos, ref, alts):
    if len(ref) > 1:  # deletion site: the deleted part becomes N
        if gt[0] in ("0", "."):
            alt = str(alts[int(gt[2]) - 1]) if gt[0] == "0" else ref[0]
            for i in range(len(ref)):
                if i + 1 > len(alt):
                    snps[pos + i] = "N"
                elif ref[i] != alt[i]:
                    snps[pos + i] = alt[i] if alt[i] != "." else "N"
    elif gt[0] == "0":
        if len(str(alts[int(gt[2]) - 1])) == 1:  # heterozygous substitution (an insertion is ignored)
            snps[pos] = "N"
    elif len(alts) == len("".join(alts)):  # no-call with single-base alleles only
        snps[pos] = "N"


def read_vcf(vcf_file, ref_file=None):
    """Parse a VCF (optionally gzipped) mapped to the reference in `ref_file`
    (FASTA); see the module docstring for the result."""
    sequences, insertions = {}, {}
    metadata = {"meta_lines": [], "chrom": None, "ploidy": None}
    opener = gzip.open if vcf_file.endswith((".gz", ".GZ")) else open
    block = "meta-information"
    samples = None
    mandatory = ["CHROM", "POS", "ID", "REF", "ALT", "QUAL", "FILTER", "INFO", "FORMAT"]
    with opener(vcf_file, mode="rt") as fh:
        for line in fh:
            if line.startswith("##"):
                if block != "meta-information":
                    raise TreeTimeError(f"Malformed VCF file {vcf_file!r} - all the meta-information (lines "
                                        "starting with ##) must appear at the top of the file.")
                metadata["meta_lines"].append(line.strip())
                continue
            if line.startswith("#"):
                start = "#" + "\t".join(mandatory)
                if not line.startswith(start):
                    raise TreeTimeError(f"Malformed VCF file {vcf_file!r} - the header line must start with {start}")
                if block != "meta-information":
                    raise TreeTimeError(f"Malformed VCF file {vcf_file!r} - the header must immediately follow the "
                                        "meta-information lines")
                block = "header"
                samples = [x.strip() for x in line.strip().split("\t")[9:]]
                for s in samples:
                    sequences[s] = {}
                continue
            if block not in ("header", "data-lines"):
                raise TreeTimeError(f"Malformed VCF file {vcf_file!r} - the data lines must follow the header line")
            block = "data-lines"
            fields = line.strip()
            if not fields:
                continue
            dat = fields.split("\t")
            chrom = str(dat[0])
            if metadata["chrom"] is None:
                metadata["chrom"] = chrom
            elif metadata["chrom"] != chrom:
                raise TreeTimeError(f"The VCF file {vcf_file!r} contains multiple chromosomes. TreeTime can not yet "
                                    "handle this.")
            pos = int(dat[1]) - 1
            ref = dat[3]
            alts = dat[4].split(",")
            calls = dat[9:]
            if len(calls) != len(samples):
                raise TreeTimeError(f"Malformed VCF file {vcf_file!r} - the data lines have different number of calls "
                                    "than the number of samples defined in the header")
            if not dat[8].startswith("GT"):
                continue
            for name, call in zip(samples, calls):
                gt = call.split(":")[0]
                parts = gt.split("|") if "|" in gt else gt.split("/")
                if metadata["ploidy"] is None:
                    metadata["ploidy"] = len(parts)
                elif metadata["ploidy"] != len(parts):
                    raise TreeTimeError(f"The VCF file {vcf_file!r} had genotype calls of ploidy "
                                        f"{metadata['ploidy']} but sample {name!r} has a genotype of ploidy "
                                        f"{len(parts)}")
                if len(parts) > 1 and len(set(parts)) == 1:
                    gt = parts[0]
                if gt.isdigit():
                    k = int(gt)
                    if k == 0:
                        continue
                    alt = _valid_alt(alts[k - 1])
                    if alt:
                        _homozygous(sequences[name], insertions.setdefault(name, {}), pos, ref, alt)
                    continue
                if gt == ".":
                    for i in range(len(ref)):
                        sequences[name][pos + i] = "N"
                    continue
                insertions.setdefault(name, {})
                _heterozygous(gt, sequences[name], pos, ref, alts)
    positions = set()
    for muts in sequences.values():
        positions.update(muts.keys())
    if not positions and not sum(len(v) for v in insertions.values()):
        raise TreeTimeError(f"VCF file {vcf_file!r} has no data-lines which we could extract genotype "
                            "information from!")
    reference = None
    if ref_file:
        from .seqdata import read_fasta
        recs = read_fasta(ref_file)
        if len(recs) != 1:
            raise TreeTimeError(f"reference file {ref_file!r} must hold exactly one sequence")
        reference = next(iter(recs.values())).upper()
    return {"reference": reference, "sequences": sequences, "insertions": insertions,
            "positions": sorted(positions), "metadata": metadata}
