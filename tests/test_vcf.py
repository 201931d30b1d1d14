"""VCF reading and sparse alignments against TreeTime's own results
(tests/golden/vcf_cases.npz, made by running TreeTime's read_vcf, its
SequenceData on the sparse alignment and a marginal reconstruction).  CPU
only, except the reconstruction."""

import os

import numpy as np
import pytest

import golden_cases as gc
from treetime_gb300.vcf import read_vcf

G = gc.load("vcf_cases")


def _write(tmp_path, name, text):
    p = os.path.join(str(tmp_path), name)
    with open(p, "w") as fh:
        fh.write(str(text))
    return p


def _flat(d):
    keys = sorted((k, p) for k, v in d.items() for p in v)
    return ([k for k, _ in keys], [p for _, p in keys], [d[k][p] for k, p in keys])


def test_read_vcf_diploid_calls_match_treetime(tmp_path, capsys):
    res = read_vcf(_write(tmp_path, "d.vcf", G["d_vcf_text"]))
    names, pos, chars = _flat(res["sequences"])
    assert names == G["d_seq_name"].tolist()
    assert pos == G["d_seq_pos"].tolist()
    assert chars == G["d_seq_chr"].tolist()
    names, pos, strs = _flat(res["insertions"])
    assert names == G["d_ins_name"].tolist() and pos == G["d_ins_pos"].tolist() and strs == G["d_ins_str"].tolist()
    assert sorted(res["insertions"].keys()) == G["d_ins_keys"].tolist()
    assert res["positions"] == G["d_positions"].tolist()
    assert res["metadata"]["ploidy"] == int(G["d_ploidy"])
    assert res["metadata"]["chrom"] == str(G["d_chrom"])
    assert "invalid allele" in capsys.readouterr().out


def test_read_vcf_haploid_with_reference_matches_treetime(tmp_path):
    ref = _write(tmp_path, "ref.fasta", ">ref\n" + str(G["h_ref"]) + "\n")
    res = read_vcf(_write(tmp_path, "h.vcf", G["h_vcf_text"]), ref)
    assert res["reference"] == str(G["h_ref"])
    names, pos, chars = _flat(res["sequences"])
    assert names == G["h_seq_name"].tolist()
    assert pos == G["h_seq_pos"].tolist()
    assert chars == G["h_seq_chr"].tolist()
    assert list(res["sequences"].keys()) == G["h_names"].tolist()
    assert res["positions"] == G["h_positions"].tolist()


def test_sparse_compression_matches_treetime(tmp_path):
    from treetime_gb300.seqdata import SequenceData
    ref = _write(tmp_path, "ref.fasta", ">ref\n" + str(G["h_ref"]) + "\n")
    res = read_vcf(_write(tmp_path, "h.vcf", G["h_vcf_text"]), ref)
    sd = SequenceData(res["sequences"], ref=res["reference"], ambiguous="N")
    assert sd.is_sparse
    assert list(sd.compressed_alignment.keys()) == G["h_comp_names"].tolist()
    np.testing.assert_array_equal(sd.compressed_codes, G["h_comp_codes"])
    np.testing.assert_array_equal(sd.multiplicity(), G["h_mult"])
    np.testing.assert_array_equal(sd.full_to_compressed_sequence_map, G["h_f2c"])
    assert sorted(sd.inferred_const_sites) == G["h_const_amb"].tolist()
    # the reference may also come as a FASTA file name
    sd2 = SequenceData(res["sequences"], ref=ref, ambiguous="N")
    np.testing.assert_array_equal(sd2.compressed_codes, G["h_comp_codes"])


def test_vcf_file_as_alignment(tmp_path):
    from treetime_gb300.seqdata import SequenceData
    sd = SequenceData(_write(tmp_path, "h.vcf", G["h_vcf_text"]), ref=str(G["h_ref"]), ambiguous="N")
    np.testing.assert_array_equal(sd.compressed_codes, G["h_comp_codes"])


@pytest.mark.gpu
def test_marginal_reconstruction_of_sparse_alignment_matches_treetime(tmp_path):
    from treetime_gb300 import TreeAnc
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import parse_newick
    ref = _write(tmp_path, "ref.fasta", ">ref\n" + str(G["h_ref"]) + "\n")
    res = read_vcf(_write(tmp_path, "h.vcf", G["h_vcf_text"]), ref)
    for precision, rel in (("f64", 1e-10), ("f32", 1e-6)):
        t = TreeAnc(tree=parse_newick(str(G["h_newick"])), aln=res["sequences"], ref=res["reference"],
                    gtr=GTR.custom(mu=1.0, pi=np.ones(5), W=np.ones((5, 5)), alphabet="nuc"), verbose=0,
                    precision=precision)
        t.infer_ancestral_sequences(marginal=True)
        want = float(G["h_marg_total_LH"])
        assert abs(t.tree.total_sequence_LH - want) <= rel * abs(want)


# ------------------------------------------------- constant sites beyond the alignment
E = gc.load("extra_sites")


@pytest.mark.parametrize("tag", ["nuc", "aa"])
def test_additional_constant_sites_match_treetime(tag):
    from treetime_gb300.seqdata import SequenceData
    aln = dict(zip(E[tag + "_aln_names"].tolist(), E[tag + "_aln_seqs"].tolist()))
    sd = SequenceData(aln, sequence_length=int(E[tag + "_seq_len"]), ambiguous="N" if tag == "nuc" else "X")
    assert sd.full_length == int(E[tag + "_seq_len"])
    assert list(sd.compressed_alignment.keys()) == E[tag + "_comp_names"].tolist()
    np.testing.assert_array_equal(sd.compressed_codes, E[tag + "_comp_codes"])
    np.testing.assert_array_equal(sd.multiplicity(), E[tag + "_mult"])
    np.testing.assert_array_equal(sd.full_to_compressed_sequence_map, E[tag + "_f2c"])


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ["nuc", "aa"])
def test_additional_constant_sites_reconstruction_matches_treetime(tag):
    from treetime_gb300 import TreeAnc
    from treetime_gb300.gtr import GTR
    from treetime_gb300.tree import parse_newick
    aln = dict(zip(E[tag + "_aln_names"].tolist(), E[tag + "_aln_seqs"].tolist()))
    alphabet = str(E[tag + "_param_alphabet"])
    g = GTR.custom(mu=1.0, pi=E[tag + "_param_pi"], W=E[tag + "_param_W"], alphabet=alphabet)
    t = TreeAnc(tree=parse_newick(str(E[tag + "_newick"])), aln=aln, gtr=g, verbose=0,
                seq_len=int(E[tag + "_seq_len"]))
    t.infer_ancestral_sequences(marginal=True)
    want = float(E[tag + "_marg_total_LH"])
    assert abs(t.tree.total_sequence_LH - want) <= 1e-10 * abs(want)


def test_treetime_vcf_reader_suite_passes_with_this_reader(tmp_path):
    """TreeTime's own read_vcf tests (its test/test_vcf.py: malformed files,
    multiple chromosomes, simple files, no-calls and missing alleles, the VCF
    specification's examples, mutation plus insertion, metadata) run against
    this package's reader.  The writing tests (write_vcf) are not part of it.
    Skipped unless TREETIME_SOURCE names the TreeTime sources."""
    import subprocess
    import sys
    src = os.environ.get("TREETIME_SOURCE")
    suite = os.path.join(src, "test", "test_vcf.py") if src else ""
    if not src or not os.path.isfile(suite):
        pytest.skip("TreeTime sources not given (set TREETIME_SOURCE to their path)")
    here = os.path.dirname(os.path.abspath(__file__))
    repo = os.path.dirname(here)
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([os.path.join(repo, "oracle", "bioshim"), src, repo,
                                         os.path.join(here, "golden"), env.get("PYTHONPATH", "")])
    r = subprocess.run([sys.executable, "-m", "pytest", suite, "-q", "-p", "vcf_reader_plugin", "-p",
                        "no:cacheprovider", "-k", "not TestWriting and not roundtrip", "--rootdir", str(tmp_path)],
                       env=env, cwd=str(tmp_path), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
