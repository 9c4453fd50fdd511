"""Frequent k-mers (the -k skip list): the CPU oracle's rules, and the GPU count against
the oracle."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import kmer_oracle as ko  # noqa: E402

import canu_gb300 as oic  # noqa: E402
from conftest import golden_inputs  # noqa: E402,F401


def test_oracle_folds_strands_and_skips_n():
    # ACGTT and its reverse complement AACGT are one k-mer; a window with N is skipped
    strs, cnt = ko.frequent([b"ACGTTN", b"AACGT"], 5, 1)
    assert strs == ["AACGT"] and list(cnt) == [2]
    strs, cnt = ko.frequent([b"ACGTTN", b"AACGT"], 5, 3)
    assert strs == [] and len(cnt) == 0


def test_oracle_matches_a_brute_force_count():
    r = np.random.default_rng(2)
    reads = [bytes(r.choice(list(b"ACGT"), 60).astype(np.uint8)) for _ in range(20)]
    comp = bytes.maketrans(b"ACGT", b"TGCA")
    k = 5
    brute = {}
    for s in reads:
        for o in range(len(s) - k + 1):
            w = s[o:o + k]
            rc = w[::-1].translate(comp)
            canon = min(w, rc, key=lambda x: ko._key([ko._CODE[b] for b in x]))
            brute[canon] = brute.get(canon, 0) + 1
    strs, cnt = ko.frequent(reads, k, 2)
    assert dict(zip(strs, cnt.tolist())) == {s.decode(): n for s, n in brute.items() if n >= 2}


@pytest.mark.gpu
@pytest.mark.parametrize("case,min_count", [("default", 1), ("default", 4), ("n_libs_minkmers", 2)])
def test_gpu_count_matches_oracle(case, min_count, built, golden_inputs):
    db = golden_inputs[case]["db"]
    lib, ln, off, bases = oic.read_seqdb(db)
    reads = [bytes(bases[o:o + l]) for o, l in zip(off.tolist(), ln.tolist())][:400]
    with oic.Overlapper(oic.default_params(kmerLen=22)) as ov:
        ov.set_reads_seqdb(db)
        strs, cnt = ov.count_kmers(1, len(reads), min_count)
    ref_s, ref_c = ko.frequent(reads, 22, min_count)
    assert len(strs) == len(ref_s) > 0
    assert strs == ref_s and np.array_equal(cnt, ref_c)


@pytest.mark.gpu
@pytest.mark.parametrize("pass_windows", [20000, 60000])
def test_gpu_count_in_key_space_passes_matches_oracle(pass_windows, built, golden_inputs, monkeypatch):
    """Read sets beyond one sort (2^32 windows, e.g. 8 Gbp of reads) are counted in
    passes over ranges of the canonical key space; forcing small passes here must give
    the same k-mers and counts, in the same ascending key order."""
    db = golden_inputs["default"]["db"]
    lib, ln, off, bases = oic.read_seqdb(db)
    reads = [bytes(bases[o:o + l]) for o, l in zip(off.tolist(), ln.tolist())][:400]
    monkeypatch.setenv("OIC_KMER_PASS_WINDOWS", str(pass_windows))
    with oic.Overlapper(oic.default_params(kmerLen=22)) as ov:
        ov.set_reads_seqdb(db)
        strs, cnt = ov.count_kmers(1, len(reads), 1)
    ref_s, ref_c = ko.frequent(reads, 22, 1)
    assert int((ln[:400].astype(np.int64) - 21).sum()) > 5 * pass_windows     # several passes
    assert strs == ref_s and np.array_equal(cnt, ref_c)


@pytest.mark.gpu
def test_skip_file_tool_writes_a_list_overlapincore_reads(built, golden_inputs, tmp_path):
    g = golden_inputs["repeats_noskip"] if "repeats_noskip" in golden_inputs else golden_inputs["default"]
    out = str(tmp_path / "ms22.dump")
    tool = os.path.join(oic.BUILD, "oic_kmers")
    r = subprocess.run([tool, "-k", "22", "--min-count", "3", "-o", out, g["db"]], stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    lines = open(out).read().split("\n")[:-1]
    assert lines and all(len(x.split("\t")[0]) == 22 and int(x.split("\t")[1]) >= 3 for x in lines)
    n = len(oic.read_seqdb(g["db"])[1])
    r = subprocess.run([built["cli"], "-k", "22", "-k", out, "--hashbits", "20", "--minlength", "500",
                        "-h", f"1-{n}", "-r", f"1-{n}", "-o", str(tmp_path / "o.ovb"), g["db"]],
                       stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0 and f"Read {len(lines)} kmers to mark to skip" in r.stderr, r.stderr[-2000:]
