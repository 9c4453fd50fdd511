"""oic_seqdb_import: FASTA / FASTQ files into the read container overlapInCore reads.
CPU only."""
import os
import subprocess

import numpy as np
import pytest

import canu_gb300 as oic
from conftest import golden_cases, sha256


@pytest.fixture(scope="module")
def importer(built):
    from canu_gb300.build import build_importer
    return build_importer()


def run(importer, *args):
    return subprocess.run([importer] + list(args), stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)


def reads_of(db):
    lib, ln, off, bases = oic.read_seqdb(db)
    return [(int(l), bytes(bases[o:o + n]).decode()) for l, n, o in zip(lib, ln, off)]


@pytest.mark.parametrize("name", ["default", "hifi", "noise"])
def test_exported_fasta_imports_to_the_same_container(importer, golden_inputs, tmp_path, name):
    """A golden case's reads written as wrapped FASTA and imported again give the
    container the fixture was made from, byte for byte."""
    db = golden_inputs[name]["db"]
    fa = tmp_path / "reads.fasta"
    with open(fa, "w") as f:
        for i, (_, s) in enumerate(reads_of(db)):
            f.write(f">read{i + 1} some description\n")
            for k in range(0, len(s), 60):
                f.write(s[k:k + 60] + "\n")
    out = str(tmp_path / "again.seqdb")
    r = run(importer, "-o", out, str(fa))
    assert r.returncode == 0, r.stderr
    assert sha256(out) == golden_cases()[name]["seqdb_sha256"]
    names = open(out + ".readNames.txt").read().splitlines()
    assert names[0] == "1\tread1" and names[-1] == f"{len(names)}\tread{len(names)}"


def test_libraries_cases_codes_wrapping_and_length_filter(importer, tmp_path):
    fa = tmp_path / "a.fasta"
    fa.write_bytes(b">r1 x\r\nacgtACGT\r\nnnRY\r\n\r\n>r2\nGG\n>r3\n\nTTTTTTTTTT\nAA\n")
    fq = tmp_path / "b.fastq"
    fq.write_text("@q1 run=7\nACGTACGTAC\n+\n@@@@@IIIII\n@q2\nACGT\nNNKM\n+q2\nIIII\nIIII\n\n@q3\nA\n+\n#\n")
    out = str(tmp_path / "r.seqdb")
    r = run(importer, "-o", out, "--min-length", "3", str(fa), str(fq))
    assert r.returncode == 0, r.stderr
    assert reads_of(out) == [(1, "ACGTACGTNNNN"), (1, "TTTTTTTTTTAA"), (2, "ACGTACGTAC"), (2, "ACGTNNNN")]
    assert open(out + ".readNames.txt").read() == "1\tr1\n2\tr3\n3\tq1\n4\tq2\n"


@pytest.mark.parametrize("content,msg", [
    ("@q1\nACGT\n+\nIII\n", "quality length 3 differs from sequence length 4"),
    ("@q1\nACGT\n", "has no '+' line"),
    ("ACGT\n", "starts neither a FASTA nor a FASTQ record"),
])
def test_malformed_input_is_rejected_and_nothing_is_written(importer, tmp_path, content, msg):
    bad = tmp_path / "bad.fq"
    bad.write_text(content)
    out = str(tmp_path / "r.seqdb")
    r = run(importer, "-o", out, str(bad))
    assert r.returncode == 1 and msg in r.stderr
    assert not os.path.exists(out)


def test_missing_input_and_unwritable_output_fail(importer, tmp_path):
    r = run(importer, "-o", str(tmp_path / "r.seqdb"), str(tmp_path / "none.fasta"))
    assert r.returncode == 1 and "cannot open" in r.stderr
    fa = tmp_path / "a.fasta"
    fa.write_text(">r\nACGT\n")
    r = run(importer, "-o", str(tmp_path / "no_dir" / "r.seqdb"), str(fa))
    assert r.returncode == 1 and "Failed to write" in r.stderr


def test_imported_reads_run_through_the_oracle(importer, oracle, golden_inputs, tmp_path):
    """The imported container is what the overlapper reads: the oracle's overlaps of the
    re-imported default case equal those of the original container."""
    db = golden_inputs["default"]["db"]
    fa = tmp_path / "reads.fa"
    fa.write_text("".join(f">x{i}\n{s.lower()}\n" for i, (_, s) in enumerate(reads_of(db))))
    out = str(tmp_path / "imp.seqdb")
    assert run(importer, "-o", out, str(fa)).returncode == 0
    n = len(reads_of(db))
    args = ["-t", "2", "-k", "22", "--hashbits", "16", "--maxerate", "0.06", "--minlength", "500", "-h", f"1-{n}",
            "-r", f"1-{n}"]
    recs = []
    for path, tag in ((db, "a"), (out, "b")):
        o = str(tmp_path / f"{tag}.ovb")
        subprocess.run([oracle["cli"]] + args + ["-o", o, path], check=True, stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL)
        recs.append(oic.sort_records(np.fromfile(o, dtype=np.uint32).reshape(-1, 6)))
    assert len(recs[0]) > 1000 and recs[0].shape == recs[1].shape and (recs[0] == recs[1]).all()


def test_read_longer_than_a_store_holds_is_rejected(importer, tmp_path):
    fa = tmp_path / "long.fa"
    fa.write_text(">ok\nACGT\n>huge\n" + "A" * ((1 << 21) - 1) + "C\n")
    out = str(tmp_path / "r.seqdb")
    r = run(importer, "-o", out, str(fa))
    assert r.returncode == 1 and "read 'huge' has 2097152 bases, more than the 2097151" in r.stderr
    assert not os.path.exists(out)
    fa.write_text(">ok\nACGT\n>edge\n" + "A" * ((1 << 21) - 1) + "\n")
    assert run(importer, "-o", out, str(fa)).returncode == 0
    assert [len(s) for _, s in reads_of(out)] == [4, (1 << 21) - 1]
