"""The drop-in command line's argument handling (no GPU needed: every case ends before
a context is created)."""
import subprocess

import pytest


def run(built, *args):
    return subprocess.run([built["cli"]] + list(args), stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)


def test_unknown_flag_prints_usage_and_fails(built, tmp_path):
    # As in overlapInCore.C:387-393, the first unrecognised argument is the store path
    # and any later one is an unknown option.
    r = run(built, "-k", "22", "-o", str(tmp_path / "o.ovb"), "store", "--bogus")
    assert r.returncode == 1 and "Unknown option '--bogus'" in r.stderr and "USAGE" in r.stderr


def test_missing_kmer_size_and_output_are_errors(built):
    r = run(built, "store")
    assert r.returncode == 1
    assert "No kmer length supplied" in r.stderr and "No output file name specified" in r.stderr


def test_overlap_cap_is_rejected(built, tmp_path):
    # -l n makes read pairs depend on each other's processing order (a documented
    # difference); -l 0 (no cap) is accepted.
    r = run(built, "-k", "22", "-l", "5", "-o", str(tmp_path / "o.ovb"), "store")
    assert r.returncode == 1 and "-l (per-read overlap limit) is not supported" in r.stderr


@pytest.mark.parametrize("tune", ["wideThreads", "nope=3", "wideTile=2,bad=1"])
def test_bad_gpu_tune_is_rejected(built, tmp_path, tune):
    r = run(built, "-k", "22", "--gpu-tune", tune, "-o", str(tmp_path / "o.ovb"), "store")
    assert r.returncode == 1 and "bad --gpu-tune value" in r.stderr


def test_missing_store_is_reported(built, tmp_path):
    r = run(built, "-k", "22", "-o", str(tmp_path / "o.ovb"), str(tmp_path / "no_such.seqdb"))
    assert r.returncode == 1 and "Failed to load read container" in r.stderr


@pytest.mark.parametrize("damage", ["magic", "truncated_index", "truncated_bases", "offset_out_of_range"])
def test_malformed_read_container_is_rejected(built, tmp_path, damage):
    import struct
    import canu_gb300 as oic
    db = str(tmp_path / "in.seqdb")
    oic.write_seqdb(db, ["ACGT" * 300, "TTGCA" * 200])
    raw = bytearray(open(db, "rb").read())
    hdr = 8 + 4 + 4 + 8
    if damage == "magic":
        raw[0:8] = b"NOTSEQ01"
    elif damage == "truncated_index":
        raw = raw[:hdr + 10]
    elif damage == "truncated_bases":
        raw = raw[:-7]
    else:   # second read's offset pushed past the bases
        struct.pack_into("<Q", raw, hdr + 16 + 8, 10**9)
    open(db, "wb").write(bytes(raw))
    r = run(built, "-k", "22", "-o", str(tmp_path / "o.ovb"), db)
    assert r.returncode == 1 and "Failed to load read container" in r.stderr


def test_malformed_skip_list_is_rejected_before_device_work(built, tmp_path):
    """A -k k-mer file whose entries are not k bases long ends the run with the
    reference's message (Build_Hash_Index.C:222-226), before any device work."""
    import canu_gb300 as oic
    db = str(tmp_path / "in.seqdb")
    oic.write_seqdb(db, ["ACGT" * 300, "TTGCA" * 200])
    skip = tmp_path / "bad.skip"
    skip.write_text(">1\n" + "A" * 22 + "\t7\n>2\n" + "ACGT" * 5 + "\t3\n")
    r = run(built, "-k", "22", "-k", str(skip), "-o", str(tmp_path / "o.ovb"), db)
    assert r.returncode == 1
    assert "Short kmer skip kmer '" + "ACGT" * 5 + "' at line 4, expecting length 22 got length 20." in r.stderr
    assert "oic_create" not in r.stderr


def test_unwritable_metrics_file_fails_before_device_work(built, tmp_path):
    import canu_gb300 as oic
    db = str(tmp_path / "in.seqdb")
    oic.write_seqdb(db, ["ACGT" * 300, "TTGCA" * 200])
    r = run(built, "-k", "22", "--gpu-metrics", str(tmp_path / "no_such_dir" / "m.json"), "-o",
            str(tmp_path / "o.ovb"), db)
    assert r.returncode == 1 and "Failed to open" in r.stderr and "m.json" in r.stderr
    assert "oic_create" not in r.stderr
