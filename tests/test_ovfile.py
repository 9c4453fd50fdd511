"""The output files (include/oic_ovfile.h) against canu's own snappy and file layout,
the merge of independent jobs, and write-failure handling.  CPU only: these are host
functions of the library and the oracle's command line.

The snappy decoder used as the checker is canu's vendored copy (src/stores/libsnappy),
compiled under oracle/ by oracle/Makefile.snappy; its tests skip where the canu tree
was not available to build it."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import canu_gb300 as oic
from conftest import ROOT, golden_cases, load_golden

SNAPPY_REF = os.path.join(ROOT, "oracle", "_ref", "libsnappy_ref.so")
BLOCK_WORDS = 262080   # ovStoreFile.C:112-121 with the default 1 MiB buffer


def snappy_ref():
    if not os.path.exists(SNAPPY_REF):
        pytest.skip("canu's snappy was not built (no canu tree here)")
    lib = ctypes.CDLL(SNAPPY_REF)
    lib.snappy_ref_uncompressed_length.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    lib.snappy_ref_uncompress.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p]
    lib.snappy_ref_is_valid.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    lib.snappy_ref_max_compressed_length.restype = ctypes.c_size_t
    lib.snappy_ref_max_compressed_length.argtypes = [ctypes.c_size_t]
    lib.snappy_ref_compress.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p,
                                        ctypes.POINTER(ctypes.c_size_t)]
    return lib


def decode_with_reference(path):
    """ovFile::loadBuffer's loop (ovStoreFile.C:341-372) with canu's snappy: returns the
    records and the block sizes in words."""
    lib = snappy_ref()
    data = open(path, "rb").read()
    p, words, sizes = 0, [], []
    while p < len(data):
        bl = int.from_bytes(data[p:p + 8], "little")
        blk = data[p + 8:p + 8 + bl]
        assert len(blk) == bl, "short block"
        assert lib.snappy_ref_is_valid(blk, bl) == 1
        n = ctypes.c_size_t()
        assert lib.snappy_ref_uncompressed_length(blk, bl, ctypes.byref(n)) == 0
        out = ctypes.create_string_buffer(n.value)
        assert lib.snappy_ref_uncompress(blk, bl, out) == 0
        w = np.frombuffer(out.raw, dtype=np.uint32)
        words.append(w)
        sizes.append(len(w))
        p += 8 + bl
    rec = np.concatenate(words).reshape(-1, 6) if words else np.zeros((0, 6), np.uint32)
    return rec, sizes


def synthetic_records(n, seed=1):
    """Records shaped like overlapInCore's: runs of one a_iid, nearby b_iids, packed hangs."""
    r = np.random.default_rng(seed)
    a = np.sort(r.integers(1, 50000, n)).astype(np.uint32)
    b = (a + r.integers(1, 300, n)).astype(np.uint32)
    dat = r.integers(0, 2**32, (n, 4), dtype=np.uint64).astype(np.uint32)
    dat[:, 1] &= 0x00ffffff
    return np.column_stack([a, b, dat]).astype(np.uint32)


@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_ovb_decodes_with_canu_snappy(built, tmp_path, name):
    rec, _, _ = load_golden(name)
    path = str(tmp_path / "g.ovb")
    oic.write_ovb(path, rec)
    got, sizes = decode_with_reference(path)
    assert got.shape == rec.shape and (got == rec).all()
    assert all(s % 6 == 0 and s <= BLOCK_WORDS for s in sizes)
    back = oic.read_ovb(path)
    assert (back == rec).all()


def test_ovb_blocks_and_compression(built, tmp_path):
    rec = synthetic_records(150000)            # 900,000 words: four blocks
    path = str(tmp_path / "s.ovb")
    oic.write_ovb(path, rec)
    got, sizes = decode_with_reference(path)
    assert (got == rec).all()
    assert sizes == [BLOCK_WORDS] * 3 + [900000 - 3 * BLOCK_WORDS]
    # Real compression, not literal-only blocks: within 10 % of canu's own encoder.
    lib = snappy_ref()
    raw = rec[:BLOCK_WORDS // 6].tobytes()
    dst = ctypes.create_string_buffer(lib.snappy_ref_max_compressed_length(len(raw)))
    n = ctypes.c_size_t()
    lib.snappy_ref_compress(raw, len(raw), dst, ctypes.byref(n))
    ours = int.from_bytes(open(path, "rb").read(8), "little")
    assert ours < len(raw) and ours <= 1.1 * n.value, (ours, n.value, len(raw))


def test_reader_decodes_canu_compressed_blocks(built, tmp_path):
    """A file framed by canu's own compressor reads back through oic_ovb_read."""
    lib = snappy_ref()
    rec = synthetic_records(100000, seed=2)
    words = rec.reshape(-1)
    path = str(tmp_path / "c.ovb")
    with open(path, "wb") as f:
        for p in range(0, len(words), BLOCK_WORDS):
            raw = words[p:p + BLOCK_WORDS].tobytes()
            dst = ctypes.create_string_buffer(lib.snappy_ref_max_compressed_length(len(raw)))
            n = ctypes.c_size_t()
            lib.snappy_ref_compress(raw, len(raw), dst, ctypes.byref(n))
            f.write(n.value.to_bytes(8, "little") + dst.raw[:n.value])
    assert (oic.read_ovb(path) == rec).all()


@pytest.mark.parametrize("data", [b"", b"a", b"abcabcabcabcabcabcabc", bytes(range(256)) * 700, b"\0" * 200000])
def test_snappy_round_trip_edge_cases(built, data):
    lib = oic.library()
    src = ctypes.create_string_buffer(data, len(data))
    dst = ctypes.create_string_buffer(lib.oic_snappy_max_length(len(data)))
    n = ctypes.c_size_t()
    assert lib.oic_snappy_compress(src, len(data), dst, ctypes.byref(n)) == 0
    back = ctypes.create_string_buffer(max(1, len(data)))
    m = ctypes.c_size_t()
    assert lib.oic_snappy_uncompress(dst, n.value, back, len(data), ctypes.byref(m)) == 0
    assert m.value == len(data) and back.raw[:len(data)] == data
    if os.path.exists(SNAPPY_REF):
        ref = snappy_ref()
        out = ctypes.create_string_buffer(max(1, len(data)))
        assert ref.snappy_ref_uncompress(dst.raw[:n.value], n.value, out) == 0 and out.raw[:len(data)] == data


def test_malformed_ovb_is_rejected(built, tmp_path):
    path = str(tmp_path / "bad.ovb")
    oic.write_ovb(path, synthetic_records(100))
    raw = open(path, "rb").read()
    open(path, "wb").write(raw[:-3])               # truncated block
    with pytest.raises(ValueError):
        oic.read_ovb(path)
    open(path, "wb").write(raw[:8] + b"\xff" * (len(raw) - 8))   # garbage block
    with pytest.raises(ValueError):
        oic.read_ovb(path)


@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_oc_writer_matches_golden(built, tmp_path, name):
    rec, oc, _ = load_golden(name)
    n_reads = (len(oc) - 12) // 4 - 1
    path = str(tmp_path / "x.oc")
    lib = oic.library()
    r = np.ascontiguousarray(rec, dtype=np.uint32)
    assert lib.oic_oc_write(path.encode(), r.ctypes.data, len(r), n_reads) == 0
    assert open(path, "rb").read() == oc


def test_oc_name_follows_the_pipeline():
    # overlap.sh runs `-o ./$job.ovb.WORKING` and collects ./$job.oc (OverlapInCore.pm:187-197).
    assert oic.oc_path("./000001.ovb.WORKING") == "./000001.oc"
    assert oic.oc_path("/a.b/c/job.ovb") == "/a.b/c/job.oc"
    assert oic.oc_path("out") == "out.oc"


def test_write_failures_are_reported(built, tmp_path):
    rec = synthetic_records(1000)
    with pytest.raises(OSError):
        oic.write_ovb(str(tmp_path / "no_such_dir" / "x.ovb"), rec)
    if os.path.exists("/dev/full"):
        with pytest.raises(OSError):
            oic.write_ovb("/dev/full", rec)
        lib = oic.library()
        r = np.ascontiguousarray(rec)
        assert lib.oic_oc_write(b"/dev/full", r.ctypes.data, len(r), 60000) == 1


@pytest.mark.parametrize("which", ["ovb", "stats"])
def test_cli_unwritable_output_fails_before_any_work(built, tmp_path, which):
    """The drop-in opens its output files first (as overlapInCore.C:169 does) and exits 1
    when it cannot, before a GPU context is made."""
    db = str(tmp_path / "in.seqdb")
    oic.write_seqdb(db, ["ACGT" * 300, "TTGCA" * 200])
    bad = str(tmp_path / "missing_dir" / "o")
    out = bad + ".ovb" if which == "ovb" else str(tmp_path / "o.ovb")
    args = [built["cli"], "-k", "22", "-o", out] + (["-s", bad + ".stats"] if which == "stats" else []) + [db]
    r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 1 and "Failed to open" in r.stderr and "oic_create" not in r.stderr


def test_merge_of_disjoint_ref_ranges_equals_one_job(built, oracle, golden_inputs, tmp_path):
    """Two jobs on disjoint -r ranges, merged with oic_merge, give the one-job output:
    the same records and the same .oc bytes (the oracle computes the jobs)."""
    g = golden_inputs["default"]
    n = len(oic.read_seqdb(g["db"])[1])
    base = ["-t", "1", "-k", "22", "--hashbits", "16", "--maxerate", "0.06", "--minlength", "500", "-h", f"1-{n}"]
    outs = []
    for tag, rng in (("all", f"1-{n}"), ("p1", f"1-{n // 3}"), ("p2", f"{n // 3 + 1}-{n}")):
        raw = str(tmp_path / f"{tag}.raw.ovb")
        subprocess.run([oracle["cli"]] + base + ["-r", rng, "-o", raw, g["db"]], check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        framed = str(tmp_path / f"{tag}.ovb")
        oic.write_ovb(framed, np.fromfile(raw, dtype=np.uint32).reshape(-1, 6))
        os.replace(str(tmp_path / f"{tag}.raw.oc"), oic.oc_path(framed))
        outs.append(framed)
    merged = str(tmp_path / "merged.ovb")
    r = subprocess.run([os.path.join(oic.BUILD, "oic_merge"), merged, outs[1], outs[2]], stderr=subprocess.PIPE,
                       text=True)
    assert r.returncode == 0, r.stderr
    one = oic.sort_records(oic.read_ovb(outs[0]))
    got = oic.sort_records(oic.read_ovb(merged))
    assert len(one) > 100 and got.shape == one.shape and (got == one).all()
    assert open(oic.oc_path(merged), "rb").read() == open(oic.oc_path(outs[0]), "rb").read()
    assert len(oic.read_ovb(outs[1])) > 0 and len(oic.read_ovb(outs[2])) > 0


def test_merge_rejects_an_unframed_input(built, tmp_path):
    bad = str(tmp_path / "bad.ovb")
    open(bad, "wb").write(b"\x10\0\0\0\0\0\0\0abc")
    open(oic.oc_path(bad), "wb").write(np.array([0], "<u8").tobytes() + np.array([1, 0], "<u4").tobytes())
    r = subprocess.run([os.path.join(oic.BUILD, "oic_merge"), str(tmp_path / "m.ovb"), bad], stderr=subprocess.PIPE,
                       text=True)
    assert r.returncode == 1
