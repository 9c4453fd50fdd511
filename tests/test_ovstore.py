"""The overlap-store directory writer (oic_ovstore_write) against canu's own sequential
store writer and store reader (src/stores/ovStoreWriter.C, ovStore.C, ovStoreFile.C,
ovStoreHistogram.C, ovOverlap.C), compiled from the reference tree into
oracle/_ref/ovstore_ref by oracle/Makefile.ovstore.

The store files must be byte-identical to the ones canu writes from the same sorted
records (info, index, data files, statistics), and canu's reader must return every
record, both in store order and read by read.  CPU only; skips where the canu tree was
not available to build the checker."""
import os
import subprocess
import sys

import numpy as np
import pytest

import canu_gb300 as oic
from conftest import ROOT, golden_cases, load_golden

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import store_oracle as so  # noqa: E402

OVSTORE_REF = os.path.join(ROOT, "oracle", "_ref", "ovstore_ref")


def need_ref():
    if not os.path.exists(OVSTORE_REF):
        pytest.skip("canu's store writer was not built (no canu tree here)")


def ref_write(tmp, records, lens):
    """canu's ovStoreWriter over the sorted records; returns the store directory."""
    d = os.path.join(tmp, "ref.ovlStore")
    np.ascontiguousarray(lens, dtype=np.uint32).tofile(os.path.join(tmp, "lens.u32"))
    np.ascontiguousarray(records, dtype=np.uint32).tofile(os.path.join(tmp, "sorted.raw"))
    r = subprocess.run([OVSTORE_REF, "write", d, os.path.join(tmp, "lens.u32"), os.path.join(tmp, "sorted.raw")],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return d


def ref_read(tmp, store, lens):
    """canu's ovStore reader over a store: (records in store order, records read by read,
    the index's total)."""
    np.ascontiguousarray(lens, dtype=np.uint32).tofile(os.path.join(tmp, "lens.u32"))
    out = os.path.join(tmp, "back.raw")
    r = subprocess.run([OVSTORE_REF, "dump", store, os.path.join(tmp, "lens.u32"), out], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    total = int(r.stdout.split(":")[1])
    return (np.fromfile(out, dtype=np.uint32).reshape(-1, 6), np.fromfile(out + ".perread", dtype=np.uint32).reshape(-1, 6),
            total)


def same_files(ours, ref):
    names = sorted(os.listdir(ref))
    assert sorted(os.listdir(ours)) == names
    for f in names:
        a = open(os.path.join(ours, f), "rb").read()
        b = open(os.path.join(ref, f), "rb").read()
        if f == "index" and a != b and len(a) == len(b):
            # ovStoreOfft has 4 bytes of padding that canu leaves as the allocator gave
            # them; every field must still agree.
            A = np.frombuffer(a, np.uint8).reshape(-1, 24).copy()
            B = np.frombuffer(b, np.uint8).reshape(-1, 24).copy()
            A[:, 12:16] = 0
            B[:, 12:16] = 0
            assert (A == B).all(), f
        else:
            assert a == b, f
    return names


def check_store(tmp, records, lens):
    """Our store against canu's writer (bytes) and reader (records)."""
    ours = os.path.join(tmp, "ours.ovlStore")
    oic.write_ovstore(ours, records, lens)
    names = same_files(ours, ref_write(tmp, records, lens))
    seq, per, total = ref_read(tmp, ours, lens)
    assert seq.shape == records.shape and (seq == records).all()
    assert per.shape == records.shape and (per == records).all()
    assert total == len(records)
    return names


def sorted_store_records(rng, n_reads, per_read, lens):
    """Store records whose a reads have per_read[i] overlaps each, sorted, with A hangs
    inside the A read, random B hangs, spans, evalues and flags."""
    a = np.repeat(np.arange(1, n_reads + 1, dtype=np.uint64), per_read)
    n = len(a)
    b = rng.integers(1, n_reads + 1, n).astype(np.uint64)
    la = lens[(a - 1).astype(np.int64)].astype(np.uint64)
    ahg5 = (rng.random(n) * la * 0.5).astype(np.uint64)
    ahg3 = (rng.random(n) * (la - ahg5)).astype(np.uint64)
    h = lambda: rng.integers(0, 1 << 21, n).astype(np.uint64)
    ev = rng.integers(0, 1 << 16, n).astype(np.uint64)
    fl = rng.integers(0, 16, n).astype(np.uint64)
    d0 = ahg5 | (ahg3 << np.uint64(21)) | (ev << np.uint64(42)) | (fl << np.uint64(58))
    d1 = h() | (h() << np.uint64(21)) | (h() << np.uint64(42))
    m32 = np.uint64(0xffffffff)
    w = np.stack([a, b, d0 >> np.uint64(32), d0 & m32, d1 >> np.uint64(32), d1 & m32], axis=1).astype(np.uint32)
    return w[np.lexsort(w.T[::-1])]


@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_store_matches_canus_writer_on_golden_records(name, golden_inputs, tmp_path):
    """The overlapper's records of every golden case, filtered, copied and sorted as
    ovStoreBuild does (the store oracle), laid out as a store."""
    need_ref()
    rec, _, _ = load_golden(name)
    _, ln, _, _ = oic.read_seqdb(golden_inputs[name]["db"])
    srt, _ = so.store_sort(rec, len(ln), 1.0)
    names = check_store(str(tmp_path), srt, ln)
    assert names == ["0001-001", "index", "info", "statistics"]


@pytest.mark.parametrize("seed", [1, 2])
def test_store_matches_canus_writer_on_deep_reads(seed, tmp_path):
    """Reads with 0, 1, a few, more than 16 and more than 160 overlaps (the score
    profile's rank step is clamped to 1..10), and one read with more than 65,536 (its
    ranks wrap at 16 bits in canu's profile)."""
    need_ref()
    rng = np.random.default_rng(seed)
    n_reads = 60
    lens = rng.integers(500, 100000, n_reads).astype(np.uint32)
    per = rng.choice([0, 1, 3, 17, 40, 200, 900], n_reads)
    if seed == 2:
        per[7] = 70000
    w = sorted_store_records(rng, n_reads, per, lens)
    check_store(str(tmp_path), w, lens)


def test_store_split_into_data_files_reads_back_through_canus_reader(tmp_path):
    """A new data file starts at the first record of a read once the current file holds
    more than the per-file limit; canu's reader finds every record through the index."""
    need_ref()
    rng = np.random.default_rng(5)
    n_reads = 80
    lens = rng.integers(1000, 20000, n_reads).astype(np.uint32)
    per = rng.integers(0, 30, n_reads)
    w = sorted_store_records(rng, n_reads, per, lens)
    tmp = str(tmp_path)
    one, many = os.path.join(tmp, "one"), os.path.join(tmp, "many")
    oic.write_ovstore(one, w, lens)
    oic.write_ovstore(many, w, lens, max_per_file=50)
    files = sorted(f for f in os.listdir(many) if f.startswith("0001-"))
    assert len(files) > 5 and files[0] == "0001-001" and files[-1] == "0001-%03d" % len(files)
    data = b"".join(open(os.path.join(many, f), "rb").read() for f in files)
    assert data == open(os.path.join(one, "0001-001"), "rb").read()
    for f in ("info", "statistics"):
        assert open(os.path.join(one, f), "rb").read() == open(os.path.join(many, f), "rb").read()
    # Each file holds whole reads and, but for the last, more than 50 records.
    idx = np.frombuffer(open(os.path.join(many, "index"), "rb").read(), dtype=np.dtype(
        [("slice", "<u2"), ("piece", "<u2"), ("offset", "<u4"), ("n", "<u4"), ("pad", "<u4"), ("first", "<u8")]))
    sizes = np.bincount(idx["piece"], weights=idx["n"])[1:]
    assert (sizes[:-1] > 50).all() and sizes.sum() == len(w)
    seq, per_read, total = ref_read(tmp, many, lens)
    assert (seq == w).all() and (per_read == w).all() and total == len(w)


def test_empty_store_matches_canus_writer(tmp_path):
    need_ref()
    lens = np.full(12, 5000, dtype=np.uint32)
    names = check_store(str(tmp_path), np.zeros((0, 6), dtype=np.uint32), lens)
    assert names == ["index", "info"]


def test_store_writer_rejects_records_a_store_cannot_hold(tmp_path):
    rng = np.random.default_rng(9)
    lens = np.full(10, 3000, dtype=np.uint32)
    w = sorted_store_records(rng, 10, np.full(10, 4), lens)
    bad = {
        "unsorted": w[::-1].copy(),
        "a_iid 0": np.concatenate([np.array([[0, 1, 0, 0, 0, 0]], dtype=np.uint32), w]),
        "b_iid past maxID": np.concatenate([w, np.array([[10, 11, 0, 0, 0, 0]], dtype=np.uint32)]),
    }
    long_hang = w.copy()
    long_hang[-1, 3] = 3001          # ahg5 of the last record past its 3000-base read
    bad["A hangs past the read"] = long_hang
    for what, r in bad.items():
        with pytest.raises(ValueError):
            oic.write_ovstore(os.path.join(str(tmp_path), what.replace(" ", "_")), r, lens)
