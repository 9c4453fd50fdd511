"""The overlap-store build's record pass on the GPU (oic_store_sort, oic_store_build)
against the store oracle (oracle/store_oracle.py, itself pinned to canu's
ovStoreFilter.C / ovOverlap.C): filtered records, ID-swapped copies, sort order,
per-read offsets and the filter counters, bit for bit."""
import os
import subprocess
import sys

import numpy as np
import pytest

import canu_gb300 as oic
from conftest import ROOT, golden_cases, golden_inputs, load_golden  # noqa: F401
from test_store_oracle import synthetic

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import store_oracle as so  # noqa: E402

pytestmark = pytest.mark.gpu
COUNTS = ("saved_unitigging", "saved_trimming", "discarded_erate", "discarded_no_trim", "discarded_flipped")


def check(rec, max_id, max_erate):
    got, per, cnt = oic.store_sort(rec, max_id, max_erate)
    ref, rcnt = so.store_sort(rec, max_id, max_erate)
    assert got.shape == ref.shape and (got == ref).all()
    assert (per == so.per_read_offsets(ref, max_id)).all()
    assert [cnt[k] for k in COUNTS] == rcnt
    return got


@pytest.mark.parametrize("max_erate", [1.0, 0.02])
@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_store_sort_matches_oracle_on_golden_records(name, max_erate):
    rec, oc, _ = load_golden(name)
    check(rec, (len(oc) - 12) // 4 - 1, max_erate)


@pytest.mark.parametrize("n,ties,max_erate", [(0, False, 1.0), (1, False, 1.0), (5000, False, 0.12),
                                               (5000, True, 0.9), (300000, False, 0.3), (300000, True, 0.05)])
def test_store_sort_matches_oracle_on_synthetic_records(n, ties, max_erate):
    rec = synthetic(n, 20000, seed=n + ties, ties=ties) if n else np.zeros((0, 6), np.uint32)
    check(rec, 20000, max_erate)


def test_ids_out_of_range_are_rejected():
    rec = synthetic(100, 50, seed=4)
    rec[7, 0] = 0
    with pytest.raises(oic.OicError) as e:
        oic.store_sort(rec, 50, 1.0)
    assert e.value.code == oic.OIC_ERR_INPUT


def test_store_build_tool_on_overlapper_output(built, golden_inputs, tmp_path):
    """overlapInCore on two disjoint ref ranges, then oic_store_build over both outputs:
    the sorted store records and per-read index equal the oracle's over their union."""
    g = golden_inputs["default"]
    n = len(oic.read_seqdb(g["db"])[1])
    base = ["-t", "4", "-k", "22", "--hashbits", "16", "--maxerate", "0.06", "--minlength", "500", "-h", f"1-{n}"]
    outs = []
    for tag, rng in (("p1", f"1-{n // 2}"), ("p2", f"{n // 2 + 1}-{n}")):
        o = str(tmp_path / f"{tag}.ovb")
        subprocess.run([built["cli"]] + base + ["-r", rng, "-o", o, g["db"]], check=True, stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL)
        outs.append(o)
    prefix = str(tmp_path / "store")
    r = subprocess.run([os.path.join(oic.BUILD, "oic_store_build"), "-O", prefix, "-S", g["db"], "-e", "0.05"] + outs,
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    allrec = np.concatenate([oic.read_ovb(o) for o in outs])
    ref, rcnt = so.store_sort(allrec, n, 0.05)
    got = oic.read_ovb(prefix + ".ovb")
    assert len(ref) > 1000 and got.shape == ref.shape and (got == ref).all()
    idx = np.fromfile(prefix + ".index", dtype=np.uint64)
    assert (idx == so.per_read_offsets(ref, n)).all()
    assert f"Saved      {rcnt[0]} unitigging overlaps" in r.stderr


def test_store_build_tool_writes_the_overlap_store_directory(built, golden_inputs, tmp_path):
    """oic_store_build --store: the store directory equals the one the library's store
    writer makes from the oracle's sorted records (tests/test_ovstore.py pins that writer
    byte for byte to canu's own ovStoreWriter)."""
    g = golden_inputs["default"]
    ln = oic.read_seqdb(g["db"])[1]
    n = len(ln)
    o = str(tmp_path / "job.ovb")
    subprocess.run([built["cli"], "-t", "4", "-k", "22", "--hashbits", "16", "--maxerate", "0.06", "--minlength",
                    "500", "-h", f"1-{n}", "-r", f"1-{n}", "-o", o, g["db"]], check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)
    store = str(tmp_path / "asm.ovlStore")
    r = subprocess.run([os.path.join(oic.BUILD, "oic_store_build"), "-O", str(tmp_path / "store"), "-S", g["db"],
                        "--store", store, o], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    ref, _ = so.store_sort(oic.read_ovb(o), n, 1.0)
    want = str(tmp_path / "want.ovlStore")
    oic.write_ovstore(want, ref, ln)
    names = sorted(os.listdir(want))
    assert len(ref) > 1000 and names == ["0001-001", "index", "info", "statistics"]
    assert sorted(os.listdir(store)) == names
    for f in names:
        assert open(os.path.join(store, f), "rb").read() == open(os.path.join(want, f), "rb").read(), f
