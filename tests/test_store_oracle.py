"""The overlap-store oracle (oracle/store_oracle.py) against canu's own ovStoreFilter.C
and ovOverlap.C (oracle/_ref/store_ref, built from the reference tree by
oracle/Makefile.store): filter, ID-swapped copies and sort, record for record.  CPU
only; skips where the canu tree was not available to build the checker."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, golden_cases, load_golden

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import store_oracle as so  # noqa: E402

STORE_REF = os.path.join(ROOT, "oracle", "_ref", "store_ref")


def run_ref(records, max_id, max_erate, tmp):
    if not os.path.exists(STORE_REF):
        pytest.skip("canu's store filter was not built (no canu tree here)")
    inp, out = os.path.join(tmp, "in.raw"), os.path.join(tmp, "out.raw")
    np.ascontiguousarray(records, dtype=np.uint32).tofile(inp)
    r = subprocess.run([STORE_REF, repr(max_erate), str(max_id), inp, out], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    return r.returncode, np.fromfile(out, dtype=np.uint32).reshape(-1, 6) if r.returncode == 0 else None, r.stdout


def synthetic(n, max_id, seed, ties=False):
    """Records with random IDs, hangs, spans, evalues, orientation and flags."""
    r = np.random.default_rng(seed)
    a = r.integers(1, max_id + 1, n).astype(np.uint64)
    b = r.integers(1, max_id + 1, n).astype(np.uint64)
    if ties:   # a few read pairs with several overlaps each
        a[: n // 2] = a[0]
        b[: n // 2] = r.integers(1, 4, n // 2)
    h = lambda: r.integers(0, 1 << 21, n).astype(np.uint64)
    ev = r.integers(0, 1 << 16, n).astype(np.uint64)
    fl = r.integers(0, 16, n).astype(np.uint64)          # flipped, forOBT, forDUP, forUTG
    d0 = h() | (h() << np.uint64(21)) | (ev << np.uint64(42)) | (fl << np.uint64(58))
    d1 = h() | (h() << np.uint64(21)) | (h() << np.uint64(42))
    m32 = np.uint64(0xffffffff)
    return np.stack([a, b, d0 >> np.uint64(32), d0 & m32, d1 >> np.uint64(32), d1 & m32], axis=1).astype(np.uint32)


@pytest.mark.parametrize("max_erate", [1.0, 0.02])
@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_oracle_matches_canu_on_golden_records(name, max_erate, tmp_path):
    rec, oc, _ = load_golden(name)
    n_reads = (len(oc) - 12) // 4 - 1
    rc, ref, counts = run_ref(rec, n_reads, max_erate, str(tmp_path))
    assert rc == 0
    got, cnt = so.store_sort(rec, n_reads, max_erate)
    assert got.shape == ref.shape and (got == ref).all()
    assert counts.split() == [str(len(ref))] + [str(c) for c in cnt]


@pytest.mark.parametrize("max_erate", [0.0, 0.005, 0.12, 0.65534, 0.65535, 0.9])
@pytest.mark.parametrize("ties", [False, True])
def test_oracle_matches_canu_on_synthetic_records(max_erate, ties, tmp_path):
    rec = synthetic(4000, 500, seed=int(max_erate * 1e5) + ties, ties=ties)
    rc, ref, counts = run_ref(rec, 500, max_erate, str(tmp_path))
    assert rc == 0
    got, cnt = so.store_sort(rec, 500, max_erate)
    assert (len(got) > 0 or max_erate == 0.0) and got.shape == ref.shape and (got == ref).all()
    assert counts.split() == [str(len(ref))] + [str(c) for c in cnt]


def test_ids_out_of_range_are_rejected_like_canu(tmp_path):
    rec = synthetic(10, 50, seed=3)
    rec[4, 1] = 51
    rc, _, _ = run_ref(rec, 50, 1.0, str(tmp_path))
    assert rc != 0
    with pytest.raises(ValueError):
        so.store_sort(rec, 50, 1.0)


def test_per_read_offsets():
    rec = np.array([[1, 2, 0, 0, 0, 0], [1, 3, 0, 0, 0, 0], [3, 1, 0, 0, 0, 0]], dtype=np.uint32)
    assert so.per_read_offsets(rec, 4).tolist() == [0, 0, 2, 2, 3, 3]
