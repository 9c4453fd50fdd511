"""CPU oracle of the overlap-store build's record pass -- test infrastructure only.

A numpy restatement of what canu's ovStoreBuild does to the overlapper's records before
its store writer lays them out (src/stores/ovStoreBuild.C:166-255):
  * ovStoreFilter::filterOverlap (src/stores/ovStoreFilter.C:62-160): IDs must lie in
    1..maxID; a record whose evalue exceeds AS_OVS_encodeEvalue(maxErate)
    (ovOverlap.H:35) loses forUTG/forOBT/forDUP; the counters count both copies;
  * ovOverlap::swapIDs (src/stores/ovOverlap.C:216-246): a and b exchanged, the A and B
    hangs exchanged, and 5' with 3' as well when the overlap is flipped;
  * a record and its copy are kept when one of the three flags is set
    (ovStoreBuild.C:190-201), then sorted by ovOverlap::operator< (a_iid, b_iid, dat[0],
    dat[1]; ovOverlap.H:264-277) -- lexicographic on the six record words.
It is pinned against canu's own ovStoreFilter.C / ovOverlap.C compiled under oracle/
(oracle/_ref/store_ref) by tests/test_store_oracle.py."""
import numpy as np

M21 = np.uint64((1 << 21) - 1)


def encode_evalue(q):
    """AS_OVS_encodeEvalue in double arithmetic."""
    return int(100000.0 * q + 0.5) if q < 65535 / 100000.0 else 65535


def store_sort(words, max_id, max_erate=1.0):
    """(sorted records (m, 6) uint32, counters [saveUTG, saveOBT, skipERATE, skipOBT,
    skipFLIPPED]); raises ValueError for an ID outside 1..max_id."""
    w = np.asarray(words, dtype=np.uint32).reshape(-1, 6).astype(np.uint64)
    a, b = w[:, 0], w[:, 1]
    if len(w) and ((a == 0) | (b == 0) | (a > max_id) | (b > max_id)).any():
        raise ValueError("overlap has IDs out of range")
    d0 = (w[:, 2] << np.uint64(32)) | w[:, 3]
    d1 = (w[:, 4] << np.uint64(32)) | w[:, 5]
    bad = ((d0 >> np.uint64(42)) & np.uint64(0xffff)) > np.uint64(encode_evalue(max_erate))
    d0 = np.where(bad, d0 & ~np.uint64(7 << 59), d0)
    ahg5, ahg3 = d0 & M21, (d0 >> np.uint64(21)) & M21
    bhg5, bhg3 = d1 & M21, (d1 >> np.uint64(21)) & M21
    flip = ((d0 >> np.uint64(58)) & np.uint64(1)).astype(bool)
    ra5, ra3 = np.where(flip, bhg3, bhg5), np.where(flip, bhg5, bhg3)
    rb5, rb3 = np.where(flip, ahg3, ahg5), np.where(flip, ahg5, ahg3)
    clear = ~(M21 | (M21 << np.uint64(21)))
    r0 = (d0 & clear) | ra5 | (ra3 << np.uint64(21))
    r1 = (d1 & clear) | rb5 | (rb3 << np.uint64(21))
    keep = ((d0 >> np.uint64(59)) & np.uint64(7)) != 0

    def rec(x, y, e0, e1):
        return np.stack([x, y, e0 >> np.uint64(32), e0 & np.uint64(0xffffffff), e1 >> np.uint64(32),
                         e1 & np.uint64(0xffffffff)], axis=1).astype(np.uint32)
    allrec = np.concatenate([rec(a, b, d0, d1)[keep], rec(b, a, r0, r1)[keep]])
    if len(allrec):
        allrec = allrec[np.lexsort(tuple(allrec[:, k] for k in range(5, -1, -1)))]
    utg = int(((d0 >> np.uint64(61)) & np.uint64(1)).sum()) * 2
    obt = int(((d0 >> np.uint64(59)) & np.uint64(1)).sum()) * 2
    return allrec.reshape(-1, 6), [utg, obt, 2 * int(bad.sum()), 0, 0]


def per_read_offsets(records, max_id):
    """Index of the first record of every a_iid (max_id + 2 entries, the last = count)."""
    cnt = np.bincount(np.asarray(records).reshape(-1, 6)[:, 0], minlength=max_id + 2)[: max_id + 2]
    off = np.zeros(max_id + 2, dtype=np.uint64)
    off[1:] = np.cumsum(cnt[:-1])
    off[max_id + 1] = len(np.asarray(records).reshape(-1, 6))
    return off
