"""CPU oracle of the frequent-k-mer count -- TEST INFRASTRUCTURE ONLY (tests/ may import
it; the product path never does).

Restates what canu's meryl does for overlapInCore's skip list (src/pipelines/canu/
Meryl.pm: count every k-mer of the reads with a k-mer and its reverse complement as
one, print those at or above a threshold), with the key encoding of the GPU engine:
base i of a window in bits 2i..2i+1 (A=0 C=1 G=2 T=3), canonical key = the smaller of
the window's key and its reverse complement's.  Windows holding an N are skipped.
"""
import numpy as np

_CODE = {ord(c): i for i, c in enumerate("ACGT")}
_CODE.update({ord(c): i for i, c in enumerate("acgt")})


def _key(codes):
    k = 0
    for i, c in enumerate(codes):
        k |= c << (2 * i)
    return k


def count(reads, k):
    """dict canonical key -> count over the reads (iterable of bytes)."""
    out = {}
    for s in reads:
        L = len(s)
        for o in range(L - k + 1):
            w = s[o:o + k]
            codes = [_CODE.get(b, -1) for b in w]
            if min(codes) < 0:
                continue
            fk = _key(codes)
            rk = _key([3 - c for c in reversed(codes)])
            key = fk if fk < rk else rk
            out[key] = out.get(key, 0) + 1
    return out


def frequent(reads, k, min_count):
    """(k-mer strings, counts) with count >= min_count, ascending canonical key."""
    c = count(reads, k)
    keys = sorted(x for x, n in c.items() if n >= min_count)
    strs = ["".join("ACGT"[(x >> (2 * i)) & 3] for i in range(k)) for x in keys]
    return strs, np.array([c[x] for x in keys], dtype=np.uint32)
