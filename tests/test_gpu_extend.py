"""The warp DP (oic_extend_batch) against the oracle's Extend_Alignment, problem by problem."""
import ctypes

import numpy as np
import pytest

import canu_gb300 as oic
from conftest import golden_inputs  # noqa: F401  (fixture)

COMP = bytes.maketrans(b"ACGTNacgtn", b"TGCANtgcan")


def port_aligner(lib, erate, noise, partial):
    lib.oic_port_aligner_new.restype = ctypes.c_void_p
    lib.oic_port_aligner_new.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int]
    lib.oic_port_extend.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int32, ctypes.c_char_p, ctypes.c_int32,
                                    ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.oic_port_aligner_free.argtypes = [ctypes.c_void_p]
    return lib.oic_port_aligner_new(erate, noise, partial)


def make_problems(db, n_pairs, rng, k=22):
    lib, ln, off, bases = oic.read_seqdb(db)
    seqs = [bytes(bases[o:o + l]).lower() for o, l in zip(off.tolist(), ln.tolist())]
    index = {}
    for t, s in enumerate(seqs):
        for p in range(0, len(s) - k + 1, 7):
            index.setdefault(s[p:p + k], []).append((t, p))
    probs = []
    for _ in range(n_pairs * 20):
        if len(probs) >= n_pairs:
            break
        si = int(rng.integers(len(seqs)))
        rev = int(rng.integers(2))
        s = seqs[si] if not rev else seqs[si][::-1].translate(COMP)
        p = int(rng.integers(0, len(s) - k))
        hits = [h for h in index.get(s[p:p + k], []) if h[0] != si]
        if hits:
            t, q = hits[int(rng.integers(len(hits)))]
            probs.append((si, rev, t, p, q, k))
        elif rng.random() < 0.2:   # an unrelated pair: exercises the non-dovetail exits
            t = int(rng.integers(len(seqs)))
            q = int(rng.integers(0, len(seqs[t]) - k))
            probs.append((si, rev, t, p, q, k))
    return seqs, probs


@pytest.mark.gpu
@pytest.mark.parametrize("case,erate,partial", [("default", 0.06, 0), ("hierr", 0.12, 0), ("hierr_partial", 0.12, 1),
                                                ("hifi", 0.01, 0), ("n_libs_minkmers", 0.06, 0)])
def test_extend_batch_matches_oracle(case, erate, partial, built, oracle, golden_inputs):
    rng = np.random.default_rng(5)
    db = golden_inputs[case]["db"]
    seqs, probs = make_problems(db, 300, rng)
    assert len(probs) >= 100
    erate = float(np.float32(erate))
    p = oic.default_params(kmerLen=22, maxErate=erate, partial=partial)
    with oic.Overlapper(p) as ov:
        ov.set_reads_seqdb(db)
        a = np.array(probs, dtype=np.int64)
        out, kind, dl = ov.extend_batch(a[:, 0] + 1, a[:, 1], a[:, 2] + 1, a[:, 3], a[:, 4], a[:, 5])
    plib = ctypes.CDLL(oracle["lib"])
    al = port_aligner(plib, erate, 1.0, partial)
    comp = bytes.maketrans(b"acgtn", b"tgcan")
    for i, (si, rev, t, ms, mo, ml) in enumerate(probs):
        S = seqs[si] if not rev else seqs[si][::-1].translate(comp)
        T = seqs[t]
        o = np.zeros(5, dtype=np.int32)
        dlen = ctypes.c_int32()
        k = plib.oic_port_extend(al, S, len(S), T, len(T), ms, mo, ml, o.ctypes.data, None, ctypes.byref(dlen), None,
                                 None)
        assert k == kind[i] and (o == out[i]).all() and dlen.value == dl[i], (i, probs[i], k, o, kind[i], out[i])
    plib.oic_port_aligner_free(al)


@pytest.mark.gpu
def test_match_limit_table_matches_oracle(built, oracle):
    plib = ctypes.CDLL(oracle["lib"])
    plib.oic_port_max_errors.restype = ctypes.c_int32
    plib.oic_port_max_errors.argtypes = [ctypes.c_double]
    plib.oic_port_match_limit.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int32]
    for erate in (0.01, 0.06, 0.12):
        e = float(np.float32(erate))
        with oic.Overlapper(oic.default_params(kmerLen=22, maxErate=erate)) as ov:
            ml = ov.match_limit()
        n = plib.oic_port_max_errors(e)
        ref = np.zeros(n + 1, dtype=np.int32)
        plib.oic_port_match_limit(ref.ctypes.data, e, n)
        assert len(ml) == n + 1 and (ml[:n] == ref[:n]).all()
