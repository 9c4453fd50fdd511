"""The no-allocation DP entry point (oic_extend_batch_noalloc) against the allocating
one (oic_extend_batch), through the C ABI.

oic_extend_batch_noalloc serves callers that cannot call cudaMalloc when they align: a
program whose own allocator holds the whole device memory pool, or a plugin given a
fixed device-memory budget by its host program.  The problems and outputs are the
caller's device buffers and the DP scratch is a static device array.  This file runs
last so that a failure here leaves every other test run; it passes on its own in a
fresh process as well as after the rest of the suite.
"""
import os

import numpy as np
import pytest

import canu_gb300 as oic
from test_gpu_extend import make_problems

# Device flags a problem's status can carry (oic_common.cuh).
ERR_ARENA_FULL, ERR_BAND_WIDE, ERR_ROWS_FULL, ERR_INTERNAL = 1 << 1, 1 << 2, 1 << 3, 1 << 10


def _noalloc(torch, lib, ctx, prob):
    """One call on fresh device outputs; returns (rc, out, kind, deltaLen, status) on the host."""
    n = len(prob)
    dprob = torch.from_numpy(np.ascontiguousarray(prob.astype(np.int32))).cuda()
    dout = torch.full((n, 5), -7, dtype=torch.int32, device="cuda")
    dkind = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    ddl = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    dst = torch.full((n,), 99, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.oic_extend_batch_noalloc(ctx, n, dprob.data_ptr(), dout.data_ptr(), dkind.data_ptr(), ddl.data_ptr(),
                                      dst.data_ptr())
    torch.cuda.synchronize()
    return rc, dout.cpu().numpy(), dkind.cpu().numpy(), ddl.cpu().numpy(), dst.cpu().numpy()


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_twice(built, golden_inputs):
    torch = pytest.importorskip("torch")
    db = golden_inputs["default"]["db"]
    _, probs = make_problems(db, 300, np.random.default_rng(9))
    a = np.array(probs, dtype=np.int64)
    n = len(a)
    assert n >= 100
    with oic.Overlapper(oic.default_params(kmerLen=22, maxErate=0.06)) as ov:
        ov.set_reads_seqdb(db)
        ref_out, ref_kind, ref_dl = ov.extend_batch(a[:, 0] + 1, a[:, 1], a[:, 2] + 1, a[:, 3], a[:, 4], a[:, 5])
        # oic_extend_problem: u32 sRead, sRev, tRead (0-based reads); i32 mStart, mOffset, mLen
        lib = oic.library()
        for call in range(2):
            rc, out, kind, dl, st = _noalloc(torch, lib, ov._ctx, a)
            assert rc == oic.OIC_OK, lib.oic_last_error(ov._ctx)
            # Integer outputs: exact equality is the tolerance.
            assert (st == 0).all()
            assert (out == ref_out).all(), f"call {call}"
            assert (kind == ref_kind).all(), f"call {call}"
            assert (dl == ref_dl).all(), f"call {call}"


@pytest.mark.gpu
def test_noalloc_flags_oversized_and_invalid_problems(built, golden_inputs, tmp_path):
    """A problem beyond the static scratch and a problem naming a read outside the store
    are flagged in their own status entries; every other problem is still exact."""
    torch = pytest.importorskip("torch")
    _, ln, off, bases = oic.read_seqdb(golden_inputs["default"]["db"])
    reads = [bytes(bases[o:o + l]) for o, l in zip(off.tolist(), ln.tolist())]
    # A 30 kb read and a copy with a substitution at every tenth base: at --maxerate 0.12
    # the band around that alignment keeps widening, far past 512 diagonals and 131072
    # kept cells, so the static scratch cannot hold its DP.
    rng = np.random.default_rng(3)
    S = bytes(rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), 30000))
    T = bytearray(S)
    for i in range(9, len(T), 10):
        T[i] = {65: 67, 67: 71, 71: 84, 84: 65}[T[i]]
    db = os.path.join(tmp_path, "big.seqdb")
    oic.write_seqdb(db, reads + [S, bytes(T)])
    nr = len(reads)
    _, probs = make_problems(golden_inputs["default"]["db"], 60, np.random.default_rng(11))
    a = np.array(probs, dtype=np.int64)
    big = np.array([[nr, 0, nr + 1, 0, 0, 9]], dtype=np.int64)
    mixed = np.concatenate([a[:20], big, a[20:]])
    bad = mixed.copy()
    bad[5, 0] = nr + 7                       # S read index beyond the store
    with oic.Overlapper(oic.default_params(kmerLen=22, maxErate=0.12)) as ov:
        ov.set_reads_seqdb(db)
        ref_out, ref_kind, ref_dl = ov.extend_batch(mixed[:, 0] + 1, mixed[:, 1], mixed[:, 2] + 1, mixed[:, 3],
                                                    mixed[:, 4], mixed[:, 5])
        lib = oic.library()
        rc, out, kind, dl, st = _noalloc(torch, lib, ov._ctx, mixed)
        assert rc == oic.OIC_ERR_OVERFLOW, (rc, lib.oic_last_error(ov._ctx))
        assert st[20] & (ERR_ARENA_FULL | ERR_BAND_WIDE | ERR_ROWS_FULL), st[20]
        keep = np.arange(len(mixed)) != 20
        assert (st[keep] == 0).all()
        assert (out[keep] == ref_out[keep]).all() and (kind[keep] == ref_kind[keep]).all()
        assert (dl[keep] == ref_dl[keep]).all()

        rc, out, kind, dl, st = _noalloc(torch, lib, ov._ctx, bad)
        assert rc == oic.OIC_ERR_ARG, (rc, lib.oic_last_error(ov._ctx))
        assert st[5] == ERR_INTERNAL and kind[5] == 0
        keep = (np.arange(len(bad)) != 5) & (np.arange(len(bad)) != 20)
        assert (st[keep] == 0).all()
        assert (out[keep] == ref_out[keep]).all() and (kind[keep] == ref_kind[keep]).all()
        assert (dl[keep] == ref_dl[keep]).all()
