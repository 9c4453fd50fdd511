"""The no-allocation DP entry point (oic_extend_batch_noalloc) against the allocating
one (oic_extend_batch), through the C ABI.

oic_extend_batch_noalloc serves callers that cannot call cudaMalloc when they align
(stream capture, a device memory pool they do not own, a fixed memory budget): the
problems and outputs are the caller's device buffers and the DP scratch is a static
device array.  This file runs last so that a failure here leaves every other test run;
it passes on its own in a fresh process as well as after the rest of the suite.
"""
import numpy as np
import pytest

import canu_gb300 as oic
from test_gpu_extend import make_problems


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
        prob = np.ascontiguousarray(a[:, [0, 1, 2, 3, 4, 5]].astype(np.int32))
        dprob = torch.from_numpy(prob).cuda()
        lib = oic.library()
        for call in range(2):
            dout = torch.full((n, 5), -7, dtype=torch.int32, device="cuda")
            dkind = torch.full((n,), -7, dtype=torch.int32, device="cuda")
            ddl = torch.full((n,), -7, dtype=torch.int32, device="cuda")
            dst = torch.full((n,), 99, dtype=torch.int32, device="cuda")
            torch.cuda.synchronize()
            rc = lib.oic_extend_batch_noalloc(ov._ctx, n, dprob.data_ptr(), dout.data_ptr(), dkind.data_ptr(),
                                              ddl.data_ptr(), dst.data_ptr())
            assert rc == oic.OIC_OK, lib.oic_last_error(ov._ctx)
            torch.cuda.synchronize()
            # Integer outputs: exact equality is the tolerance.
            assert (dst.cpu().numpy() == 0).all()
            assert (dout.cpu().numpy() == ref_out).all(), f"call {call}"
            assert (dkind.cpu().numpy() == ref_kind).all(), f"call {call}"
            assert (ddl.cpu().numpy() == ref_dl).all(), f"call {call}"
