"""Learned candidate filter on the GPU: the tensor-core MLP kernels against the CPU
oracle (forward values, gradients, Adam), the feature rows against the oracle's, and
the filtered path's output against the plain path's."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import filter_oracle as fo  # noqa: E402

import canu_gb300 as oic  # noqa: E402
from canu_gb300 import filter_train, workloads  # noqa: E402

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _params(seed):
    r = np.random.default_rng(seed)
    p = fo.init_params(seed).astype(np.float64)
    for k in ("b1", "b2"):
        o = fo.OFF[k][0]
        p[o:o + 128] = r.normal(0, 0.2, 128)
    p[fo.OFF["b3"][0]] = 0.3
    return p.astype(np.float16)


def _x(n, seed):
    r = np.random.default_rng(seed)
    x = r.normal(0, 1, (n, fo.IN))
    x[:, 67:] = 0
    return x.astype(np.float16)


def _dev16(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int16).copy()).cuda()


def _host16(t):
    return t.cpu().numpy().view(np.float16)


def _forward(p16, x16):
    n = len(x16)
    dp, dx = _dev16(p16), _dev16(x16)
    logit = torch.empty(n, dtype=torch.float32, device="cuda")
    h1 = torch.empty((n, 128), dtype=torch.int16, device="cuda")
    h2 = torch.empty_like(h1)
    oic.mlp_forward(dp.data_ptr(), dx.data_ptr(), n, logit.data_ptr(), h1.data_ptr(), h2.data_ptr())
    torch.cuda.synchronize()
    return dp, dx, logit, h1, h2


@pytest.mark.parametrize("n", [1, 16, 1000, 4099])
def test_forward_matches_oracle_layer_by_layer(n):
    p16, x16 = _params(n), _x(n, n + 1)
    _, _, logit, h1, h2 = _forward(p16, x16)
    P = fo.unpack(p16)
    H1, H2 = _host16(h1).astype(np.float64), _host16(h2).astype(np.float64)
    X = x16.astype(np.float64)
    # each layer from the kernel's own input: FP32 accumulation vs float64, then FP16
    ref1 = np.maximum(X @ P["w1"].T + P["b1"], 0).astype(np.float16).astype(np.float64)
    np.testing.assert_allclose(H1, ref1, rtol=2e-3, atol=1e-4)
    ref2 = np.maximum(H1 @ P["w2"].T + P["b2"], 0).astype(np.float16).astype(np.float64)
    np.testing.assert_allclose(H2, ref2, rtol=2e-3, atol=1e-4)
    np.testing.assert_allclose(logit.cpu().numpy(), H2 @ P["w3"] + P["b3"][0], rtol=1e-5, atol=1e-5)
    # and end to end against the oracle's own rounding chain
    z, _, _ = fo.forward(p16, x16)
    np.testing.assert_allclose(logit.cpu().numpy(), z, rtol=2e-2, atol=2e-2)


def test_forward_without_activations_gives_the_same_logits():
    p16, x16 = _params(7), _x(777, 8)
    dp, dx, logit, _, _ = _forward(p16, x16)
    l2 = torch.empty_like(logit)
    oic.mlp_forward(dp.data_ptr(), dx.data_ptr(), len(x16), l2.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(logit, l2)


def _backward(dp, dx, h1, h2, logit, y, w, n):
    dy = torch.from_numpy(y.astype(np.float32)).cuda()
    dw = torch.from_numpy(w.astype(np.float32)).cuda() if w is not None else None
    grad = torch.zeros(fo.NPARAM, dtype=torch.float32, device="cuda")
    g1 = torch.empty((n, 128), dtype=torch.int16, device="cuda")
    g2 = torch.empty_like(g1)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    oic.mlp_backward(dp.data_ptr(), dx.data_ptr(), h1.data_ptr(), h2.data_ptr(), logit.data_ptr(), dy.data_ptr(),
                     dw.data_ptr() if dw is not None else 0, n, grad.data_ptr(), g1.data_ptr(), g2.data_ptr(),
                     loss.data_ptr())
    torch.cuda.synchronize()
    return grad.cpu().numpy().astype(np.float64), float(loss.item())


@pytest.mark.parametrize("n,weighted", [(37, True), (1000, False), (5003, True)])
def test_gradients_match_the_cpu_oracle(n, weighted):
    p16, x16 = _params(n + 11), _x(n, n + 12)
    r = np.random.default_rng(n)
    y = (r.random(n) < 0.3).astype(np.float64)
    w = r.uniform(0.2, 3.0, n) if weighted else None
    dp, dx, logit, h1, h2 = _forward(p16, x16)
    g, l = _backward(dp, dx, h1, h2, logit, y, w, n)
    ref, lref = fo.backward(p16, x16, _host16(h1).astype(np.float64), _host16(h2).astype(np.float64),
                            logit.cpu().numpy().astype(np.float64), y, w)
    assert abs(l - lref) <= 1e-4 * abs(lref) + 1e-4
    for k, (o, s) in fo.OFF.items():
        a, b = g[o:o + int(np.prod(s))], ref[o:o + int(np.prod(s))]
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        assert err < 3e-3, (k, err)
    assert np.all(g[:128 * 80].reshape(128, 80)[:, 67:] == 0)


def test_gradients_accumulate_over_calls():
    n = 2048
    p16, x16 = _params(3), _x(n, 4)
    y = (np.arange(n) % 3 == 0).astype(np.float64)
    dp, dx, logit, h1, h2 = _forward(p16, x16)
    whole, _ = _backward(dp, dx, h1, h2, logit, y, None, n)
    half = n // 2
    parts = np.zeros_like(whole)
    for lo in (0, half):
        dpx, dxx, lx, h1x, h2x = _forward(p16, x16[lo:lo + half])
        g, _ = _backward(dpx, dxx, h1x, h2x, lx, y[lo:lo + half], None, half)
        parts += g
    np.testing.assert_allclose(parts, whole, rtol=1e-4, atol=1e-4)


def test_adam_step_matches_numpy():
    r = np.random.default_rng(9)
    p16 = _params(9)
    master = p16.astype(np.float32)
    g = r.normal(0, 1, fo.NPARAM).astype(np.float32)
    m = r.normal(0, 0.1, fo.NPARAM).astype(np.float32)
    v = r.uniform(0, 0.1, fo.NPARAM).astype(np.float32)
    dm, dmm, dv, dg = (torch.from_numpy(a.copy()).cuda() for a in (master, m, v, g))
    dp = _dev16(p16)
    lr, b1, b2, eps, scale, wd, step = 1e-3, 0.9, 0.999, 1e-8, 0.5, 1e-4, 3
    oic.mlp_adam(dm.data_ptr(), dmm.data_ptr(), dv.data_ptr(), dg.data_ptr(), dp.data_ptr(), lr, b1, b2, eps, scale,
                 wd, step)
    torch.cuda.synchronize()
    gs = g.astype(np.float64) * scale
    m2 = b1 * m + (1 - b1) * gs
    v2 = b2 * v + (1 - b2) * gs * gs
    w2 = master - lr * ((m2 / (1 - b1 ** step)) / (np.sqrt(v2 / (1 - b2 ** step)) + eps) + wd * master)
    np.testing.assert_allclose(dm.cpu().numpy(), w2, rtol=1e-5, atol=1e-6)
    assert np.all(_host16(dp) == dm.cpu().numpy().astype(np.float16))
    assert torch.count_nonzero(dg).item() == 0


def test_training_kernels_learn_a_separable_problem():
    r = np.random.default_rng(21)
    n = 40000
    x = r.normal(0, 1, (n, fo.IN))
    x[:, 67:] = 0
    u = r.normal(0, 1, 67)
    y = (x[:, :67] @ u + 0.5 * x[:, 0] * x[:, 1] > 0).astype(np.float32)
    X = torch.from_numpy(x.astype(np.float16)).cuda()
    tr = filter_train.Trainer(filter_train.init_params(1))
    hist = tr.fit(X, torch.from_numpy(y).cuda(), torch.ones(n, device="cuda"), epochs=8, batch=1024, lr=3e-3)
    assert hist[-1] < 0.5 * hist[0]
    acc = ((tr.predict(X).cpu().numpy() > 0) == (y > 0)).mean()
    assert acc > 0.95


@pytest.fixture(scope="module")
def small_c2(tmp_path_factory):
    """A 1 Mbp c2-like read set (4 repeat copies, tandem arrays, 30x 15 kb reads)."""
    d = str(tmp_path_factory.mktemp("filter_c2"))
    return d, workloads.generate("c2", d, scale=0.02, seed=7)


def test_feature_rows_match_the_oracle(small_c2):
    d, (db, skip) = small_c2
    lib, length, offset, bases = oic.read_seqdb(db)
    with oic.Overlapper(workloads.params("c2"), 0) as ov:
        ov.set_reads_seqdb(db)
        ov.set_skip_kmers(workloads.read_skip(skip))
        ov.collect_pairs(2)
        ov.run()
        info, feat, runs = ov.pairs(nodes=True)
    assert len(info) > 1000 and runs.shape[0] == int(info["nodes"].sum())
    start = np.concatenate([[0], np.cumsum(info["nodes"].astype(np.int64))])
    r = np.random.default_rng(0)
    pick = r.choice(len(info), size=min(3000, len(info)), replace=False)
    for i in pick:
        q = info[i]
        ref = fo.features(int(length[q["aID"] - 1]), int(length[q["bID"] - 1]), int(q["seeds"]),
                          runs[start[i]:start[i + 1]], 22)
        got = feat[i]
        assert np.array_equal(got[:64], ref[:64]), i
        np.testing.assert_allclose(got[64:67].astype(np.float32), ref[64:67].astype(np.float32), rtol=2e-3, atol=2e-3)
        assert np.all(got[67:] == 0)


def test_filtered_output_is_an_exact_subset(small_c2):
    d, (db, skip) = small_c2
    p16 = _params(5)

    def run(params, thr, collect=0):
        with oic.Overlapper(workloads.params("c2"), 0) as ov:
            ov.set_reads_seqdb(db)
            ov.set_skip_kmers(workloads.read_skip(skip))
            if params is not None:
                ov.set_filter(params, thr, domain=filter_train.training_domain("c2"))
            if collect:
                ov.collect_pairs(1)
            ov.run()
            return ov.overlaps(), ov.stats(), (ov.pairs()[0] if collect else None)

    plain, sp, _ = run(None, 0)
    same, s0, info0 = run(p16, 0.0, collect=1)
    assert np.array_equal(oic.sort_records(plain), oic.sort_records(same)) and s0["filteredPairs"] == 0
    assert s0["dpCells"] == sp["dpCells"]
    # a cut at the median score drops about half the pairs
    thr = float(1 / (1 + np.exp(-np.median(info0["score"]))))
    filt, sf, info = run(p16, thr, collect=1)
    dropped = (info["flags"] & 2) != 0
    assert sf["filteredPairs"] == int(dropped.sum()) > 0
    assert np.all(info["overlaps"][dropped] == 0) and np.all(info["cells"][dropped] == 0)
    recall, exact = filter_train.compare(plain, filt)
    assert exact and len(filt) <= len(plain)
    assert sf["dpCells"] <= sp["dpCells"]
    # the kept pairs' records are exactly the plain records of those pairs (a record
    # names the pair's reads in either order; flipped = the S strand)
    kept = set()
    for a_, b_, f_ in zip(info["aID"][~dropped].tolist(), info["bID"][~dropped].tolist(),
                          (info["flags"][~dropped] & 1).tolist()):
        kept.add((a_, b_, f_))
        kept.add((b_, a_, f_))
    want = [r for r in oic.sort_records(plain) if (int(r[0]), int(r[1]), int(r[2] >> 26) & 1) in kept]
    assert np.array_equal(oic.sort_records(filt), np.array(want, dtype=np.uint32).reshape(-1, 6))


def test_trained_filter_gains_over_the_plain_path(small_c2):
    path = os.path.join(ROOT, "canu_gb300", "filter_c2.npz")
    if not os.path.exists(path):
        pytest.skip("no trained filter")
    params, thr, full, meta = filter_train.load(path)
    assert "6" not in meta["train_seeds"].split(",")
    d, _ = small_c2
    ev = filter_train.evaluate(params, thr, "c2", seed=6, scale=0.05, workdir=d, full_threshold=full,
                               budget=meta["budget"])
    assert ev["records_exact"]
    assert ev["recall"] >= 0.995
    assert ev["dp_cells_skipped_frac"] > 0.3
    assert ev["filter"]["dp_cells"] < ev["plain"]["dp_cells"]


def test_filter_is_refused_outside_its_training_parameters(small_c2):
    """The shipped network was trained at -k 22 --minlength 1000 --maxerate 0.01 on
    0.5 %-error reads; on other parameters (here the smoke run's --maxerate 0.06
    --minlength 500) its scores mean nothing, so the library refuses it."""
    path = os.path.join(ROOT, "canu_gb300", "filter_c2.npz")
    params, thr, full, meta = filter_train.load(path)
    assert meta["domain"] == filter_train.training_domain("c2")
    d, (db, _) = small_c2
    for over in ({"maxErate": 0.06, "minOlapLen": 500}, {"maxErate": 0.06}, {"minOlapLen": 500}, {"kmerLen": 20}):
        with oic.Overlapper(workloads.params("c2", **over), 0) as ov:
            ov.set_reads_seqdb(db)
            with pytest.raises(oic.OicError) as e:
                ov.set_filter(params, thr, full, meta["budget"], domain=meta["domain"])
            assert e.value.code == oic.OIC_ERR_ARG and "trained for" in str(e.value)
            with pytest.raises(oic.OicError):
                ov.set_filter(params, thr, full, meta["budget"])          # no domain given
    with oic.Overlapper(workloads.params("c2"), 0) as ov:
        ov.set_reads_seqdb(db)
        ov.set_filter(params, thr, full, meta["budget"], domain=meta["domain"])   # its own parameters: accepted
