"""The CTA-bin DP -- speculative (every warp of the CTA extends one of the pair's next
match nodes, replayed in the reference's order) and CTA-wide rows (several warps per
row, U diagonals per thread) -- and the autotuner: same alignments as the oracle, same
records as the reference."""
import ctypes
import os

import numpy as np
import pytest

import canu_gb300 as oic
from conftest import golden_cases, golden_inputs, load_golden, run_cli  # noqa: F401
from test_gpu_extend import make_problems, port_aligner

pytestmark = pytest.mark.gpu

SMALL_ARENA = 1 << 22   # keeps the tests' CTA-bin scratch small


@pytest.mark.parametrize("threads,tile", [(64, 1), (128, 2), (256, 4), (512, 1)])
@pytest.mark.parametrize("case,erate,partial", [("default", 0.06, 0), ("hierr", 0.12, 0), ("hierr_partial", 0.12, 1)])
def test_cta_dp_matches_oracle(threads, tile, case, erate, partial, built, oracle, golden_inputs):
    rng = np.random.default_rng(11)
    db = golden_inputs[case]["db"]
    seqs, probs = make_problems(db, 200, rng)
    erate = float(np.float32(erate))
    with oic.Overlapper(oic.default_params(kmerLen=22, maxErate=erate, partial=partial)) as ov:
        ov.set_reads_seqdb(db)
        ov.set_tuning(forceWide=1, wideThreads=threads, wideTile=tile, wideArena=SMALL_ARENA, wideCtas=64)
        assert ov.tuning()["wideThreads"] == threads
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


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_cta_bin_matches_reference(name, mode, built, golden_inputs, tmp_path):
    """Every pair through the CTA bin (1 speculative, 2 CTA-wide rows): records, .oc and
    stats equal the reference's."""
    g = golden_inputs[name]
    tune = f"forceWide=1,wideMode={mode},wideThreads=128,wideTile=2,wideArena={SMALL_ARENA},wideCtas=64"
    rec, oc, st, log = run_cli(built["cli"], g["args"], g["db"], g["skip"], str(tmp_path), extra=["--gpu-tune", tune])
    grec, goc, gst = load_golden(name)
    assert rec.shape == grec.shape, log[-2000:]
    assert (rec == grec).all()
    assert oc == goc
    assert st == gst


def test_length_bin_and_small_one_warp_arena_keep_records(built, golden_inputs, tmp_path):
    """A length-bin boundary inside the read-length range and a one-warp arena small
    enough to overflow move pairs between bins without changing a record."""
    name = "hierr"
    g = golden_inputs[name]
    tune = f"wideMinLen=6000,narrowArena=65536,wideThreads=256,wideTile=4,wideArena={SMALL_ARENA},wideCtas=64"
    rec, oc, st, log = run_cli(built["cli"], g["args"], g["db"], g["skip"], str(tmp_path), extra=["--gpu-tune", tune])
    grec, goc, gst = load_golden(name)
    assert (rec == grec).all() and oc == goc and st == gst
    import re
    m = re.search(r"CTA (\d+) pairs", log)
    assert m and int(m.group(1)) > 0, log[-1000:]


def test_autotune_reports_the_grid_and_keeps_records(built, golden_inputs):
    g = golden_inputs["hierr"]
    db = g["db"]
    n = len(oic.read_seqdb(db)[1])
    p = oic.default_params(kmerLen=22, maxErate=0.12, minOlapLen=500, hashBits=22)

    def run(tuned):
        with oic.Overlapper(p) as ov:
            ov.set_reads_seqdb(db)
            ov.set_tuning(wideArena=SMALL_ARENA, wideCtas=64)
            lines = None
            if tuned:
                ov.load_hash_block(1, n)
                lines = ov.autotune(1, min(n, 400))
            ov.load_hash_block(1, n)
            ov.run_refs(1, n)
            return oic.sort_records(ov.overlaps()), lines, ov.tuning()

    base, _, _ = run(False)
    recs, lines, tun = run(True)
    assert len(lines) == 17     # speculative, 4 warps-per-pair x 3 tiles of CTA rows, then 4 length bins
    assert lines[0]["wideTile"] == 0
    assert {(l["wideThreads"], l["wideTile"]) for l in lines[1:13]} == {(t, u) for t in (64, 128, 256, 512)
                                                                         for u in (1, 2, 4)}
    best = min(lines, key=lambda l: l["msTotal"])
    if best["wideTile"] == 0:
        assert tun["wideMode"] == 1
    else:
        assert tun["wideMode"] == 2 and tun["wideThreads"] == best["wideThreads"] and tun["wideTile"] == best["wideTile"]
    assert np.array_equal(recs, base)


@pytest.mark.parametrize("name", ["hierr", "hierr_partial", "multi", "repeats_noskip"])
def test_speculative_bin_counts_only_the_reference_extensions(name, built, golden_inputs):
    """Extensions whose node an earlier extension of the same round removed are
    discarded: the speculative CTA bin reports exactly the DP work of the sequential
    loop (extensions, DP cells, rows, slide bases) and the same records."""
    g = golden_inputs[name]
    args = g["args"].format(db=g["db"], skip=g["skip"] or "").split()

    def opt(flag, default=None):
        return args[args.index(flag) + 1] if flag in args else default
    kw = dict(kmerLen=22, hashBits=16, maxHashLoad=0.8, maxErate=float(opt("--maxerate")),
              minOlapLen=int(opt("--minlength")), partial=int("-partial" in args),
              uniqueOlapPerPair=0 if "-m" in args else 1, numThreads=int(opt("-t")))
    out = []
    for mode in (1, 2):
        with oic.Overlapper(oic.default_params(**kw)) as ov:
            ov.set_reads_seqdb(g["db"])
            ov.set_tuning(forceWide=1, wideMode=mode, wideArena=SMALL_ARENA, wideCtas=64)
            ov.run()
            out.append((oic.sort_records(ov.overlaps()), ov.stats()))
    (ra, sa), (rb, sb) = out
    assert len(ra) > 0 and np.array_equal(ra, rb)
    for k in ("extensions", "dpCells", "dpRows", "slideBases", "totalOverlaps", "kmerHitsWithOlap"):
        assert sa[k] == sb[k], (k, sa[k], sb[k])


def test_captured_graph_matches_kernel_by_kernel(built, tmp_path_factory):
    """The DP stage relaunched as one captured CUDA graph gives the records and counters
    of the kernel-by-kernel launch, with and without the learned filter."""
    import os
    from canu_gb300 import filter_train, workloads
    d = str(tmp_path_factory.mktemp("graph"))
    db, skip = workloads.generate("c2", d, scale=0.02, seed=7)
    fpath = os.path.join(os.path.dirname(oic.__file__), "filter_c2.npz")
    params, thr, full, meta = filter_train.load(fpath)

    def run(no_graph, filt):
        with oic.Overlapper(workloads.params("c2")) as ov:
            ov.set_reads_seqdb(db)
            ov.set_skip_kmers(workloads.read_skip(skip))
            ov.set_tuning(noGraph=no_graph, wideArena=SMALL_ARENA, wideCtas=64)
            if filt:
                ov.set_filter(params, thr, full, meta["budget"], domain=meta["domain"])
            ov.run()
            return oic.sort_records(ov.overlaps()), ov.stats()

    for filt in (False, True):
        a, sa = run(0, filt)
        b, sb = run(1, filt)
        assert len(a) > 1000 and np.array_equal(a, b)
        for k in ("dpCells", "extensions", "kmerHitsWithOlap", "kmerHitsWithoutOlap", "filteredPairs", "slideBases"):
            assert sa[k] == sb[k], k
        assert sa["graphLaunches"] > 0 and sb["graphLaunches"] == 0
