"""Bit-exactness at the benchmark configurations' shapes: the drop-in command line on the
GPU against the oracle's command line, same flags, same reads -- every record, the .oc
counts and the -s stats.

  c1  in full: 5 Mbp genome, 20x lognormal 8 kb reads, 2 % errors, --maxerate 0.06,
      one hash block, every ref read;
  c3  shape at 1/4 scale (Pareto 0.5-100 kb reads, 5 % errors, --maxerate 0.12, the CTA
      DP bin) with --hashdatalen cut so that the reads need several hash blocks, a
      contiguous slice of ref reads against every block;
  c5  shape at 1/20 scale (repeat families, tandem arrays, skip list, 40x HiFi-like
      reads) with four hash blocks, a slice of ref reads against every block.

Both sides get the same -t (it decides which ref reads a chunked run visits,
overlapInCore.C:225); the oracle uses that many host threads."""
import os
import subprocess

import numpy as np
import pytest

import canu_gb300 as oic
from canu_gb300 import workloads

pytestmark = pytest.mark.gpu
THREADS = str(max(2, min(16, os.cpu_count() or 2)))


def args_for(name, db, skip, refs=None, hashdatalen=None):
    a = workloads.cli_args(name, db, skip)
    a[a.index("-t") + 1] = THREADS
    if refs:
        a[a.index("-r") + 1] = refs
    if hashdatalen:
        a[a.index("--hashdatalen") + 1] = str(hashdatalen)
    return a


def run_both(built, oracle, tmp, db, args):
    out = {}
    for tool, tag in ((built["cli"], "gpu"), (oracle["cli"], "port")):
        ovb, st = str(tmp / f"{tag}.ovb"), str(tmp / f"{tag}.stats")
        r = subprocess.run([tool] + args + ["-o", ovb, "-s", st, db], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                           text=True)
        assert r.returncode == 0, (tag, r.stderr[-3000:])
        raw = oic.read_ovb(ovb) if tag == "gpu" else np.fromfile(ovb, dtype=np.uint32).reshape(-1, 6)
        out[tag] = (oic.sort_records(raw), open(str(tmp / f"{tag}.oc"), "rb").read(), open(st).read(), r.stderr)
    g, p = out["gpu"], out["port"]
    assert g[0].shape == p[0].shape, (g[0].shape, p[0].shape)
    assert (g[0] == p[0]).all(), "records differ"
    assert g[1] == p[1], ".oc differs"
    assert g[2] == p[2], (g[2], p[2])
    return g[0], p[3].count("oic_port: hash block")


def test_c1_in_full_matches_the_oracle(built, oracle, tmp_path_factory):
    d = tmp_path_factory.mktemp("c1")
    db, skip = workloads.generate("c1", str(d))
    rec, blocks = run_both(built, oracle, d, db, args_for("c1", db, skip))
    assert len(rec) > 200000 and blocks == 1


def test_c3_shape_slice_over_several_blocks_matches_the_oracle(built, oracle, tmp_path_factory):
    d = tmp_path_factory.mktemp("c3")
    db, skip = workloads.generate("c3", str(d), scale=0.25)
    n = len(oic.read_seqdb(db)[1])
    a = args_for("c3", db, skip, refs=f"{n // 2}-{n // 2 + 199}", hashdatalen=40_000_000)
    rec, blocks = run_both(built, oracle, d, db, a)
    assert len(rec) > 1000 and blocks >= 3


def test_c5_shape_slice_over_four_blocks_matches_the_oracle(built, oracle, tmp_path_factory):
    d = tmp_path_factory.mktemp("c5")
    db, skip = workloads.generate("c5", str(d), scale=0.05)
    lens = oic.read_seqdb(db)[1]
    n = len(lens)
    hdl = int(lens.sum()) // 4 + 1_000_000     # four hash blocks
    a = args_for("c5", db, skip, refs=f"{n // 3}-{n // 3 + 299}", hashdatalen=hdl)
    rec, blocks = run_both(built, oracle, d, db, a)
    assert len(rec) > 1000 and blocks == 4
