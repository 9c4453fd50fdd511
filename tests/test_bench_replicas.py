"""bench.py's replica arithmetic across ranks, on CPU with a gloo process group
(world size 2): the whole-job rate is every rank's units over the slowest rank's time."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, ROOT)
    import torch.distributed as td
    import bench
    td.init_process_group("gloo", rank=rank, world_size=ws)
    seconds = [2.0, 5.0][rank]
    out[rank] = (bench.barrier_max(seconds, ws, "cpu"), bench.replica_rate(1000, seconds, ws, "cpu"))
    td.barrier()
    td.destroy_process_group()


def test_replica_rate_uses_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        mx, rate = out[r]
        assert mx == 5.0
        assert rate == 2 * 1000 / 5.0


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.barrier_max(3.0, 1) == 3.0
    assert bench.replica_rate(500, 2.0, 1) == 250.0


def test_workload_text_says_when_the_skip_list_is_left_out():
    """A run without its skip list is labelled as the configuration as written, so its
    line cannot be mistaken for the skip-list run; workloads without a list are unchanged."""
    import argparse
    sys.path.insert(0, ROOT)
    import bench
    for wl in ("c2", "c5"):
        with_list = bench.workload_text(argparse.Namespace(workload=wl, no_skip_list=False))
        without = bench.workload_text(argparse.Namespace(workload=wl, no_skip_list=True))
        assert "frequent-k-mer skip list" in with_list and "no frequent-k-mer skip list" not in with_list
        assert without.endswith("no frequent-k-mer skip list (the configuration as written)")
        assert without.startswith(wl + ":")
    c1 = bench.workload_text(argparse.Namespace(workload="c1", no_skip_list=False))
    assert c1 == bench.WORKLOAD_TEXT["c1"]


def test_both_arms_describe_the_job_with_the_same_config(tmp_path):
    """The reference arm and the GPU arm build `config` with the same function, from the
    read container's header and the arguments: same keys, same values."""
    import argparse
    sys.path.insert(0, ROOT)
    import bench
    import canu_gb300 as oic
    db = str(tmp_path / "r.seqdb")
    oic.write_seqdb(db, ["ACGT" * 50, "GATTACA" * 30, "T" * 7])
    a = argparse.Namespace(workload="c2", no_skip_list=False, scale=0.5)
    c = bench.job_config(a, db, 2)
    assert c == {"workload": bench.WORKLOAD_TEXT["c2"], "scale": 0.5, "reads": 3, "bases": 200 + 210 + 7,
                 "parallelism": "replicas2", "l2": bench.L2_NOTE}
