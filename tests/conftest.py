"""Shared fixtures: build steps, golden cases, the CPU oracle."""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def sha256(path):
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for blk in iter(lambda: f.read(1 << 20), b""):
            h.update(blk)
    return h.hexdigest()


@pytest.fixture(scope="session")
def built():
    """liboic_gpu.so, overlapInCore and oic_synth (cross-compiled; no GPU needed)."""
    from canu_gb300.build import build_lib, build_tools
    lib = build_lib()
    cli, synth = build_tools()
    return {"lib": lib, "cli": cli, "synth": synth}


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (oracle/oic_port.c): CLI and shared library."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    return {"cli": os.path.join(ROOT, "oracle", "_build", "oic_port"),
            "lib": os.path.join(ROOT, "oracle", "_build", "liboic_port.so")}


def golden_cases():
    with open(os.path.join(GOLDEN, "cases.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_inputs(built, tmp_path_factory):
    """Regenerate every golden case's inputs; check them against the stored digests."""
    d = tmp_path_factory.mktemp("golden_inputs")
    out = {}
    for name, c in golden_cases().items():
        db = str(d / (name + ".seqdb"))
        skip = str(d / (name + ".skip"))
        args = [built["synth"]] + c["synth"].split() + ["--out", db]
        if c["skip_sha256"]:
            args += ["--skip-out", skip]
        subprocess.run(args, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        assert sha256(db) == c["seqdb_sha256"], f"{name}: regenerated reads differ from the fixture's"
        if c["skip_sha256"]:
            assert sha256(skip) == c["skip_sha256"], f"{name}: regenerated skip list differs"
        out[name] = {"db": db, "skip": skip if c["skip_sha256"] else None, "args": c["args"]}
    return out


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return z["records"], bytes(z["oc"]), bytes(z["stats"]).decode()


def run_cli(binary, args_template, db, skip, workdir, extra=()):
    """Run the drop-in CLI (snappy-framed .ovb, as canu's ovFile writes) or the oracle's
    CLI (the same records unframed); returns (sorted records, .oc bytes, stats, log)."""
    out = os.path.join(workdir, "out.ovb")
    stats = os.path.join(workdir, "out.stats")
    args = args_template.format(db=db, skip=skip or "").split()
    r = subprocess.run([binary] + args + list(extra) + ["-o", out, "-s", stats], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    from canu_gb300 import read_ovb, sort_records
    framed = os.path.basename(binary) == "overlapInCore"
    rec = sort_records(read_ovb(out) if framed else np.fromfile(out, dtype=np.uint32).reshape(-1, 6))
    oc = open(os.path.join(workdir, "out.oc"), "rb").read()
    st = open(stats).read()
    return rec, oc, st, r.stderr
