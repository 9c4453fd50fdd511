"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer (CPU only).

The parts of this project that run on the host's CPU -- the CPU oracle
(oracle/oic_port.c), the library's output-file code (canu_gb300/host/oic_ovfile.cpp:
.ovb / .oc / snappy / merge / overlap-store writer) and the read generator
(canu_gb300/synth/oic_synth.cpp) -- are rebuilt with -fsanitize=address,undefined and
run on the golden cases' inputs: every run must exit cleanly with no sanitizer report
and produce exactly the unsanitized results (the golden records, .oc and stats; the
fixtures' read digests)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_cases, load_golden, run_cli, sha256

SAN = ["-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined"]
ENV = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")


@pytest.fixture(scope="module")
def san_dir(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("sanitized"))
    probe = os.path.join(d, "probe.c")
    open(probe, "w").write("int main(void) { return 0; }\n")
    if not shutil.which("gcc") or subprocess.run(["gcc"] + SAN + [probe, "-o", probe + ".x"]).returncode != 0:
        pytest.skip("no sanitizer runtime for gcc here")
    return d


def build(cmd, out):
    r = subprocess.run(cmd + ["-o", out], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-3000:]
    return out


def clean(log):
    return "runtime error" not in log and "Sanitizer" not in log


@pytest.fixture(scope="module")
def oracle_san(san_dir):
    o = os.path.join(ROOT, "oracle")
    return build(["gcc", "-std=gnu11", "-fopenmp", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include")] + SAN +
                 [os.path.join(o, "oic_port_main.c"), os.path.join(o, "oic_port.c"), "-lm"],
                 os.path.join(san_dir, "oic_port"))


@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_oracle_under_sanitizers_reproduces_the_golden_case(name, oracle_san, golden_inputs, tmp_path):
    g = golden_inputs[name]
    old = os.environ.copy()
    os.environ.update(ENV)
    try:
        rec, oc, st, log = run_cli(oracle_san, g["args"], g["db"], g["skip"], str(tmp_path))
    finally:
        os.environ.clear()
        os.environ.update(old)
    assert clean(log), log[-3000:]
    grec, goc, gst = load_golden(name)
    from canu_gb300 import sort_records
    grec = sort_records(grec)
    assert rec.shape == grec.shape and (rec == grec).all()
    assert oc == bytes(goc) and st == gst


def test_host_file_code_under_sanitizers(san_dir, tmp_path):
    exe = build(["g++", "-std=c++17", "-I" + os.path.join(ROOT, "include")] + SAN +
                [os.path.join(ROOT, "tests", "host_sanitize_main.cpp"),
                 os.path.join(ROOT, "canu_gb300", "host", "oic_ovfile.cpp")], os.path.join(san_dir, "host_check"))
    r = subprocess.run([exe, str(tmp_path)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=ENV)
    assert r.returncode == 0 and clean(r.stderr), r.stderr[-3000:]
    assert "all checks passed" in r.stdout


def test_read_generator_under_sanitizers(san_dir, tmp_path):
    exe = build(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include")] + SAN[1:] +
                [os.path.join(ROOT, "canu_gb300", "synth", "oic_synth.cpp")], os.path.join(san_dir, "oic_synth"))
    for name in ("default", "skip", "n_libs_minkmers"):
        c = golden_cases()[name]
        db, skip = str(tmp_path / (name + ".seqdb")), str(tmp_path / (name + ".skip"))
        args = [exe] + c["synth"].split() + ["--out", db] + (["--skip-out", skip] if c["skip_sha256"] else [])
        r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=ENV)
        assert r.returncode == 0 and clean(r.stderr), r.stderr[-3000:]
        assert sha256(db) == c["seqdb_sha256"]
        if c["skip_sha256"]:
            assert sha256(skip) == c["skip_sha256"]


def test_read_importer_under_sanitizers(san_dir, tmp_path):
    """oic_seqdb_import on well-formed, wrapped, mixed-case and malformed FASTA / FASTQ."""
    exe = build(["g++", "-std=c++17", "-I" + os.path.join(ROOT, "include")] + SAN +
                [os.path.join(ROOT, "canu_gb300", "host", "oic_seqdb_import.cpp")], os.path.join(san_dir, "imp"))
    good = tmp_path / "g.fa"
    good.write_bytes(b">a x\r\nacgtRYKM\r\n\r\n>b\n" + b"ACGT" * 5000 + b"\n>c\n\n")
    fq = tmp_path / "g.fq"
    fq.write_text("@q1\nACGT\nAC\n+\n@@@@\nII\n@q2\nNNNN\n+\n####\n")
    r = subprocess.run([exe, "-o", str(tmp_path / "o.seqdb"), str(good), str(fq)], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, env=ENV)
    assert r.returncode == 0 and clean(r.stderr), r.stderr[-3000:]
    for content in ("@q\nACGT\n+\nII\n", "@q\nAC", ">", "xyz\n", ""):
        bad = tmp_path / "bad.fq"
        bad.write_text(content)
        r = subprocess.run([exe, "-o", str(tmp_path / "b.seqdb"), str(bad)], stdout=subprocess.PIPE,
                           stderr=subprocess.PIPE, text=True, env=ENV)
        assert r.returncode in (0, 1) and clean(r.stderr), (content, r.stderr[-3000:])
