"""Degenerate and boundary inputs through the whole command line, against the CPU oracle:
no eligible ref read, reads of N only, a single read, identical and reverse-complement
reads, lower-case bases, reads shorter than k that are not in the length window, ranges
past the last read, a read at the maximum length the 21-bit fields hold."""
import os
import subprocess

import numpy as np
import pytest

import canu_gb300 as oic

pytestmark = pytest.mark.gpu

COMP = str.maketrans("ACGT", "TGCA")


def rand_seq(r, n):
    return "".join(r.choice(list("ACGT"), n))


def mutate(r, s, rate):
    out = []
    for c in s:
        x = r.random()
        if x < rate / 3:
            out.append(r.choice([b for b in "ACGT" if b != c]))
        elif x < 2 * rate / 3:
            continue
        elif x < rate:
            out.append(c)
            out.append(r.choice(list("ACGT")))
        else:
            out.append(c)
    return "".join(out)


def run_both(built, oracle, tmp, seqs, args):
    db = str(tmp / "in.seqdb")
    oic.write_seqdb(db, seqs)
    res = []
    for tool, name in ((built["cli"], "gpu"), (oracle["cli"], "port")):
        out = str(tmp / f"{name}.ovb")
        st = str(tmp / f"{name}.stats")
        r = subprocess.run([tool] + args + ["-o", out, "-s", st, db], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                           text=True)
        assert r.returncode == 0, (name, r.stderr[-2000:])
        raw = oic.read_ovb(out) if name == "gpu" else np.fromfile(out, dtype=np.uint32).reshape(-1, 6)
        rec = oic.sort_records(raw)
        res.append((rec, open(out[:-4] + ".oc", "rb").read(), open(st).read()))
    (g, goc, gst), (p, poc, pst) = res
    assert g.shape == p.shape and (g == p).all()
    assert goc == poc and gst == pst
    return g


ARGS = ["-t", "2", "-k", "22", "--hashbits", "16", "--maxerate", "0.06", "--minlength", "500"]


def test_no_read_reaches_the_minimum_length(built, oracle, tmp_path):
    r = np.random.default_rng(1)
    g = run_both(built, oracle, tmp_path, [rand_seq(r, 300) for _ in range(20)], ARGS + ["-h", "1-20", "-r", "1-20"])
    assert len(g) == 0


def test_reads_of_n_only(built, oracle, tmp_path):
    g = run_both(built, oracle, tmp_path, ["N" * 3000, "N" * 2500, "n" * 4000], ARGS + ["-h", "1-3", "-r", "1-3"])
    assert len(g) == 0


def test_single_read(built, oracle, tmp_path):
    r = np.random.default_rng(2)
    g = run_both(built, oracle, tmp_path, [rand_seq(r, 5000)], ARGS + ["-h", "1-1", "-r", "1-1"])
    assert len(g) == 0


def test_identical_reverse_complement_and_lower_case_reads(built, oracle, tmp_path):
    r = np.random.default_rng(3)
    genome = rand_seq(r, 20000)
    a = genome[2000:9000]
    seqs = [a, a, a[::-1].translate(COMP), a.lower(), mutate(r, genome[5000:12000], 0.02),
            mutate(r, genome[8000:15000], 0.02)[::-1].translate(COMP)]
    g = run_both(built, oracle, tmp_path, seqs, ARGS + ["-h", "1-6", "-r", "1-6"])
    assert len(g) >= 10


def test_ranges_past_the_last_read_are_clamped(built, oracle, tmp_path):
    r = np.random.default_rng(4)
    genome = rand_seq(r, 30000)
    seqs = [mutate(r, genome[s:s + 6000], 0.02) for s in range(0, 24000, 1500)]
    g = run_both(built, oracle, tmp_path, seqs, ARGS + ["-h", "1-1000", "-r", "3-5000"])
    assert len(g) > 0


def test_short_reads_below_k_outside_the_length_window(built, oracle, tmp_path):
    r = np.random.default_rng(5)
    genome = rand_seq(r, 30000)
    seqs = [mutate(r, genome[s:s + 5000], 0.02) for s in range(0, 24000, 1000)] + ["ACGT", "AC", rand_seq(r, 15)]
    n = len(seqs)
    g = run_both(built, oracle, tmp_path, seqs, ARGS + ["-h", f"1-{n}", "-r", f"1-{n}"])
    assert len(g) > 0


def test_maximum_read_length(built, oracle, tmp_path):
    """Two overlapping reads of 2^21 - 1 bases (AS_MAX_READLEN) and a short one: the
    21-bit hang and span fields at their limit."""
    r = np.random.default_rng(6)
    L = (1 << 21) - 1
    genome = rand_seq(r, L + 40000)
    seqs = [genome[:L], genome[40000:40000 + L], genome[100000:120000]]
    args = ["-t", "2", "-k", "22", "--hashbits", "22", "--maxerate", "0.01", "--minlength", "1000",
            "--hashdatalen", "10000000", "-h", "1-3", "-r", "1-3"]
    g = run_both(built, oracle, tmp_path, seqs, args)
    assert len(g) >= 2
