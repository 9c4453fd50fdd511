"""The synthetic read generator and the read container."""
import subprocess

import numpy as np

import canu_gb300 as oic
from conftest import sha256


def test_generator_is_deterministic(built, tmp_path):
    a, b = str(tmp_path / "a.seqdb"), str(tmp_path / "b.seqdb")
    for p in (a, b):
        subprocess.run([built["synth"], "--genome", "20000", "--coverage", "5", "--seed", "7", "--out", p], check=True,
                       stderr=subprocess.DEVNULL)
    assert sha256(a) == sha256(b)


def test_generator_shapes(built, tmp_path):
    p = str(tmp_path / "c.seqdb")
    subprocess.run([built["synth"], "--genome", "200000", "--coverage", "10", "--len-mean", "5000", "--len-sd", "1000",
                    "--len-min", "1000", "--len-max", "9000", "--seed", "3", "--out", p], check=True,
                   stderr=subprocess.DEVNULL)
    lib, ln, off, bases = oic.read_seqdb(p)
    assert ln.sum() >= 0.95 * 10 * 200000
    assert 4000 < ln.mean() < 6000
    assert set(np.unique(bases).tolist()) <= set(b"ACGT")


def test_seqdb_roundtrip(tmp_path):
    p = str(tmp_path / "r.seqdb")
    oic.write_seqdb(p, ["ACGT", "NNAC", "a"], libs=[1, 2, 3])
    lib, ln, off, bases = oic.read_seqdb(p)
    assert lib.tolist() == [1, 2, 3] and ln.tolist() == [4, 4, 1] and off.tolist() == [0, 4, 8]
    assert bytes(bases) == b"ACGTNNACa"
