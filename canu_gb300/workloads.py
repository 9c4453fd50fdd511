"""The benchmark read sets and overlapInCore settings.

Each workload is a seeded oic_synth invocation plus the overlapInCore parameters it is
run with.  Sizes follow the benchmark configurations of the overlap stage:

  c1  5 Mbp iid genome, 20x lognormal reads (mean 8 kb, sd 3 kb, 1-30 kb), 2% errors
      (sub:ins:del 1:1:1), k=22, --minlength 500, --maxerate 0.06, one hash block
  c2  50 Mbp genome with 200 copies of a 6 kb repeat (1% per-copy divergence) and 2%
      tandem arrays of a 171 bp unit (2% divergence); 30x HiFi-like reads (normal,
      mean 15 kb, sd 3 kb), 0.5% errors, k=22, --minlength 1000, --maxerate 0.01,
      --hashbits 25, --hashdatalen 1.6 Gbp; with a frequent-k-mer skip list (k-mers of
      genome multiplicity > 10, i.e. read count > 10x coverage).  Seed 6: the learned
      filter trains on seeds 1-5 of this shape and is evaluated on seed 6.
  c3  20 Mbp iid genome, 25x Pareto reads (alpha 1.5, min 500, cap 100 kb), 5% errors
      (1:2:2), --minlength 500, --maxerate 0.12, --hashbits 24
  c5  200 Mbp genome with 1000 x 6 kb repeats and 3% tandem arrays, 40x c2-like reads,
      --hashbits 27, --hashdatalen 2 Gbp (several hash blocks)

`scale` shrinks the genome (and the repeat copy count with it) for quick runs.
"""
import os
import subprocess

import numpy as np

from . import BUILD, default_params

WORKLOADS = {
    "c1": dict(
        synth=dict(genome=5_000_000, coverage=20, len_dist="lognormal", len_mean=8000, len_sd=3000, len_min=1000,
                   len_max=30000, err=0.02, ratio="1:1:1", seed=1),
        params=dict(kmerLen=22, hashBits=23, maxHashLoad=0.8, maxErate=0.06, minOlapLen=500,
                    maxHashDataLen=110_000_000, numThreads=8),
        skip=False),
    "c2": dict(
        synth=dict(genome=50_000_000, coverage=30, len_dist="normal", len_mean=15000, len_sd=3000, len_min=1000,
                   len_max=30000, err=0.005, ratio="1:1:1", repeat_copies=200, repeat_len=6000, repeat_div=0.01,
                   tandem_frac=0.02, tandem_unit=171, tandem_div=0.02, seed=6),
        params=dict(kmerLen=22, hashBits=25, maxErate=0.01, minOlapLen=1000, maxHashDataLen=1_600_000_000,
                    numThreads=8),
        skip=True, skip_min_count=11),
    "c3": dict(
        synth=dict(genome=20_000_000, coverage=25, len_dist="pareto", pareto_alpha=1.5, len_min=500, len_max=100000,
                   err=0.05, ratio="1:2:2", seed=3),
        params=dict(kmerLen=22, hashBits=24, maxErate=0.12, minOlapLen=500, maxHashDataLen=600_000_000,
                    numThreads=8),
        skip=False),
    "c5": dict(
        synth=dict(genome=200_000_000, coverage=40, len_dist="normal", len_mean=15000, len_sd=3000, len_min=1000,
                   len_max=30000, err=0.005, ratio="1:1:1", repeat_copies=1000, repeat_len=6000, repeat_div=0.01,
                   tandem_frac=0.03, tandem_unit=171, tandem_div=0.02, seed=5),
        params=dict(kmerLen=22, hashBits=27, maxErate=0.01, minOlapLen=1000, maxHashDataLen=2_000_000_000,
                    numThreads=8),
        skip=True, skip_min_count=11),
}


def synth_args(spec, scale=1.0, seed=None):
    s = dict(spec)
    if seed is not None:
        s["seed"] = seed
    if scale != 1.0:
        s["genome"] = int(s["genome"] * scale)
        if "repeat_copies" in s:
            s["repeat_copies"] = max(1, int(round(s["repeat_copies"] * scale)))
    args = []
    for k, v in s.items():
        args += ["--" + k.replace("_", "-"), str(v)]
    return args


def generate(name, outdir, scale=1.0, seed=None):
    """Generate (or reuse) a workload's reads; returns (seqdb path, skip path or None)."""
    w = WORKLOADS[name]
    os.makedirs(outdir, exist_ok=True)
    tag = f"{name}_s{seed if seed is not None else w['synth']['seed']}_x{scale:g}"
    db = os.path.join(outdir, tag + ".seqdb")
    skip = os.path.join(outdir, tag + ".skip") if w.get("skip") else None
    if not os.path.exists(db) or (skip and not os.path.exists(skip)):
        cmd = [os.path.join(BUILD, "oic_synth")] + synth_args(w["synth"], scale, seed) + ["--out", db + ".tmp"]
        if skip:
            cmd += ["--skip-out", skip + ".tmp", "--skip-min-count", str(w["skip_min_count"])]
        subprocess.run(cmd, check=True, stderr=subprocess.DEVNULL)
        if skip:
            os.replace(skip + ".tmp", skip)
        os.replace(db + ".tmp", db)
    return db, skip


def params(name, **over):
    p = dict(WORKLOADS[name]["params"])
    p.update(over)
    return default_params(**p)


def read_skip(path):
    """The k-mers of a skip file (one per line, the first token; '>' lines skipped)."""
    out = []
    with open(path) as f:
        for line in f:
            if line.startswith(">"):
                continue
            t = line.split()
            if t:
                out.append(t[0])
    return out


def cli_args(name, db, skip=None):
    """overlapInCore command-line arguments for a workload (all reads in -h and -r)."""
    from . import read_seqdb
    p = WORKLOADS[name]["params"]
    n = len(read_seqdb(db)[1])
    a = ["-t", str(p["numThreads"]), "-k", str(p["kmerLen"])]
    if skip:
        a += ["-k", skip]
    a += ["--hashbits", str(p["hashBits"]), "--maxerate", str(p["maxErate"]), "--minlength", str(p["minOlapLen"]),
          "--hashdatalen", str(p["maxHashDataLen"]), "-h", f"1-{n}", "-r", f"1-{n}"]
    if "maxHashLoad" in p:
        a += ["--hashload", str(p["maxHashLoad"])]
    return a
