"""Generate the golden fixtures of the overlap path from canu's own sources.

The fixtures pin both the CPU oracle (oracle/oic_port.c) and the CUDA path to the
reference: each case is a seeded synthetic read set (regenerated from its oic_synth
arguments; the SHA-256 of the container is stored to catch drift) plus the outputs of
canu's overlapInCore compiled from the reference tree (oracle/Makefile.ref): the sorted
overlap records, the .oc counts and the stats file.

    python tests/golden/make_golden.py [--ref /path/to/canu]

Writes tests/golden/<case>.npz and tests/golden/cases.json.

The -partial cases run the reference single-threaded: with more threads its
Output_Partial_Overlap increments the global overlap counter outside the critical
section (overlapInCore-Output.C:204), so the "Total overlaps produced" line of its
stats file can lose counts; the records themselves are unaffected.
"""
import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# name -> (oic_synth arguments, overlapInCore arguments with {db} and {skip} placeholders)
BASE = "-k 22 --hashbits 16 --hashload 0.8"
CASES = {
    "default": ("--genome 60000 --coverage 10 --len-mean 4000 --len-sd 1500 --len-min 500 --len-max 12000 --err 0.02 --seed 11",
                f"-t 4 {BASE} --maxerate 0.06 --minlength 500 -h 1-10000 -r 1-10000 {{db}}"),
    "partial": ("--genome 60000 --coverage 10 --len-mean 4000 --len-sd 1500 --len-min 500 --len-max 12000 --err 0.02 --seed 11",
                f"-t 1 -partial {BASE} --maxerate 0.06 --minlength 500 -h 1-10000 -r 1-10000 {{db}}"),
    "multi": ("--genome 60000 --coverage 10 --len-mean 4000 --len-sd 1500 --len-min 500 --len-max 12000 --err 0.02 --seed 12",
              f"-t 4 -m {BASE} --maxerate 0.06 --minlength 500 -h 1-10000 -r 1-10000 {{db}}"),
    "skip": ("--genome 80000 --coverage 10 --len-mean 4000 --len-sd 1500 --len-min 500 --len-max 12000 --err 0.01 "
             "--repeat-copies 8 --repeat-len 2000 --repeat-div 0.01 --tandem-frac 0.04 --tandem-div 0.02 "
             "--skip-min-count 4 --seed 13",
             f"-t 4 {BASE} -k {{skip}} --maxerate 0.06 --minlength 500 -h 1-10000 -r 1-10000 {{db}}"),
    "skip_z": ("--genome 80000 --coverage 10 --len-mean 4000 --len-sd 1500 --len-min 500 --len-max 12000 --err 0.01 "
               "--repeat-copies 8 --repeat-len 2000 --repeat-div 0.01 --tandem-frac 0.04 --tandem-div 0.02 "
               "--skip-min-count 4 --seed 13",
               f"-t 4 -z {BASE} -k {{skip}} --maxerate 0.06 --minlength 500 -h 1-10000 -r 1-10000 {{db}}"),
    "repeats_noskip": ("--genome 80000 --coverage 10 --len-mean 4000 --len-sd 1500 --len-min 500 --len-max 12000 --err 0.01 "
                       "--repeat-copies 8 --repeat-len 2000 --repeat-div 0.01 --tandem-frac 0.04 --tandem-div 0.02 --seed 14",
                       f"-t 4 {BASE} --maxerate 0.06 --minlength 500 -h 1-10000 -r 1-10000 {{db}}"),
    "blocks": ("--genome 60000 --coverage 10 --len-mean 4000 --len-sd 1500 --len-min 500 --len-max 12000 --err 0.02 --seed 15",
               f"-t 8 -k 22 --hashbits 16 --hashload 0.8 --hashdatalen 120000 --maxerate 0.06 --minlength 500 "
               f"-h 5-140 -r 20-150 {{db}}"),
    "entry_limit": ("--genome 60000 --coverage 10 --len-mean 4000 --len-sd 1500 --len-min 500 --len-max 12000 --err 0.02 --seed 16",
                    f"-t 2 -k 22 --hashbits 12 --hashload 0.5 --maxerate 0.06 --minlength 500 -h 1-10000 -r 1-10000 {{db}}"),
    "hierr": ("--genome 60000 --coverage 10 --len-dist pareto --len-min 500 --len-max 20000 --err 0.05 --ratio 1:2:2 --seed 17",
              f"-t 4 {BASE} --maxerate 0.12 --minlength 500 -h 1-10000 -r 1-10000 {{db}}"),
    "hierr_partial": ("--genome 60000 --coverage 10 --len-dist pareto --len-min 500 --len-max 20000 --err 0.05 --ratio 1:2:2 --seed 17",
                      f"-t 1 -partial {BASE} --maxerate 0.12 --minlength 500 -h 1-10000 -r 1-10000 {{db}}"),
    "hifi": ("--genome 80000 --coverage 12 --len-dist normal --len-mean 6000 --len-sd 1500 --len-min 1000 --len-max 20000 "
             "--err 0.005 --seed 18",
             f"-t 4 {BASE} --maxerate 0.01 --minlength 1000 -h 1-10000 -r 1-10000 {{db}}"),
    "n_libs_minkmers": ("--genome 60000 --coverage 10 --len-mean 4000 --len-sd 1500 --len-min 500 --len-max 12000 --err 0.02 "
                        "--n-rate 0.003 --libs 3 --seed 19",
                        f"-t 4 --minkmers {BASE} --maxerate 0.06 --minlength 500 -H 1-2 -R 2-3 -h 1-10000 -r 1-10000 {{db}}"),
    "noise": ("--genome 60000 --coverage 10 --len-mean 4000 --len-sd 1500 --len-min 500 --len-max 12000 --err 0.03 --seed 20",
              f"-t 4 {BASE} --maxerate 0.045 --alignnoise 1.3 --minlength 400 -h 1-10000 -r 1-10000 {{db}}"),
}


def sha256(path):
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for blk in iter(lambda: f.read(1 << 20), b""):
            h.update(blk)
    return h.hexdigest()


def make_inputs(synth, synth_args, tmp, name):
    db = os.path.join(tmp, name + ".seqdb")
    skip = os.path.join(tmp, name + ".skip")
    args = [synth] + synth_args.split() + ["--out", db]
    if "--skip-min-count" in synth_args:
        args += ["--skip-out", skip]
    subprocess.run(args, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return db, (skip if os.path.exists(skip) else None)


def oic_args(template, db, skip):
    return template.format(db=db, skip=skip or "").split()


def load_records(path):
    from canu_gb300 import sort_records
    return sort_records(np.fromfile(path, dtype=np.uint32).reshape(-1, 6))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CANU_SRC") or os.path.join(ROOT, "..", "reference"))
    a = ap.parse_args()
    from canu_gb300.build import build_tools, build_lib
    build_lib()
    _, synth = build_tools()
    subprocess.run(["make", "-s", "-f", "Makefile.ref", f"REF={a.ref}", "-j8"], cwd=os.path.join(ROOT, "oracle"),
                   check=True)
    ref_bin = os.path.join(ROOT, "oracle", "_ref", "oic_ref")
    meta = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (sargs, oargs) in CASES.items():
            db, skip = make_inputs(synth, sargs, tmp, name)
            out = os.path.join(tmp, name + ".ovb")
            stats = os.path.join(tmp, name + ".stats")
            subprocess.run([ref_bin] + oic_args(oargs, db, skip) + ["-o", out, "-s", stats], check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            rec = load_records(out)
            oc = np.fromfile(os.path.join(tmp, name + ".oc"), dtype=np.uint8)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), records=rec, oc=oc,
                                stats=np.frombuffer(open(stats, "rb").read(), dtype=np.uint8))
            meta[name] = {"synth": sargs, "args": oargs, "seqdb_sha256": sha256(db),
                          "skip_sha256": sha256(skip) if skip else None, "n_records": int(len(rec))}
            print(f"{name}: {len(rec)} records")
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
