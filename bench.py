#!/usr/bin/env python3
"""Benchmark of the GB300 overlapInCore path (one JSON line on stdout, rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c2] [--scale 1.0] [--no-skip-list]

A step is one whole overlapInCore job on the workload's read set: the hash block of
all reads, then every read (both strands) against it -- seed lookup, per-pair match
lists, and the banded edit-distance extensions that emit the overlap records.

  value  overlaps/s with the reads already resident in HBM (CUDA-event time of the
         job on the library's stream);
  e2e    the same through the C ABI with host buffers: every step uploads the reads
         from pinned host memory, runs the job and copies the records back (wall clock).

learned_filter  the same job with the learned candidate filter (weights trained on other
         seeds of the c2 shape): overlaps/s, recall against this run's plain records,
         and whether every filtered record equals its plain record.

--impl reference times the CPU restatement of the reference (oracle/oic_port.c, the
reference's algorithm step for step; canu's own sources cannot be built on the GPU
host) on all host cores: the hash block is built once and timed, each step runs a
sample of ref reads against it (chunks of 16 IDs spread evenly over the ID range),
and a step's rate charges the sample its share of the block build -- the full job's
rate, extrapolated from the sample.  That arm builds and loads only the oracle and
the read generator, never the CUDA library.

parity_vs_cpu  the GPU's records for the CPU baseline's sampled ref reads (same hash
         block) compared record for record with the oracle's.

--no-skip-list runs a workload that has a frequent-k-mer skip list (c2, c5) without it,
as those configurations are written.  Their tandem arrays then give k-mers with
~10^4-10^5 occurrences, and the seeds of the reads that cross them grow with the square
of the genome size, for this engine and for the reference alike: use it at reduced
--scale.

Multi-GPU (torchrun): every rank runs an independent replica on its own GPU (the
stage shards into independent jobs; there is no data exchange), value = all ranks'
overlaps / the slowest rank's time.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD_TEXT = {
    "c2": ("c2: 50 Mbp genome with 200 x 6 kb repeat copies (1% divergence) and 2% 171 bp tandem arrays; 30x "
           "HiFi-like reads (normal 15+-3 kb), 0.5% errors, 50% reverse-complemented; k=22, --minlength 1000, "
           "--maxerate 0.01, --hashbits 25, --hashdatalen 1.6e9; frequent-k-mer skip list (genome multiplicity "
           "> 10)"),
    "c1": ("c1: 5 Mbp iid genome, 20x lognormal reads (8+-3 kb, 1-30 kb), 2% errors 1:1:1; k=22, --minlength 500, "
           "--maxerate 0.06, --hashbits 23"),
    "c3": ("c3: 20 Mbp iid genome, 25x Pareto reads (alpha 1.5, 0.5-100 kb), 5% errors 1:2:2; --maxerate 0.12"),
    "c5": ("c5: 200 Mbp genome with 1000 x 6 kb repeat copies and 3% tandem arrays; 40x c2-like reads; --hashbits 27, "
           "--hashdatalen 2e9 (4 hash blocks); frequent-k-mer skip list"),
}

def workload_text(a):
    """The workload's description; without its skip list, said so."""
    t = WORKLOAD_TEXT.get(a.workload, a.workload)
    if a.no_skip_list:
        t = t.split("; frequent-k-mer skip list")[0] + "; no frequent-k-mer skip list (the configuration as written)"
    return t


L2_NOTE = "inputs (2-bit reads, hash table, seed lists) larger than L2"


def seqdb_counts(path):
    """(reads, bases) of an oic_seqdb container, from its header."""
    import struct
    with open(path, "rb") as f:
        head = f.read(24)
    n, _, nb = struct.unpack("<IIQ", head[8:24])
    return n, nb


def job_config(a, db, ws):
    """The line's `config`: what the job is, identical in both arms."""
    n, nb = seqdb_counts(db)
    return {"workload": workload_text(a), "scale": a.scale, "reads": n, "bases": nb, "parallelism": f"replicas{ws}",
            "l2": L2_NOTE}


# Nominal INT32 lanes per SM (Blackwell: 128 unified FP32/INT32 lanes).
INT_LANES_PER_SM = 128


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.proc, self.lines = gpu, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier_max(value, ws, device="cuda"):
    """max over ranks (and a barrier); device "cpu" for a gloo process group."""
    if ws == 1:
        return value
    import torch
    import torch.distributed as td
    t = torch.tensor([value], dtype=torch.float64, device=device)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def dp_bins(res):
    """Per-bin DP figures of the timed steps (mean over steps): the one-warp bin and the
    CTA bin (its pairs include the one-warp bin's reruns)."""
    def mean(k):
        return statistics.mean(float(r[0].get(k, 0)) for r in res)
    cells_all, cells_wide = mean("dpCells"), mean("cellsWide")
    out = {}
    for name, pairs, ms, cells in (("one_warp", mean("pairsNarrow"), mean("msNarrow"), cells_all - cells_wide),
                                   ("cta", mean("pairsWide"), mean("msWide"), cells_wide)):
        out[name] = {"pairs": pairs, "ms": ms, "dp_cells": cells,
                     "dp_cells_per_sec": cells / (ms / 1000.0) if ms > 0 else None}
    return out


def replica_rate(units_per_rank, seconds, ws, device="cuda"):
    """Whole-job rate of independent replicas: every rank's units over the slowest
    rank's time (the ranks run the same workload, so units_per_rank is this rank's)."""
    return ws * units_per_rank / barrier_max(seconds, ws, device)


# ----------------------------------------------------------------------------------
# CPU path (the oracle, test infrastructure)

class PortParams(ctypes.Structure):
    _fields_ = [("maxErate", ctypes.c_double), ("alignNoise", ctypes.c_double), ("partial", ctypes.c_int),
                ("bgnHashID", ctypes.c_uint32), ("endHashID", ctypes.c_uint32),
                ("minLibToHash", ctypes.c_uint32), ("maxLibToHash", ctypes.c_uint32),
                ("bgnRefID", ctypes.c_uint32), ("endRefID", ctypes.c_uint32),
                ("minLibToRef", ctypes.c_uint32), ("maxLibToRef", ctypes.c_uint32),
                ("kmerLen", ctypes.c_uint32), ("kmerSkipFile", ctypes.c_char_p), ("minKmers", ctypes.c_int),
                ("uniqueOlapPerPair", ctypes.c_int), ("hashBits", ctypes.c_uint32),
                ("maxHashDataLen", ctypes.c_uint64), ("maxHashLoad", ctypes.c_double),
                ("numThreads", ctypes.c_uint32), ("minOlapLen", ctypes.c_int32), ("useHopelessCheck", ctypes.c_int)]


class PortStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "kmerHitsWithoutOlap", "kmerHitsWithOlap", "kmerHitsSkipped", "multiOverlap", "totalOverlaps",
        "containedOverlaps", "dovetailOverlaps", "badShortWindow", "badLongWindow", "dpCells", "slideBases",
        "extensions", "seeds", "candidatePairs")] + [("nHashBlocks", ctypes.c_uint32)]


class CpuPath:
    """The oracle on all host cores: block built once, ref samples timed against it."""

    def __init__(self, wl, db, skip, threads):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
        lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "liboic_port.so"))
        lib.oic_port_seqdb_load.restype = ctypes.c_void_p
        lib.oic_port_seqdb_load.argtypes = [ctypes.c_char_p]
        lib.oic_port_session_new.restype = ctypes.c_void_p
        lib.oic_port_session_new.argtypes = [ctypes.POINTER(PortParams), ctypes.c_void_p,
                                             ctypes.POINTER(ctypes.c_double)]
        lib.oic_port_session_refs.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32,
                                              ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_uint64),
                                              ctypes.POINTER(PortStats)]
        lib.oic_port_records_free.argtypes = [ctypes.c_void_p]
        lib.oic_port_session_free.argtypes = [ctypes.c_void_p]
        lib.oic_port_seqdb_free.argtypes = [ctypes.c_void_p]
        lib.oic_port_default_params.argtypes = [ctypes.POINTER(PortParams)]
        self.lib = lib
        from canu_gb300 import workloads
        g = workloads.WORKLOADS[wl]["params"]
        p = PortParams()
        lib.oic_port_default_params(ctypes.byref(p))
        p.maxErate = float(np.float32(g["maxErate"]))
        p.kmerLen = g["kmerLen"]
        p.hashBits = g["hashBits"]
        p.maxHashDataLen = g["maxHashDataLen"]
        p.maxHashLoad = g.get("maxHashLoad", 0.6)
        p.minOlapLen = g["minOlapLen"]
        p.numThreads = threads
        if p.maxErate > 0.06:
            p.useHopelessCheck = 0
        self._skip = skip.encode() if skip else None
        p.kmerSkipFile = self._skip
        self.db = lib.oic_port_seqdb_load(db.encode())
        from canu_gb300 import read_seqdb
        self.nReads = len(read_seqdb(db)[1])
        bs = ctypes.c_double()
        self.sess = lib.oic_port_session_new(ctypes.byref(p), self.db, ctypes.byref(bs))
        if not self.sess:
            raise RuntimeError("oracle session failed")
        self.build_s = bs.value

    def sample(self, bgn, end, keep=False):
        """Ref reads [bgn, end] against the block: (seconds, stats, records or None)."""
        recs = ctypes.c_void_p()
        n = ctypes.c_uint64()
        st = PortStats()
        t0 = time.perf_counter()
        self.lib.oic_port_session_refs(self.sess, bgn, end, ctypes.byref(recs), ctypes.byref(n), ctypes.byref(st))
        dt = time.perf_counter() - t0
        out = None
        if keep:
            out = np.zeros((n.value, 6), dtype=np.uint32)
            if n.value:
                ctypes.memmove(out.ctypes.data, recs.value, 24 * n.value)
        self.lib.oic_port_records_free(recs)
        return dt, st, out

    def close(self):
        self.lib.oic_port_session_free(self.sess)
        self.lib.oic_port_seqdb_free(self.db)

    def rate(self, dt, nref, overlaps):
        """Overlaps/s of the full job: the sample's time plus its share of the block build."""
        return overlaps / (dt + self.build_s * nref / self.nReads)


def spread_chunks(n_reads, chunk=16):
    """Ref-read chunks [bgn, end] in van der Corput order of their index: every prefix of
    the sequence is spread evenly over the read IDs.  A ref read only pairs with reads of
    higher ID, so a sample taken from the first IDs would see more than its share of
    the pairs; a spread sample sees its share."""
    m = (n_reads + chunk - 1) // chunk
    bits = max(1, (m - 1).bit_length())
    while True:
        for i in range(1 << bits):
            j = int(format(i, f"0{bits}b")[::-1], 2)
            if j < m:
                yield 1 + j * chunk, min(n_reads, (j + 1) * chunk)


def cpu_sample(cpu, chunks, target_s=15.0, keep=False):
    """Run ref chunks from the iterator until about target_s seconds of CPU work.
    Returns (seconds, overlaps, ref reads, DP cells, chunks run, records or None)."""
    dt_tot, ov, nref, cells, done, recs = 0.0, 0, 0, 0, [], []
    seen = set()
    while dt_tot < target_s:
        b, e = next(chunks)
        if (b, e) in seen:        # the whole read set has been sampled once
            break
        seen.add((b, e))
        dt, st, r = cpu.sample(b, e, keep)
        dt_tot += dt
        ov += st.totalOverlaps
        cells += st.dpCells
        nref += e - b + 1
        done.append((b, e))
        if keep:
            recs.append(r)
    return dt_tot, ov, nref, cells, done, (np.concatenate(recs) if keep and recs else None)


def gpu_parity(ov, oic, n_reads, chunks, cpu_recs):
    """The GPU's records for the CPU sample's ref chunks, against the same first hash
    block, compared record for record (and as .oc per-read counts) with the oracle's."""
    ov.clear()
    ov.load_hash_block(1, n_reads)
    for b, e in chunks:
        ov.run_refs(b, e)
    got = oic.sort_records(ov.overlaps())
    ref = oic.sort_records(cpu_recs.reshape(-1, 6)) if cpu_recs is not None else np.zeros((0, 6), np.uint32)
    same = got.shape == ref.shape and bool((got == ref).all())
    oc_got = np.bincount(got[:, :2].ravel(), minlength=n_reads + 1)
    oc_ref = np.bincount(ref[:, :2].ravel(), minlength=n_reads + 1)
    ov.clear()
    return {"refs": int(sum(e - b + 1 for b, e in chunks)), "chunks": len(chunks), "records": int(len(ref)),
            "records_gpu": int(len(got)), "records_identical": same,
            "oc_identical": bool(oc_got.shape == oc_ref.shape and (oc_got == oc_ref).all()),
            "sample": "ref-read chunks of 16 IDs spread over the whole ID range (van der Corput order), each "
                      "against the first hash block; the oracle's records vs the GPU's, sorted"}


# ----------------------------------------------------------------------------------

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c5"])
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--data-dir", default=os.environ.get("OIC_BENCH_DATA", "/tmp/oic_bench"))
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-filter", action="store_true", help="skip the learned-filter leg")
    ap.add_argument("--no-skip-list", action="store_true",
                    help="run the workload without its frequent-k-mer skip list (c2 / c5 as their configurations "
                         "are written); the learned filter, trained with the list, is left out")
    a = ap.parse_args()
    if a.no_skip_list:
        a.no_filter = True
    ws, rank, local = dist()
    cores = os.cpu_count() or 1

    import __graft_entry__
    if a.impl == "reference":
        # The CPU arm builds and loads only the read generator and the oracle.
        if rank == 0:
            __graft_entry__.build_oracle()
    elif rank == 0:
        __graft_entry__.build()
    import canu_gb300 as oic
    from canu_gb300 import workloads

    if a.impl == "reference":
        if rank != 0:
            return 0
        db, skip = workloads.generate(a.workload, a.data_dir, a.scale)
        skip = None if a.no_skip_list else skip
        cpu = CpuPath(a.workload, db, skip, cores)
        vals, samples = [], []
        chunks = spread_chunks(cpu.nReads)
        for i in range(a.warmup + a.steps):
            per = max(2.0, a.cpu_seconds / max(1, a.steps))
            dt, ov, nref, cells, _, _ = cpu_sample(cpu, chunks, per)
            if i >= a.warmup:
                vals.append(cpu.rate(dt, nref, ov))
                samples.append((dt, nref, ov))
        cpu.close()
        v = statistics.mean(vals)
        nrefs = sum(s[1] for s in samples)
        line = {"impl": "reference", "metric": "overlaps_per_sec", "value": v, "unit": "overlaps/s", "n_gpus": 0,
                "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1000 * statistics.mean(s[0] for s in samples),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
                "data": "synthetic", "config": job_config(a, db, ws),
                "cpu_baseline": {"value": v, "unit": "overlaps/s", "cores": cores, "kind": "port",
                                 "sample": f"{nrefs} ref reads (both strands) in chunks of 16 spread over the ID "
                                           f"range, against the first hash block; block build {cpu.build_s:.1f} s "
                                           f"charged pro rata; full-job rate extrapolated"},
                "e2e": {"value": v, "unit": "overlaps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0

    # ------------------------------------------------------------------ our arm
    if ws > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(local)
        td.init_process_group("nccl")
        td.barrier()
    if rank == 0:
        db, skip = workloads.generate(a.workload, a.data_dir, a.scale)
    if ws > 1:
        td.barrier()
    db, skip = workloads.generate(a.workload, a.data_dir, a.scale)
    skip = None if a.no_skip_list else skip
    lib_, ln, off, bases = oic.read_seqdb(db)
    nReads = len(ln)
    try:
        import torch
        pinned = torch.empty(bases.size, dtype=torch.uint8, pin_memory=True)
        pinned.numpy()[:] = bases
        host_bases = pinned.numpy()
        pinned_ok = True
    except Exception:
        host_bases = np.ascontiguousarray(bases)
        pinned_ok = False

    p = workloads.params(a.workload)
    ov = oic.Overlapper(p, device=local if ws > 1 else 0)
    if skip:
        ov.set_skip_kmers(workloads.read_skip(skip))
    ov.set_reads(lib_, ln, off, host_bases)

    peaks, peak_kind = measured_peaks()

    def timed(with_clocks):
        """W untimed + K timed steps; each step uploads the reads, runs the job and reads
        the records back.  Returns ([(stats, wall s, records)], clocks, last records)."""
        clocks = Clocks(local) if with_clocks else None
        out, rec = [], None
        for i in range(a.warmup + a.steps):
            if i == a.warmup:
                barrier_max(0.0, ws)
                if clocks:
                    clocks.start()
            t0 = time.perf_counter()
            ov.clear()
            ov.set_reads(lib_, ln, off, host_bases)        # H2D of the step's input (pinned)
            ov.run()
            rec = ov.overlaps()                            # D2H of the step's result
            t1 = time.perf_counter()
            st = ov.stats()
            if i >= a.warmup:
                out.append((st, t1 - t0, len(rec)))
        return out, (clocks.stop() if clocks else None), rec

    res, clk, plain_rec = timed(True)

    # The learned candidate filter on the same reads (trained on other seeds).
    filt = None
    fpath = os.path.join(ROOT, "canu_gb300", "filter_c2.npz")
    fmeta = None
    if os.path.exists(fpath) and not a.no_filter:
        from canu_gb300 import filter_train
        fprm, fthr, ffull, fmeta = filter_train.load(fpath)
        if fmeta["domain"] != filter_train.training_domain(a.workload):
            fmeta = None        # the network serves only the parameters it was trained under
    if fmeta is not None:
        ov.set_filter(fprm, fthr, ffull, fmeta.get("budget", 1), domain=fmeta["domain"])
        fres, _, frec = timed(False)
        ov.set_filter(None, 0.0)
        recall, exact = filter_train.compare(plain_rec, frec)
        fms = statistics.mean(r[0]["msTotal"] for r in fres)
        fe2e = statistics.mean(r[1] for r in fres)
        fms_max, fe2e_max = barrier_max(fms, ws), barrier_max(fe2e, ws)
        fst = fres[0][0]
        filt = {"value": ws * fst["totalOverlaps"] / (fms_max / 1000.0), "unit": "overlaps/s",
                "dp_cells_per_sec": ws * fst["dpCells"] / (fms_max / 1000.0),
                "e2e": {"value": ws * fst["totalOverlaps"] / fe2e_max, "unit": "overlaps/s"},
                "ms_per_step": fms_max, "overlaps_per_step": fst["totalOverlaps"],
                "recall_vs_plain": recall, "records_identical_to_plain": exact,
                "dp_cells": fst["dpCells"], "dp_cells_skipped_frac": None, "filtered_pairs": fst["filteredPairs"],
                "ms_filter": fst["msFilter"], "ms_align": fst["msAlign"],
                "thresholds": {"drop_below_p": fthr, "budget_tier_below_p": ffull,
                               "extension_budget": fmeta.get("budget", 1)},
                "trained_on": f"c2 seeds {fmeta.get('train_seeds')}; this read set is {a.workload} seed "
                              f"{workloads.WORKLOADS[a.workload]['synth']['seed']} (not seen in training)",
                "gpu_launches": int(sum(r[0]["kernelLaunches"] for r in fres))}
    # The CPU baseline (rank 0, one GPU): the oracle on a spread sample of ref reads, and
    # the GPU's records for the same ref reads compared with the oracle's.
    cpu_line, parity = None, None
    if rank == 0 and ws == 1 and not a.no_cpu_baseline:
        cpu = CpuPath(a.workload, db, skip, cores)
        dt, ovs, nref, ccells, done, crec = cpu_sample(cpu, spread_chunks(cpu.nReads), a.cpu_seconds, keep=True)
        cpu.close()
        cpu_line = {"value": cpu.rate(dt, nref, ovs), "unit": "overlaps/s", "cores": cores, "kind": "port",
                    "sample": f"{nref} ref reads (both strands) in {len(done)} chunks of 16 spread over the ID range, "
                              f"against the first hash block ({dt:.1f} s); block build {cpu.build_s:.1f} s charged "
                              f"pro rata; full-job rate extrapolated; {ccells} DP cells"}
        parity = gpu_parity(ov, oic, nReads, done, crec)
    ov.close()

    ms_dev = statistics.mean(r[0]["msTotal"] for r in res)
    s_e2e = statistics.mean(r[1] for r in res)
    st0 = res[0][0]
    n_ov = st0["totalOverlaps"]
    ms_dev_max = barrier_max(ms_dev, ws)
    value = replica_rate(n_ov, ms_dev / 1000.0, ws)
    e2e = replica_rate(n_ov, s_e2e, ws)

    # Roofline of the dominant kernel, the pair DP (align_kernel).
    ms_align = statistics.mean(r[0]["msAlign"] for r in res)
    pairs, nodes, cells, slides = st0["candidatePairs"], st0["nodes"], st0["dpCells"], st0["slideBases"]
    mean_len = float(ln.mean())
    alg_bytes = pairs * (32 + 72 + 4 + 2 * mean_len / 4) + nodes * 16
    achieved = alg_bytes / (ms_align / 1000.0) / 1e9
    # DRAM bytes per DP cell of the one-warp DP kernel, from one ncu capture of a 1/50
    # scale c2 launch (10.54 GB read + 22.94 GB written for 6.598 G cells; the figures and
    # the command are in profiles/align_kernel_c2_scale0.02_ncu.md), scaled to this job.
    traffic = 5.074 * cells
    sm_mhz = clk.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    int_peak = 152 * INT_LANES_PER_SM * sm_mhz * 1e6 / 1e12
    int_ops = 6 * cells + slides / 16.0
    # Instruction issue, the one-warp DP's binding resource: 15.85 warp instructions per
    # DP cell (ncu smsp__inst_executed.sum of the same 1/50-scale c2 launch) against 152
    # SMs x 4 schedulers x one warp instruction per cycle.
    issue_peak = 152 * 4 * sm_mhz * 1e6 / 1e9
    issue_ach = 15.85 * cells / (ms_align / 1000.0) / 1e9
    # The memory stages by the byte model of the hash build and probe: build 0.25 B per
    # base read + 12 B per k-mer written (8 B key, 4 B position), and separately the sort
    # passes (6 passes x 24 B per k-mer); probe 2 strands x (0.25 B per base + one 32 B
    # sector per lookup) + 12 B per seed (4 B position read, 8 B seed written).
    K = p.kmerLen
    n_kmers = float(np.maximum(ln.astype(np.int64) - K + 1, 0).sum())
    n_bases = float(ln.astype(np.int64).sum())
    ms_hash = statistics.mean(r[0]["msHash"] for r in res)
    ms_seed = statistics.mean(r[0]["msSeed"] for r in res)
    sort_passes = (2 * K + 1 + 7) // 8

    def stage_roof(nbytes, ms, basis, traffic=None, traffic_basis=None):
        ach = nbytes / (ms / 1000.0) / 1e9 if ms > 0 else None
        return {"achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": ach / peaks["hbm_gbs"] if ach else None, "bytes": nbytes, "ms": ms, "basis": basis,
                "traffic": traffic, "traffic_basis": traffic_basis}
    hash_bytes = 0.25 * n_bases + 12 * n_kmers
    seed_bytes = 2 * n_bases * (0.25 + 32) + 12 * float(st0["seeds"])
    line = {
        "metric": "overlaps_per_sec", "value": value, "unit": "overlaps/s", "n_gpus": ws, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_dev_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": job_config(a, db, ws),
        "overlaps_per_step": n_ov,
        "dp_cells_per_sec": ws * cells / (ms_dev_max / 1000.0),
        "work": {"seeds": st0["seeds"], "candidate_pairs": pairs, "match_nodes": nodes, "extensions": st0["extensions"],
                 "dp_cells": cells, "dp_rows": st0.get("dpRows"), "slide_bases": slides,
                 "ms_hash": statistics.mean(r[0]["msHash"] for r in res),
                 "ms_seed": statistics.mean(r[0]["msSeed"] for r in res), "ms_align": ms_align},
        "dp_bins": dp_bins(res),
        "e2e": {"value": e2e, "unit": "overlaps/s", "h2d_bytes_per_step": int(host_bases.nbytes + ln.nbytes * 3 + off.nbytes),
                "d2h_bytes_per_step": int(n_ov * 24), "pinned": pinned_ok, "timing": "wall clock"},
        "roofline": {"bound": "hbm", "kernel": "align_kernel", "achieved": achieved,
                     "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                     "traffic": traffic, "traffic_basis": "ncu dram read+write per DP cell of a 1/50-scale c2 "
                                                          "launch x this job's DP cells (bytes per job)",
                     "peak_kind": peak_kind,
                     "int_ops": {"achieved_tops": int_ops / (ms_align / 1000.0) / 1e12, "peak_tops": int_peak,
                                 "frac": int_ops / (ms_align / 1000.0) / 1e12 / int_peak,
                                 "basis": "6 INT ops per DP cell + 1/16 per slide base; peak = 152 SMs x 128 "
                                          "INT32 lanes x median SM clock"},
                     "issue": {"achieved_g_warp_inst_per_s": issue_ach, "peak_g_warp_inst_per_s": issue_peak,
                               "frac": issue_ach / issue_peak,
                               "basis": "15.85 warp instructions per DP cell (ncu, one-warp DP kernel, 1/50-scale "
                                        "c2 launch: profiles/align_kernel_c2_scale0.02_ncu.md) x this job's DP "
                                        "cells / DP stage time; peak = 152 SMs x 4 schedulers x median SM clock"},
                     "hash": stage_roof(hash_bytes, ms_hash, "0.25 B/base + 12 B/k-mer (sort passes excluded)"),
                     "hash_with_sort": stage_roof(hash_bytes + sort_passes * 24 * n_kmers, ms_hash,
                                                  f"as hash + {sort_passes} radix passes x 24 B/k-mer",
                                                  sort_passes * 24.1 * n_kmers,
                                                  "radix passes only: ncu 24.1 B DRAM per key and pass "
                                                  "(profiles/radix_downsweep_c2_scale0.25_ncu.md)"),
                     "seed": stage_roof(seed_bytes, ms_seed, "2 strands x (0.25 B/base + 32 B/lookup) + 12 B/seed",
                                        54.9 * float(st0["seeds"]),
                                        "ncu 54.9 B DRAM per seed of a 1/4-scale c2 launch x this job's seeds "
                                        "(profiles/seed_kernel_c2_scale0.25_ncu.md)")},
        "gpu_launches": int(sum(r[0]["kernelLaunches"] for r in res)),
        "clocks": clk,
    }
    if filt:
        filt["dp_cells_skipped_frac"] = 1.0 - filt["dp_cells"] / max(cells, 1)
        filt["speedup_vs_plain"] = filt["value"] / value
        line["learned_filter"] = filt
    if cpu_line:
        line["cpu_baseline"] = cpu_line
        line["parity_vs_cpu"] = parity
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        td.barrier()
        td.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
