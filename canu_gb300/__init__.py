"""GB300 overlapInCore engine -- Python binding of liboic_gpu.so (include/oic_gpu.h).

The compute path is the CUDA library; this module only marshals host buffers through
ctypes.  There is no CPU fallback: if the library or a CUDA device is missing, every
call raises OicError.

    from canu_gb300 import Overlapper, default_params
    p = default_params(kmerLen=22, maxErate=0.06, minOlapLen=500, hashBits=23)
    with Overlapper(p) as ov:
        ov.set_reads_seqdb("reads.seqdb")
        ov.run()
        recs = ov.overlaps()          # (n, 6) uint32, the ovFile record words
"""
import ctypes
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "liboic_gpu.so")

OIC_OK, OIC_ERR_ARG, OIC_ERR_INPUT, OIC_ERR_CUDA, OIC_ERR_NOMEM, OIC_ERR_OVERFLOW, OIC_ERR_STATE, OIC_ERR_DEVICE = range(8)

# Exported entry points of include/oic_gpu.h.
EXPORTS = (
    "oic_default_params", "oic_create", "oic_destroy", "oic_set_reads", "oic_set_skip_kmers",
    "oic_load_hash_block", "oic_run_refs", "oic_run", "oic_num_overlaps", "oic_fetch_overlaps",
    "oic_clear_overlaps", "oic_get_stats", "oic_extend_batch", "oic_get_match_limit", "oic_last_error",
    "oic_extend_batch_noalloc", "oic_set_filter", "oic_collect_pairs", "oic_num_pairs", "oic_get_pairs",
    "oic_clear_pairs", "oic_mlp_forward", "oic_mlp_backward", "oic_mlp_adam", "oic_set_tuning", "oic_get_tuning",
    "oic_autotune", "oic_count_kmers", "oic_store_sort", "oic_stats_json",
)
# Output files (include/oic_ovfile.h): host code of the same library, no GPU needed.
OVFILE_EXPORTS = (
    "oic_ovb_write", "oic_ovb_read", "oic_oc_path", "oic_oc_write", "oic_oc_read", "oic_merge_outputs",
    "oic_snappy_max_length", "oic_snappy_compress", "oic_snappy_uncompress", "oic_ovstore_write",
)

# Learned candidate filter (include/oic_gpu.h): feature row width, hidden width and the
# FP16 parameter array w1[128][80] | b1[128] | w2[128][128] | b2[128] | w3[128] | b3.
FILTER_FEATURES, FILTER_IN, FILTER_HIDDEN = 67, 80, 128
FILTER_OFFSETS = {"w1": (0, (128, 80)), "b1": (10240, (128,)), "w2": (10368, (128, 128)),
                  "b2": (26752, (128,)), "w3": (26880, (128,)), "b3": (27008, (1,))}
FILTER_NPARAM = 27009

# oic_pair_info
PAIR_DTYPE = np.dtype([("aID", "<u4"), ("bID", "<u4"), ("flags", "<u4"), ("seeds", "<u4"), ("nodes", "<u4"),
                       ("overlaps", "<u4"), ("cells", "<u4"), ("score", "<f4"), ("extensions", "<u4"),
                       ("firstHit", "<i4"), ("cellsFirst", "<u4"), ("extLimit", "<u4")])


class OicError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"oic error {code}: {msg}")
        self.code = code


class OicParams(ctypes.Structure):
    """oic_params (overlapInCore.H:367-473)."""
    _fields_ = [
        ("maxErate", ctypes.c_double), ("alignNoise", ctypes.c_double),
        ("partial", ctypes.c_int32), ("uniqueOlapPerPair", ctypes.c_int32),
        ("useHopelessCheck", ctypes.c_int32), ("minKmers", ctypes.c_int32),
        ("kmerLen", ctypes.c_uint32), ("hashBits", ctypes.c_uint32),
        ("maxHashLoad", ctypes.c_double), ("maxHashDataLen", ctypes.c_uint64),
        ("minOlapLen", ctypes.c_int32), ("numThreads", ctypes.c_uint32),
        ("bgnHashID", ctypes.c_uint32), ("endHashID", ctypes.c_uint32),
        ("minLibToHash", ctypes.c_uint32), ("maxLibToHash", ctypes.c_uint32),
        ("bgnRefID", ctypes.c_uint32), ("endRefID", ctypes.c_uint32),
        ("minLibToRef", ctypes.c_uint32), ("maxLibToRef", ctypes.c_uint32),
    ]


class OicStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "kmerHitsWithoutOlap", "kmerHitsWithOlap", "kmerHitsSkipped", "multiOverlap",
        "totalOverlaps", "containedOverlaps", "dovetailOverlaps", "badShortWindow", "badLongWindow",
        "dpCells", "slideBases", "extensions", "seeds", "candidatePairs", "nodes", "dpRows")] + [
        ("nHashBlocks", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
        ("msHash", ctypes.c_double), ("msSeed", ctypes.c_double),
        ("msAlign", ctypes.c_double), ("msTotal", ctypes.c_double),
        ("msReads", ctypes.c_double), ("kernelLaunches", ctypes.c_uint64), ("dpCellsNoOverlap", ctypes.c_uint64),
        ("filteredPairs", ctypes.c_uint64), ("msFilter", ctypes.c_double),
        ("msNarrow", ctypes.c_double), ("msWide", ctypes.c_double), ("pairsNarrow", ctypes.c_uint64),
        ("pairsWide", ctypes.c_uint64), ("cellsWide", ctypes.c_uint64), ("graphLaunches", ctypes.c_uint64)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}

    def to_json(self):
        """oic_stats_json: the counters, device times and rates as JSON text."""
        lib, n = library(), ctypes.c_size_t()
        lib.oic_stats_json(ctypes.byref(self), None, 0, ctypes.byref(n))
        buf = ctypes.create_string_buffer(n.value + 1)
        rc = lib.oic_stats_json(ctypes.byref(self), buf, n.value + 1, ctypes.byref(n))
        if rc:
            raise OicError(rc, "oic_stats_json")
        return buf.value.decode()


class FilterDomain(ctypes.Structure):
    """oic_filter_domain: the parameters a filter network was trained under."""
    _fields_ = [("kmerLen", ctypes.c_uint32), ("minOlapLen", ctypes.c_int32), ("maxErate", ctypes.c_double)]


def filter_domain(params):
    """The filter domain of an oic_params (or of a dict with kmerLen, minOlapLen, maxErate)."""
    g = (lambda k: params[k]) if isinstance(params, dict) else (lambda k: getattr(params, k))
    return {"kmerLen": int(g("kmerLen")), "minOlapLen": int(g("minOlapLen")),
            "maxErate": float(np.float32(g("maxErate")))}


class OicTuning(ctypes.Structure):
    """oic_tuning: DP launch configuration (zeros = defaults)."""
    _fields_ = [("narrowArena", ctypes.c_uint32), ("wideMinLen", ctypes.c_uint32), ("wideThreads", ctypes.c_uint32),
                ("wideTile", ctypes.c_uint32), ("wideBandW", ctypes.c_uint32), ("wideCtas", ctypes.c_uint32),
                ("wideArena", ctypes.c_uint64), ("forceWide", ctypes.c_uint32), ("noGraph", ctypes.c_uint32),
                ("wideMode", ctypes.c_uint32)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_lib = None


def library():
    """Load liboic_gpu.so (built in-tree by canu_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OicError(OIC_ERR_CUDA, f"{LIB_PATH} is not built; run python -m canu_gb300.build")
        lib = ctypes.CDLL(LIB_PATH)
        P, U32, U64, I32 = ctypes.POINTER, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32
        vp = ctypes.c_void_p
        lib.oic_default_params.argtypes = [P(OicParams)]
        lib.oic_create.argtypes = [P(OicParams), ctypes.c_int, P(vp)]
        lib.oic_destroy.argtypes = [vp]
        lib.oic_set_reads.argtypes = [vp, U32, vp, vp, vp, vp, U64]
        lib.oic_set_skip_kmers.argtypes = [vp, ctypes.c_char_p, U64]
        lib.oic_load_hash_block.argtypes = [vp, U32, U32, P(U32)]
        lib.oic_run_refs.argtypes = [vp, U32, U32]
        lib.oic_run.argtypes = [vp]
        lib.oic_num_overlaps.argtypes = [vp, P(U64)]
        lib.oic_fetch_overlaps.argtypes = [vp, vp, U64, P(U64)]
        lib.oic_clear_overlaps.argtypes = [vp]
        lib.oic_get_stats.argtypes = [vp, P(OicStats)]
        lib.oic_stats_json.argtypes = [P(OicStats), ctypes.c_char_p, ctypes.c_size_t, P(ctypes.c_size_t)]
        lib.oic_extend_batch.argtypes = [vp, U32] + [vp] * 9
        lib.oic_get_match_limit.argtypes = [vp, vp, U32, P(U32)]
        lib.oic_extend_batch_noalloc.argtypes = [vp, U32, vp, vp, vp, vp, vp]
        lib.oic_store_sort.argtypes = [ctypes.c_int, vp, U64, U32, ctypes.c_double, vp, P(U64), vp, vp]
        lib.oic_ovb_write.argtypes = [ctypes.c_char_p, vp, U64, ctypes.c_int]
        lib.oic_ovstore_write.argtypes = [ctypes.c_char_p, vp, U64, vp, U32, U64]
        lib.oic_ovb_read.argtypes = [ctypes.c_char_p, vp, U64, P(U64)]
        lib.oic_oc_path.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
        lib.oic_oc_write.argtypes = [ctypes.c_char_p, vp, U64, U32]
        lib.oic_oc_read.argtypes = [ctypes.c_char_p, P(U64), vp, U32, P(U32)]
        lib.oic_merge_outputs.argtypes = [ctypes.c_char_p, P(ctypes.c_char_p), U32]
        lib.oic_snappy_max_length.restype = ctypes.c_size_t
        lib.oic_snappy_max_length.argtypes = [ctypes.c_size_t]
        lib.oic_snappy_compress.argtypes = [vp, ctypes.c_size_t, vp, P(ctypes.c_size_t)]
        lib.oic_snappy_uncompress.argtypes = [vp, ctypes.c_size_t, vp, ctypes.c_size_t, P(ctypes.c_size_t)]
        lib.oic_set_filter.argtypes = [vp, vp, ctypes.c_float, ctypes.c_float, U32, P(FilterDomain)]
        lib.oic_collect_pairs.argtypes = [vp, ctypes.c_int]
        lib.oic_num_pairs.argtypes = [vp, P(U64), P(U64)]
        lib.oic_get_pairs.argtypes = [vp, vp, vp, vp, U64, U64]
        lib.oic_clear_pairs.argtypes = [vp]
        lib.oic_mlp_forward.argtypes = [vp, vp, U32, vp, vp, vp, vp]
        lib.oic_mlp_backward.argtypes = [vp, vp, vp, vp, vp, vp, vp, U32, vp, vp, vp, vp, vp]
        F = ctypes.c_float
        lib.oic_mlp_adam.argtypes = [vp, vp, vp, vp, vp, F, F, F, F, F, F, U32, vp]
        lib.oic_set_tuning.argtypes = [vp, P(OicTuning)]
        lib.oic_get_tuning.argtypes = [vp, P(OicTuning)]
        lib.oic_autotune.argtypes = [vp, U32, U32, vp, U32, P(U32)]
        lib.oic_count_kmers.argtypes = [vp, U32, U32, U32, vp, vp, U64, P(U64)]
        lib.oic_last_error.argtypes = [vp]
        lib.oic_last_error.restype = ctypes.c_char_p
        _lib = lib
    return _lib


def default_params(**kw):
    """The reference defaults (oicParameters::initialize) with overrides by field name.
    Float flags are rounded through float32 as overlapInCore's strtof does."""
    p = OicParams()
    library().oic_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if k in ("maxErate", "alignNoise"):
            v = float(np.float32(v))
        setattr(p, k, v)
    return p


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def read_seqdb(path):
    """Load an oic_seqdb container: (libID, length, offset, bases) as numpy arrays."""
    with open(path, "rb") as f:
        head = f.read(24)
        if head[:8] != b"OICSEQ01":
            raise ValueError(f"{path}: not an oic_seqdb container")
        n, _, nb = struct.unpack("<IIQ", head[8:24])
        idx = np.frombuffer(f.read(16 * n), dtype=np.dtype([("lib", "<u4"), ("len", "<u4"), ("off", "<u8")]))
        bases = np.frombuffer(f.read(nb), dtype=np.uint8)
    return (np.ascontiguousarray(idx["lib"]), np.ascontiguousarray(idx["len"]),
            np.ascontiguousarray(idx["off"]), bases)


def write_seqdb(path, seqs, libs=None):
    """Write reads (list of str/bytes) as an oic_seqdb container."""
    seqs = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
    lens = [len(s) for s in seqs]
    libs = libs if libs is not None else [1] * len(seqs)
    with open(path, "wb") as f:
        f.write(b"OICSEQ01" + struct.pack("<IIQ", len(seqs), 0, sum(lens)))
        off = 0
        for lb, ln in zip(libs, lens):
            f.write(struct.pack("<IIQ", lb, ln, off))
            off += ln
        for s in seqs:
            f.write(s)


class Overlapper:
    """One engine context (one CUDA stream) -- the GPU overlapInCore."""

    def __init__(self, params, device=0):
        self._lib = library()
        self._ctx = ctypes.c_void_p()
        self.params = params
        rc = self._lib.oic_create(ctypes.byref(params), int(device), ctypes.byref(self._ctx))
        if rc != OIC_OK:
            raise OicError(rc, "oic_create failed (invalid parameters or no usable CUDA device)")

    def close(self):
        if self._ctx:
            self._lib.oic_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != OIC_OK:
            raise OicError(rc, self._lib.oic_last_error(self._ctx).decode())

    def set_reads(self, lib, length, offset, bases):
        lib = np.ascontiguousarray(lib, dtype=np.uint32)
        length = np.ascontiguousarray(length, dtype=np.uint32)
        offset = np.ascontiguousarray(offset, dtype=np.uint64)
        bases = np.ascontiguousarray(bases, dtype=np.uint8)
        self._keep = (lib, length, offset, bases)
        self._check(self._lib.oic_set_reads(self._ctx, len(length), _ptr(lib), _ptr(length), _ptr(offset),
                                            _ptr(bases), bases.size))

    def set_reads_seqdb(self, path):
        self.set_reads(*read_seqdb(path))

    def set_skip_kmers(self, kmers):
        k = self.params.kmerLen
        blob = "".join(kmers).encode() if not isinstance(kmers, (bytes, bytearray)) else bytes(kmers)
        self._check(self._lib.oic_set_skip_kmers(self._ctx, blob, len(blob) // k))

    def load_hash_block(self, bgn, end):
        last = ctypes.c_uint32()
        self._check(self._lib.oic_load_hash_block(self._ctx, bgn, end, ctypes.byref(last)))
        return last.value

    def run_refs(self, bgn, end):
        self._check(self._lib.oic_run_refs(self._ctx, bgn, end))

    def run(self):
        self._check(self._lib.oic_run(self._ctx))

    def overlaps(self):
        n = ctypes.c_uint64()
        self._check(self._lib.oic_num_overlaps(self._ctx, ctypes.byref(n)))
        out = np.zeros((n.value, 6), dtype=np.uint32)
        got = ctypes.c_uint64()
        self._check(self._lib.oic_fetch_overlaps(self._ctx, _ptr(out), n.value, ctypes.byref(got)))
        return out[: got.value]

    def clear(self):
        self._check(self._lib.oic_clear_overlaps(self._ctx))

    def stats(self):
        s = OicStats()
        self._check(self._lib.oic_get_stats(self._ctx, ctypes.byref(s)))
        return s.as_dict()

    def match_limit(self):
        n = ctypes.c_uint32()
        self._check(self._lib.oic_get_match_limit(self._ctx, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.int32)
        self._check(self._lib.oic_get_match_limit(self._ctx, _ptr(out), n.value, ctypes.byref(n)))
        return out

    def set_filter(self, params, threshold, full_threshold=0.0, ext_budget=1, domain=None):
        """Learned candidate filter: params = FILTER_NPARAM float16 values (None: off).
        Pairs scored below threshold are dropped; below full_threshold they stop once
        ext_budget extensions have found no overlap.  domain: the parameters the network
        was trained under (kmerLen, minOlapLen, maxErate; a trained file's
        meta["domain"]); the library refuses a network trained under other values."""
        if params is None:
            self._check(self._lib.oic_set_filter(self._ctx, None, 0.0, 0.0, 0, None))
            return
        prm = np.ascontiguousarray(params, dtype=np.float16).view(np.uint16)
        if prm.size != FILTER_NPARAM:
            raise ValueError(f"filter needs {FILTER_NPARAM} parameters, got {prm.size}")
        dom = None
        if domain is not None:
            d = filter_domain(domain)
            dom = FilterDomain(d["kmerLen"], d["minOlapLen"], d["maxErate"])
        self._check(self._lib.oic_set_filter(self._ctx, _ptr(prm), float(threshold), float(full_threshold),
                                             int(ext_budget), ctypes.byref(dom) if dom is not None else None))

    def collect_pairs(self, mode=1):
        """0 off, 1 candidate pairs + feature rows, 2 also their match runs."""
        self._check(self._lib.oic_collect_pairs(self._ctx, int(mode)))

    def pairs(self, nodes=False):
        """Collected pairs: (info [PAIR_DTYPE], feature rows [n, 80] float16[, runs [m, 3] int32])."""
        n, m = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self._lib.oic_num_pairs(self._ctx, ctypes.byref(n), ctypes.byref(m)))
        info = np.zeros(n.value, dtype=PAIR_DTYPE)
        feat = np.zeros((n.value, FILTER_IN), dtype=np.float16)
        runs = np.zeros((m.value if nodes else 0, 3), dtype=np.int32)
        self._check(self._lib.oic_get_pairs(self._ctx, _ptr(info), _ptr(feat), _ptr(runs) if nodes else None,
                                            n.value, m.value if nodes else 0))
        return (info, feat, runs) if nodes else (info, feat)

    def clear_pairs(self):
        self._check(self._lib.oic_clear_pairs(self._ctx))

    def set_tuning(self, **kw):
        """DP launch configuration by field name (OicTuning); no arguments: defaults."""
        if not kw:
            self._check(self._lib.oic_set_tuning(self._ctx, None))
            return
        t = OicTuning()
        for k, v in kw.items():
            setattr(t, k, v)
        self._check(self._lib.oic_set_tuning(self._ctx, ctypes.byref(t)))

    def tuning(self):
        t = OicTuning()
        self._check(self._lib.oic_get_tuning(self._ctx, ctypes.byref(t)))
        return t.as_dict()

    def count_kmers(self, bgn, end, min_count):
        """Canonical k-mers of reads [bgn, end] seen at least min_count times:
        (list of k-mer strings, uint32 counts), ascending canonical 2-bit key."""
        n = ctypes.c_uint64()
        rc = self._lib.oic_count_kmers(self._ctx, bgn, end, min_count, None, None, 0, ctypes.byref(n))
        if rc not in (OIC_OK, OIC_ERR_OVERFLOW):
            self._check(rc)
        k = self.params.kmerLen
        buf = np.zeros(n.value * k, dtype=np.uint8)
        cnt = np.zeros(n.value, dtype=np.uint32)
        if n.value:
            self._check(self._lib.oic_count_kmers(self._ctx, bgn, end, min_count, _ptr(buf), _ptr(cnt), n.value,
                                                  ctypes.byref(n)))
        s = buf.tobytes().decode()
        return [s[i * k:(i + 1) * k] for i in range(n.value)], cnt

    def autotune(self, bgn, end, max_lines=64):
        """Time the DP grid on ref reads [bgn, end] of the loaded block; sets the fastest.
        Returns one dict per configuration."""
        rep = np.zeros((max_lines, 8), dtype=np.float64)
        n = ctypes.c_uint32()
        self._check(self._lib.oic_autotune(self._ctx, bgn, end, _ptr(rep), max_lines, ctypes.byref(n)))
        keys = ("wideTile", "wideThreads", "wideMinLen", "msNarrow", "msWide", "msTotal", "pairsNarrow", "cellsWide")
        return [dict(zip(keys, map(float, r))) for r in rep[: n.value]]

    def extend_batch(self, sRead, sRev, tRead, mStart, mOffset, mLen):
        """Batched Extend_Alignment; returns (out[n,5], kind[n], deltaLen[n])."""
        a = [np.ascontiguousarray(x, dtype=t) for x, t in zip(
            (sRead, sRev, tRead, mStart, mOffset, mLen),
            (np.uint32, np.uint32, np.uint32, np.int32, np.int32, np.int32))]
        n = len(a[0])
        out = np.zeros((n, 5), dtype=np.int32)
        kind = np.zeros(n, dtype=np.int32)
        dl = np.zeros(n, dtype=np.int32)
        self._check(self._lib.oic_extend_batch(self._ctx, n, *[_ptr(x) for x in a], _ptr(out), _ptr(kind), _ptr(dl)))
        return out, kind, dl


def _mlp_check(rc, what):
    if rc != OIC_OK:
        raise OicError(rc, what + " failed")


def mlp_forward(params, x, n, logit, h1=0, h2=0, stream=0):
    """oic_mlp_forward on device pointers (ints)."""
    _mlp_check(library().oic_mlp_forward(params, x, n, logit, h1 or None, h2 or None, stream or None), "mlp forward")


def mlp_backward(params, x, h1, h2, logit, label, weight, n, grad, g1, g2, loss=0, stream=0):
    """oic_mlp_backward on device pointers (ints); weight/loss may be 0 (NULL)."""
    _mlp_check(library().oic_mlp_backward(params, x, h1, h2, logit, label, weight or None, n, grad, g1, g2,
                                          loss or None, stream or None), "mlp backward")


def mlp_adam(master, m, v, grad, params, lr, beta1, beta2, eps, grad_scale, weight_decay, step, stream=0):
    """oic_mlp_adam on device pointers (ints)."""
    _mlp_check(library().oic_mlp_adam(master, m, v, grad, params, lr, beta1, beta2, eps, grad_scale, weight_decay,
                                      step, stream or None), "mlp adam")


def _file_check(rc, what, path):
    if rc == 1:
        raise OSError(ctypes.get_errno() or 5, f"{what} failed", path)
    if rc:
        raise ValueError(f"{path}: {what}: malformed file or argument")


def write_ovb(path, records, framing=1):
    """Write records ((n, 6) uint32) as canu's ovFile(ovFileFullWrite): snappy blocks
    (framing 1) or unframed words (framing 0)."""
    r = np.ascontiguousarray(records, dtype=np.uint32).reshape(-1, 6)
    _file_check(library().oic_ovb_write(os.fsencode(path), _ptr(r), len(r), int(framing)), "write .ovb", path)


def read_ovb(path):
    """Records ((n, 6) uint32) of a snappy-framed .ovb file."""
    lib, n = library(), ctypes.c_uint64()
    _file_check(lib.oic_ovb_read(os.fsencode(path), None, 0, ctypes.byref(n)), "read .ovb", path)
    out = np.zeros((n.value, 6), dtype=np.uint32)
    _file_check(lib.oic_ovb_read(os.fsencode(path), _ptr(out), n.value, ctypes.byref(n)), "read .ovb", path)
    return out


def write_ovstore(path, records, read_lens, max_per_file=0):
    """Write an overlap-store directory as canu's sequential store writer lays it out
    (info, index, data files 0001-NNN, statistics) from store records ((n, 6) uint32,
    sorted as store_sort returns them); read_lens[i] is the length of read ID i+1."""
    r = np.ascontiguousarray(records, dtype=np.uint32).reshape(-1, 6)
    ln = np.ascontiguousarray(read_lens, dtype=np.uint32)
    _file_check(library().oic_ovstore_write(os.fsencode(path), _ptr(r), len(r), _ptr(ln), len(ln), int(max_per_file)),
                "write ovStore", path)


def oc_path(ovb_path):
    """The .oc name canu pairs with an .ovb name (cut at the first '.' of the file name)."""
    buf = ctypes.create_string_buffer(4096)
    _file_check(library().oic_oc_path(os.fsencode(ovb_path), buf, 4096), "oc name", ovb_path)
    return os.fsdecode(buf.value)


def read_oc(path):
    """(number of records, per-read counts [oprMax] uint32) of an .oc file."""
    lib, n, m = library(), ctypes.c_uint64(), ctypes.c_uint32()
    _file_check(lib.oic_oc_read(os.fsencode(path), ctypes.byref(n), None, 0, ctypes.byref(m)), "read .oc", path)
    opr = np.zeros(m.value, dtype=np.uint32)
    if m.value:
        _file_check(lib.oic_oc_read(os.fsencode(path), ctypes.byref(n), _ptr(opr), m.value - 1, ctypes.byref(m)),
                    "read .oc", path)
    return n.value, opr


def merge_outputs(out_ovb, inputs):
    """Merge independent jobs' .ovb/.oc outputs into out_ovb and its .oc."""
    arr = (ctypes.c_char_p * len(inputs))(*[os.fsencode(x) for x in inputs])
    _file_check(library().oic_merge_outputs(os.fsencode(out_ovb), arr, len(inputs)), "merge", out_ovb)


def store_sort(records, max_id, max_erate=1.0, device=0):
    """The overlap-store build's record pass on the GPU (oic_store_sort): returns (sorted
    records (m, 6) uint32, perRead first-record offsets (max_id + 2) uint64, counters
    dict)."""
    r = np.ascontiguousarray(records, dtype=np.uint32).reshape(-1, 6)
    out = np.zeros((2 * len(r), 6), dtype=np.uint32)
    per = np.zeros(int(max_id) + 2, dtype=np.uint64)
    cnt = np.zeros(5, dtype=np.uint64)
    m = ctypes.c_uint64()
    rc = library().oic_store_sort(int(device), _ptr(r), len(r), int(max_id), float(max_erate), _ptr(out),
                                  ctypes.byref(m), _ptr(per), _ptr(cnt))
    if rc != OIC_OK:
        raise OicError(rc, "oic_store_sort failed")
    names = ("saved_unitigging", "saved_trimming", "discarded_erate", "discarded_no_trim", "discarded_flipped")
    return out[: m.value], per, dict(zip(names, map(int, cnt)))


def sort_records(rec):
    """Records in ovOverlap::operator< order (ovOverlap.H:264-277): a_iid, b_iid, then
    the data words as two 64-bit values -- the same as lexicographic on the six words."""
    rec = np.asarray(rec, dtype=np.uint32).reshape(-1, 6)
    if len(rec) == 0:
        return rec
    order = np.lexsort(tuple(rec[:, k] for k in range(5, -1, -1)))
    return rec[order]
