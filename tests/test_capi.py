"""The C-ABI library: exports, parameter validation, no silent CPU fallback."""
import ctypes
import os
import re

import pytest

import canu_gb300 as oic

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions(header="oic_gpu.h"):
    src = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|size_t|const char \*)\s*(oic_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built["lib"])
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(oic.EXPORTS)
    files = header_functions("oic_ovfile.h")
    for n in files:
        assert hasattr(lib, n), n
    assert set(files) == set(oic.OVFILE_EXPORTS)


def test_default_params_match_reference_defaults(built):
    p = oic.default_params()
    assert p.maxErate == 0.06 and p.alignNoise == 1.0
    assert p.hashBits == 22 and p.maxHashLoad == 0.6 and p.maxHashDataLen == 100000000
    assert p.uniqueOlapPerPair == 1 and p.useHopelessCheck == 1
    assert p.bgnHashID == 1 and p.endHashID == 0xffffffff


def test_maxerate_is_rounded_like_strtof(built):
    # float(0.06f) = 0.0599999986588955 < 0.06: the hopeless check stays on at 0.06.
    assert oic.default_params(maxErate=0.06).maxErate == 0.05999999865889549
    assert oic.default_params(maxErate=0.01).maxErate == 0.009999999776482582
    assert oic.default_params(maxErate=0.06).maxErate < 0.06


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the behaviour without a GPU")
def test_no_gpu_fails_loudly(built):
    with pytest.raises(oic.OicError) as e:
        oic.Overlapper(oic.default_params(kmerLen=22))
    assert e.value.code == oic.OIC_ERR_CUDA


def test_bad_parameters_rejected(built):
    lib = oic.library()
    ctx = ctypes.c_void_p()
    p = oic.default_params(kmerLen=0)
    assert lib.oic_create(ctypes.byref(p), 0, ctypes.byref(ctx)) == oic.OIC_ERR_ARG
    p = oic.default_params(kmerLen=40)
    assert lib.oic_create(ctypes.byref(p), 0, ctypes.byref(ctx)) == oic.OIC_ERR_ARG


def test_stats_json_carries_every_counter_and_the_rates(built):
    """oic_stats_json (host code): every oic_stats field by name, and overlaps/s and DP
    cells/s from the device times; a buffer one byte short is refused with the size."""
    import ctypes
    import json
    s = oic.OicStats()
    for i, (name, typ) in enumerate(s._fields_):
        setattr(s, name, (1.5 * (i + 1)) if typ is ctypes.c_double else (i + 1) * 1000003)
    s.totalOverlaps, s.msTotal, s.dpCells, s.msAlign = 12345, 250.0, 9 * 10**11, 4500.0
    d = json.loads(s.to_json())
    for name, typ in s._fields_:
        if name != "reserved":
            assert d[name] == getattr(s, name), name
    assert d["overlapsPerSec"] == pytest.approx(12345 / 0.25)
    assert d["dpCellsPerSec"] == pytest.approx(9e11 / 4.5)
    lib, n = oic.library(), ctypes.c_size_t()
    assert lib.oic_stats_json(ctypes.byref(s), None, 0, ctypes.byref(n)) == oic.OIC_ERR_ARG and n.value > 0
    buf = ctypes.create_string_buffer(n.value)
    assert lib.oic_stats_json(ctypes.byref(s), buf, n.value, ctypes.byref(n)) == oic.OIC_ERR_ARG
    s.msTotal = s.msAlign = 0.0
    d = json.loads(s.to_json())
    assert d["overlapsPerSec"] == 0 and d["dpCellsPerSec"] == 0
