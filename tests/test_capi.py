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
