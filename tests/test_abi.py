"""The C ABI: header declarations vs the library's exports (no GPU needed)."""
import ctypes
import os
import re

import pytest

from ffgpu import _lib
from ffgpu.build import build

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(REPO, "include", "ffgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ffgpu_[a-z0-9_]+)\s*\(", txt)))


def test_library_builds_and_exports_every_declared_symbol():
    path = build()
    L = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 16
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert sorted(_lib.EXPORTS) == syms


def test_binding_signatures_cover_the_header():
    L = _lib.lib()
    for s in declared_symbols():
        assert getattr(L, s).restype is not None or s.endswith("destroy")


def test_no_gpu_reports_an_error_not_a_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    code = _lib.lib().ffgpu_ctx_create(0, ctypes.byref(h))
    assert code != 0
    assert _lib.lib().ffgpu_last_error()
