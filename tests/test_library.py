"""CPU checks of the CUDA library artefact: it builds for sm_103a, loads, and
exports every entry point include/centre_gpu.h declares; without a device it
refuses to run instead of falling back to the CPU."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib_path():
    from centre_gb300 import build as B
    return B.build()


def header_symbols():
    with open(os.path.join(ROOT, "include", "centre_gpu.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"\b(centre_gpu_\w+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = header_symbols()
    assert "centre_gpu_create" in syms and "centre_gpu_entropy2d" in syms
    assert len(syms) >= 15


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header(lib_path):
    from centre_gb300 import _lib
    assert set(header_symbols()) <= set(_lib.exported_symbols())


def test_no_silent_cpu_fallback(lib_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from centre_gb300.api import CentreError, Context
    with pytest.raises(CentreError) as e:
        Context(0)
    assert e.value.status == -7


def test_strerror_names_every_status(lib_path):
    from centre_gb300 import _lib
    L = _lib.load()
    for st in range(0, -8, -1):
        assert L.centre_gpu_strerror(st).decode() != "unknown status"
