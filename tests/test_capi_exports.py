"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?(?:int|void|char|float|double)\s*\*?\s*(swe_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_functions():
    names = declared_functions()
    assert "swe_gpu_step" in names and "swe_gpu_domain_create" in names and "swe_host_init_block" in names


def test_library_exports_every_declared_symbol(swe):
    lib = ctypes.CDLL(swe.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_exports(swe):
    for n in declared_functions():
        assert n in swe.EXPORTED or n.startswith("swe_gpu_"), n


def test_invalid_descriptor_is_rejected_without_gpu(swe):
    with pytest.raises(swe.SweGpuError):
        swe.Domain([0], [4], 1.0, 1.0)
    assert "width" in swe.lib().swe_gpu_last_error().decode()
