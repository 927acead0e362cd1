"""The C-ABI libraries load and export every symbol their headers declare (CPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(swm_[a-z0-9_]+)\s*\(", text)))


@pytest.mark.parametrize("header,lib", [("swmapper.h", "LIB_CUDA"), ("swm_synth.h", "LIB_SYNTH")])
def test_library_exports_header(header, lib):
    from swmapper_gb300 import _build
    if lib == "LIB_CUDA":
        _build.build_cuda()
    path = getattr(_build, lib)
    names = declared(header)
    assert names, header
    handle = ctypes.CDLL(path)
    missing = [n for n in names if not hasattr(handle, n)]
    assert not missing, missing


def test_product_has_no_oracle_dependency():
    """Nothing in the product package imports or links the oracle."""
    pkg = os.path.join(ROOT, "swmapper_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".c", ".h")):
                text = open(os.path.join(dirpath, f), errors="ignore").read()
                assert "pyoracle" not in text and "swm_oracle" not in text and "libswref" not in text, f
