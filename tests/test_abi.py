"""The C ABI library loads and exports every function include/trw.h declares
(no GPU needed: loading the library does not initialise CUDA)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(trw_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared("trw.h")
    assert "trw_walk" in names and "trw_graph_create" in names and "trw_ppr_batch" in names


def test_library_exports_every_declared_symbol():
    from thunderrw_gb300 import _native as N
    if not os.path.exists(N.LIB_PATH):
        pytest.skip("libtrw_gpu.so not built")
    lib = N.load()
    for name in declared("trw.h"):
        assert hasattr(lib, name), name
    assert lib.trw_version() >= 1000
