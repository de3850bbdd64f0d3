"""The C-ABI library builds for sm_103a, loads on a machine without a GPU and
exports every entry point include/rumdeed_gpu.h declares (no compute calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:int|const char\s*\*)\s*(rd_\w+)\s*\(", src, flags=re.M)
    return names


def test_library_exports_every_declared_symbol(rg):
    lib = ctypes.CDLL(rg.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers the same set
    assert set(names) <= set(rg.SIGNATURES), set(names) - set(rg.SIGNATURES)


def test_version_and_error_entry_points(rg):
    L = rg.lib()
    assert L.rd_version() >= 10000
    assert isinstance(L.rd_last_error(), bytes)
    # invalid arguments are reported as status codes, never by aborting
    assert L.rd_engine_create(None, None) == -1
    assert b"null" in L.rd_last_error()
    assert L.rd_sync(None) == -1


def test_no_oracle_in_product_path():
    """The product path never imports or links the oracle."""
    pkg = os.path.join(ROOT, "rumdeed_gb300")
    for dp, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                txt = open(os.path.join(dp, f)).read()
                assert "orc" + "_" not in txt and "import orc" not in txt, f


def test_invalid_chunking_is_refused_before_touching_the_gpu(rg):
    with pytest.raises(rg.RumdeedError, match="chunk_min"):
        rg.Engine(chunk_min=100)
    with pytest.raises(rg.RumdeedError, match="chunk_count_max"):
        rg.Engine(chunk_count_max=64)
