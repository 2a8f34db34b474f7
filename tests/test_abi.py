"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/s1g.h (no GPU calls)."""
import ctypes
import os
import re

from conftest import ROOT
from sentinel1_decode_gb300 import EXPORTS, load_library


def declared():
    with open(os.path.join(ROOT, "include", "s1g.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"\b(s1g_[a-z0-9_]+)\s*\(", src)))


def test_header_matches_binding_list():
    assert declared() == sorted(EXPORTS)


def test_library_exports_all_symbols(lib_path):
    lib = ctypes.CDLL(lib_path)
    for name in declared():
        assert hasattr(lib, name), name
    assert load_library().s1g_version().startswith(b"s1g")
