"""The C-ABI library loads and exports every function the public header
declares (no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

from conftest import ROOT
from tensormesh_gb300 import _lib


def _declared():
    with open(os.path.join(ROOT, "include", "tensormesh_gb300.h")) as fh:
        text = fh.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tm_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_header_symbols():
    lib = ctypes.CDLL(_lib.load().__dict__["_name"])
    names = _declared()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_error_strings():
    lib = _lib.load()
    assert lib.tm_error_string(0) == b"ok"
    assert lib.tm_version() >= 1
