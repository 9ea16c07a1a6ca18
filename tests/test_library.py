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
    assert lib.tm_error_string(6) == b"a device-side wait ran out"


def test_matrix_call_rejects_unaligned_staged_arrays():
    """The argument checks run before any CUDA call: a plan whose staged
    arrays are not 16-byte aligned is refused with TM_ERR_INVALID_ARG."""
    lib = _lib.load()
    a = _lib.MatrixArgs()
    a.dtype, a.forms, a.n_points = _lib.TM_F64, 1, 4
    a.points = a.out_diffusion = 0x10000
    a.tables.element_type, a.tables.n_quad, a.tables.packed = 1, 4, 0x10000
    p = a.plan
    p.n_elements, p.n_basis, p.n_local, p.chunk_elems, p.n_chunks, p.n_targets = 1, 4, 10, 256, 1, 16
    p.max_chunk_slots, p.max_chunk_contrib = 16, 16
    for name in ("elem_perm", "conn", "chunk_begin", "slot_ptr", "contrib", "slot_target", "slot_mirror",
                 "chunk_contrib"):
        setattr(p, name, 0x10000)
    p.contrib = 0x10004
    assert lib.tm_assemble_matrix(ctypes.byref(a), None) == _lib.TM_ERR_INVALID_ARG
    assert b"16-byte aligned" in lib.tm_last_error_message()
    p.contrib = 0x10000
    p.max_chunk_contrib = 0
    assert lib.tm_assemble_matrix(ctypes.byref(a), None) == _lib.TM_ERR_INVALID_ARG
    assert b"max_chunk" in lib.tm_last_error_message()
