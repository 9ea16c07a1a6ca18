"""ctypes binding of ``libtmgb300.so`` (the C ABI declared in
``include/tensormesh_gb300.h``).

The library is loaded on first use.  If it is missing it is built with
``tensormesh_gb300.build.build()``; if that is impossible the import fails
with an error -- the package has no CPU or eager-PyTorch substitute for the
kernels.
"""
import ctypes as C
import os
import threading

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
_LOCK = threading.Lock()
_LIB = None

(TM_OK, TM_ERR_INVALID_ARG, TM_ERR_UNSUPPORTED, TM_ERR_CUDA, TM_ERR_PLAN, TM_ERR_TOO_LARGE,
 TM_ERR_DEVICE_WAIT) = range(7)
TM_F64, TM_F32 = 0, 1
TM_FORM_DIFFUSION, TM_FORM_MASS, TM_FORM_ELASTICITY = 1, 2, 4
TM_SOURCE_NODAL, TM_SOURCE_CONST, TM_SOURCE_QUAD = 0, 1, 2
TM_PLAN_KIND_MATRIX, TM_PLAN_KIND_NODE = 0, 1
(PLAN_EDGE_ROW, PLAN_EDGE_COL, PLAN_SLOT, PLAN_CHUNK_BEGIN, PLAN_SLOT_PTR, PLAN_CONTRIB,
 PLAN_SLOT_TARGET, PLAN_SLOT_MIRROR, PLAN_SHARED_PTR, PLAN_SHARED_TARGET, PLAN_SHARED_MIRROR,
 PLAN_CONN, PLAN_PERM, PLAN_CHUNK_CONTRIB) = range(14)


class TmError(RuntimeError):
    """A status code other than TM_OK returned by the native library."""


class ElementTables(C.Structure):
    _fields_ = [("element_type", C.c_int32), ("n_quad", C.c_int32), ("packed", C.c_void_p)]


class ChunkPlan(C.Structure):
    _fields_ = [
        ("n_elements", C.c_int64), ("n_basis", C.c_int32), ("n_local", C.c_int32),
        ("chunk_elems", C.c_int32), ("n_chunks", C.c_int32), ("n_targets", C.c_int64),
        ("n_shared", C.c_int32), ("n_partials", C.c_int32),
        ("elem_perm", C.c_void_p), ("conn", C.c_void_p), ("chunk_begin", C.c_void_p),
        ("slot_ptr", C.c_void_p), ("contrib", C.c_void_p), ("slot_target", C.c_void_p),
        ("slot_mirror", C.c_void_p), ("shared_ptr", C.c_void_p), ("shared_target", C.c_void_p),
        ("shared_mirror", C.c_void_p), ("chunk_contrib", C.c_void_p), ("max_chunk_slots", C.c_int32),
        ("max_chunk_contrib", C.c_int32),
    ]


class DeviceChunkPlan(C.Structure):
    _fields_ = [
        ("conn", C.c_void_p), ("chunk_begin", C.c_void_p), ("chunk_contrib", C.c_void_p),
        ("slot_ptr", C.c_void_p), ("contrib", C.c_void_p), ("slot_target", C.c_void_p),
        ("slot_mirror", C.c_void_p), ("shared_ptr", C.c_void_p), ("shared_target", C.c_void_p),
        ("shared_mirror", C.c_void_p), ("cap_slots", C.c_int64), ("cap_contrib", C.c_int64),
        ("cap_shared", C.c_int64), ("n_chunks", C.c_int64), ("n_slots", C.c_int64), ("n_contrib", C.c_int64),
        ("n_shared", C.c_int64), ("n_partials", C.c_int64), ("max_chunk_slots", C.c_int32),
        ("max_chunk_contrib", C.c_int32),
    ]


class MatrixArgs(C.Structure):
    _fields_ = [
        ("dtype", C.c_int32), ("forms", C.c_int32), ("n_points", C.c_int64),
        ("points", C.c_void_p), ("kappa", C.c_void_p), ("kappa_scale", C.c_double),
        ("mass_scale", C.c_double), ("young", C.c_void_p), ("young_scale", C.c_double),
        ("poisson", C.c_double), ("out_diffusion", C.c_void_p), ("out_mass", C.c_void_p),
        ("out_elasticity", C.c_void_p), ("workspace", C.c_void_p),
        ("tables", ElementTables), ("plan", ChunkPlan),
        ("event_begin", C.c_void_p), ("event_end", C.c_void_p), ("stats", C.c_void_p),
        ("event_done", C.c_void_p),
    ]


class VectorArgs(C.Structure):
    _fields_ = [
        ("dtype", C.c_int32), ("source", C.c_int32), ("width", C.c_int32), ("n_points", C.c_int64),
        ("points", C.c_void_p), ("values", C.c_void_p), ("constant", C.c_double * 3),
        ("out", C.c_void_p), ("workspace", C.c_void_p),
        ("tables", ElementTables), ("plan", ChunkPlan),
    ]


class FacetTables(C.Structure):
    _fields_ = [("facet_type", C.c_int32), ("n_quad", C.c_int32), ("packed", C.c_void_p)]


class FacetVectorArgs(C.Structure):
    _fields_ = [
        ("dtype", C.c_int32), ("source", C.c_int32), ("width", C.c_int32), ("pad0", C.c_int32),
        ("n_points", C.c_int64), ("points", C.c_void_p), ("values", C.c_void_p),
        ("const_value", C.c_double * 3), ("out", C.c_void_p), ("workspace", C.c_void_p),
        ("tables", FacetTables), ("plan", ChunkPlan),
    ]


class FacetAdjointArgs(C.Structure):
    _fields_ = [("base", FacetVectorArgs), ("lam", C.c_void_p), ("grad_points", C.c_void_p),
                ("grad_values", C.c_void_p)]


class AdjointArgs(C.Structure):
    _fields_ = [
        ("dtype", C.c_int32), ("k_mode", C.c_int32), ("load_source", C.c_int32), ("reserved", C.c_int32),
        ("n_points", C.c_int64), ("points", C.c_void_p), ("kappa", C.c_void_p), ("kappa_scale", C.c_double),
        ("weights", C.c_void_p), ("slot_map", C.c_void_p), ("u", C.c_void_p), ("lam", C.c_void_p),
        ("load_const", C.c_double), ("load_values", C.c_void_p), ("grad_kappa", C.c_void_p),
        ("grad_points", C.c_void_p), ("workspace", C.c_void_p),
        ("tables", ElementTables), ("plan", ChunkPlan), ("poisson", C.c_double),
    ]


class CoefGradArgs(C.Structure):
    _fields_ = [
        ("form", C.c_int32), ("flags", C.c_int32),
        ("n_points", C.c_int64), ("points", C.c_void_p), ("weights", C.c_void_p), ("slot_map", C.c_void_p),
        ("scale", C.c_double), ("poisson", C.c_double), ("grad", C.c_void_p),
        ("tables", ElementTables), ("plan", ChunkPlan),
    ]


TM_ADJ_K_NONE, TM_ADJ_K_CSR, TM_ADJ_K_OUTER, TM_ADJ_M_CSR, TM_ADJ_E_CSR = 0, 1, 2, 3, 4
TM_ADJ_LOAD_NONE, TM_ADJ_LOAD_CONST, TM_ADJ_LOAD_NODAL, TM_ADJ_LOAD_QUAD = 0, 1, 2, 3


class CondenseArgs(C.Structure):
    _fields_ = [
        ("dtype", C.c_int32), ("width", C.c_int32), ("values", C.c_void_p),
        ("n_kept", C.c_int64), ("kept_src", C.c_void_p), ("out_kept", C.c_void_p),
        ("n_io", C.c_int64), ("io_src", C.c_void_p), ("out_io", C.c_void_p),
        ("n_inner", C.c_int64), ("inner_dof", C.c_void_p), ("row_ptr", C.c_void_p),
        ("n_row_entries", C.c_int64), ("row_src", C.c_void_p), ("row_col", C.c_void_p),
        ("outer_value", C.c_void_p), ("rhs", C.c_void_p), ("out_rhs", C.c_void_p),
    ]


class LinearOperator(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("block", C.c_int32), ("n_rows", C.c_int64),
                ("row_ptr", C.c_void_p), ("col", C.c_void_p), ("values", C.c_void_p),
                ("row_order", C.c_void_p)]


class PcgArgs(C.Structure):
    _fields_ = [("A", LinearOperator), ("b", C.c_void_p), ("x", C.c_void_p), ("r", C.c_void_p),
                ("z", C.c_void_p), ("p", C.c_void_p), ("q", C.c_void_p), ("dinv", C.c_void_p),
                ("scalars", C.c_void_p), ("partials", C.c_void_p)]


class BicgstabArgs(C.Structure):
    _fields_ = [("A", LinearOperator), ("b", C.c_void_p), ("x", C.c_void_p), ("work", C.c_void_p),
                ("scalars", C.c_void_p), ("partials", C.c_void_p), ("atol", C.c_double), ("rtol", C.c_double)]


class PcgStatus(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("flag", C.c_int32), ("relative_residual", C.c_double)]


class BatchedPcgArgs(C.Structure):
    _fields_ = [("n_systems", C.c_int32), ("max_iter", C.c_int32), ("rtol", C.c_double),
                ("system_offset", C.c_void_p), ("A", LinearOperator), ("dirichlet", C.c_void_p),
                ("b", C.c_void_p), ("x", C.c_void_p), ("work", C.c_void_p), ("queue", C.c_void_p),
                ("status", C.c_void_p), ("order", C.c_void_p)]


class BatchedMixedArgs(C.Structure):
    _fields_ = [("base", BatchedPcgArgs), ("values32", C.c_void_p), ("inner_rtol", C.c_double),
                ("max_outer", C.c_int32), ("reserved", C.c_int32)]


TM_PCG_CONVERGED, TM_PCG_MAX_ITER, TM_PCG_BREAKDOWN = 1, 2, 3
TM_COEF_GRAD_LAME_PARTS = 1
TM_BICG_RR, TM_BICG_BB, TM_BICG_ITER, TM_BICG_FLAG = 5, 7, 8, 9


_SIGNATURES = {
    "tm_error_string": (C.c_char_p, [C.c_int]),
    "tm_last_error_message": (C.c_char_p, []),
    "tm_version": (C.c_int, []),
    "tm_device_fault": (C.c_int, []),
    "tm_plan_build": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int64, C.c_int32, C.c_int32,
                                C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "tm_plan_array_size": (C.c_int64, [C.c_void_p, C.c_int32]),
    "tm_plan_copy_array": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "tm_plan_scalar": (C.c_int64, [C.c_void_p, C.c_int32]),
    "tm_plan_free": (None, [C.c_void_p]),
    "tm_matrix_workspace_bytes": (C.c_size_t, [C.POINTER(MatrixArgs)]),
    "tm_assemble_matrix": (C.c_int, [C.POINTER(MatrixArgs), C.c_void_p]),
    "tm_vector_workspace_bytes": (C.c_size_t, [C.POINTER(VectorArgs)]),
    "tm_assemble_vector": (C.c_int, [C.POINTER(VectorArgs), C.c_void_p]),
    "tm_shape_grad_jxw": (C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, ElementTables, C.c_void_p,
                                    C.c_void_p, C.c_void_p]),
    "tm_quadrature_points": (C.c_int, [C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, ElementTables,
                                       C.c_void_p, C.c_void_p]),
    "tm_morton_order": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p]),
    "tm_pattern_workspace_bytes": (C.c_size_t, [C.c_int64, C.c_int32, C.c_int64]),
    "tm_morton_workspace_bytes": (C.c_size_t, [C.c_int64, C.c_int32, C.c_int32]),
    "tm_morton_order_device": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64, C.c_int32,
                                         C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "tm_chunk_plan_device_workspace_bytes": (C.c_size_t, [C.c_int64, C.c_int32, C.c_int64, C.c_int32, C.c_int32]),
    "tm_chunk_plan_device": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int64, C.c_int32, C.c_int32,
                                       C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                       C.POINTER(DeviceChunkPlan), C.c_void_p]),
    "tm_pattern_count": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p,
                                   C.POINTER(C.c_int64), C.c_void_p]),
    "tm_pattern_fill": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "tm_facet_vector_workspace_bytes": (C.c_size_t, [C.POINTER(FacetVectorArgs)]),
    "tm_assemble_facet_vector": (C.c_int, [C.POINTER(FacetVectorArgs), C.c_void_p]),
    "tm_facet_adjoint_workspace_bytes": (C.c_size_t, [C.POINTER(FacetAdjointArgs)]),
    "tm_facet_adjoint": (C.c_int, [C.POINTER(FacetAdjointArgs), C.c_void_p]),
    "tm_condense": (C.c_int, [C.POINTER(CondenseArgs), C.c_void_p]),
    "tm_project_reduce": (C.c_int, [C.c_int32, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p]),
    "tm_spmv": (C.c_int, [C.POINTER(LinearOperator), C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                          C.c_void_p]),
    "tm_adjoint_workspace_bytes": (C.c_size_t, [C.POINTER(AdjointArgs)]),
    "tm_adjoint_p1": (C.c_int, [C.POINTER(AdjointArgs), C.c_void_p]),
    "tm_adjoint_general": (C.c_int, [C.POINTER(AdjointArgs), C.c_void_p]),
    "tm_coef_grad": (C.c_int, [C.POINTER(CoefGradArgs), C.c_void_p]),
    "tm_batched_pcg": (C.c_int, [C.POINTER(BatchedPcgArgs), C.c_void_p]),
    "tm_batched_pcg_mixed": (C.c_int, [C.POINTER(BatchedMixedArgs), C.c_void_p]),
    "tm_pcg_partials_bytes": (C.c_size_t, []),
    "tm_pcg_start": (C.c_int, [C.POINTER(PcgArgs), C.c_void_p]),
    "tm_bicgstab_start": (C.c_int, [C.POINTER(BicgstabArgs), C.c_void_p]),
    "tm_bicgstab_iterate": (C.c_int, [C.POINTER(BicgstabArgs), C.c_int32, C.c_void_p]),
    "tm_pcg_iterate": (C.c_int, [C.POINTER(PcgArgs), C.c_int32, C.c_void_p]),
    "tm_pcg_iterate_until": (C.c_int, [C.POINTER(PcgArgs), C.c_int32, C.c_double, C.c_void_p]),
}

EXPORTED = tuple(_SIGNATURES)


def lib_path() -> str:
    return os.path.join(_HERE, "libtmgb300.so")


def load(build_if_missing: bool = True):
    """Load (and if needed build) the native library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = lib_path()
        if build_if_missing:
            from .build import build
            build()
        if not os.path.exists(path):
            raise ImportError(f"tensormesh_gb300 native library not found at {path}; run "
                              f"tensormesh_gb300.build.build()")
        lib = C.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def check(status: int, what: str = "") -> None:
    if status != TM_OK:
        lib = load()
        msg = lib.tm_last_error_message().decode(errors="replace")
        kind = lib.tm_error_string(status).decode(errors="replace")
        err = TmError(f"{what}: {kind}: {msg}" if what else f"{kind}: {msg}")
        err.status = status
        raise err


def ptr(t) -> int:
    return 0 if t is None else t.data_ptr()


def stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def dtype_code(dtype: torch.dtype) -> int:
    if dtype == torch.float64:
        return TM_F64
    if dtype == torch.float32:
        return TM_F32
    raise TypeError(f"tensormesh_gb300 computes in float64 or float32, got {dtype}")


def require_cuda(t: torch.Tensor, what: str) -> None:
    if not t.is_cuda:
        raise RuntimeError(f"{what} must be a CUDA tensor: tensormesh_gb300 assembles on the GPU only "
                           f"(got device {t.device})")
