"""tm_assemble_matrix_noalloc: the assembly entry point for callers that
cannot allocate GPU memory (an FFI host holding only device pointers handed
to it by another framework, or a process confined to a fixed device pool).
It takes its partial-sum workspace from a static device array instead of a
caller-provided buffer.

Checked through the C ABI against tm_assemble_matrix on the same inputs,
on two calls in a row (the static array keeps the previous call's contents,
which must not leak into the next result), plus its size limit.  This file
is collected last so that a stop at the first failure has already run every
other test."""
import ctypes as C

import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import load_golden, rel_fro
from tensormesh_gb300 import _lib

pytestmark = pytest.mark.gpu


def _noalloc_fn():
    lib = _lib.load()
    fn = lib.tm_assemble_matrix_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(_lib.MatrixArgs), C.c_void_p]
    return lib, fn


def _args(topo, dev, pts, kappa, outK, outM):
    a = _lib.MatrixArgs()
    a.dtype = _lib.TM_F64
    a.forms = _lib.TM_FORM_DIFFUSION | _lib.TM_FORM_MASS
    a.n_points = topo.n_points
    a.points = _lib.ptr(pts)
    a.kappa = _lib.ptr(kappa)
    a.kappa_scale = a.mass_scale = a.young_scale = 1.0
    a.poisson = 0.3
    a.out_diffusion, a.out_mass = _lib.ptr(outK), _lib.ptr(outM)
    a.plan = topo.matrix_plan(dev).struct()
    a.tables = topo.table_struct(dev)
    return a


MESHES = {
    "tetra": lambda: tg.gen_unit_cube(6, jitter=0.2, seed=21),                 # 1296 elements, 6 chunks
    "triangle6": lambda: tg.gen_unit_square(24, order=2, jitter=0.1, seed=22),  # 1152 elements, 18 chunks
}


@pytest.mark.parametrize("etype", list(MESHES))
def test_noalloc_matches_workspace_entry_point(etype, cuda):
    lib, noalloc = _noalloc_fn()
    mesh = MESHES[etype]().to(cuda)
    asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    topo = asm._topology
    pts = mesh.points.contiguous()
    kappa = torch.from_numpy(np.random.default_rng(23).lognormal(0.0, 1.0, mesh.n_elements)).to(cuda)
    stream = _lib.stream_handle(cuda)

    refK = torch.empty(topo.nnz, dtype=torch.float64, device=cuda)
    refM = torch.empty_like(refK)
    a = _args(topo, cuda, pts, kappa, refK, refM)
    ws = torch.empty(max(1, lib.tm_matrix_workspace_bytes(C.byref(a))), dtype=torch.uint8, device=cuda)
    a.workspace = _lib.ptr(ws)
    _lib.check(lib.tm_assemble_matrix(C.byref(a), stream), "tm_assemble_matrix")
    assert topo.matrix_plan(cuda).n_partials > 0          # the variant's scratch is actually used

    for call in range(2):
        K = torch.full((topo.nnz,), float("nan"), dtype=torch.float64, device=cuda)
        M = torch.full_like(K, float("nan"))
        kap = kappa * (1.0 + call)                            # second call: different inputs
        b = _args(topo, cuda, pts, kap, K, M)
        _lib.check(noalloc(C.byref(b), stream), "tm_assemble_matrix_noalloc")
        torch.cuda.synchronize()
        assert rel_fro(K, refK * (1.0 + call)) <= 1e-12
        assert rel_fro(M, refM) <= 1e-12


def test_noalloc_rejects_plans_above_the_limit(cuda):
    lib, noalloc = _noalloc_fn()
    g = load_golden("tet4")
    mesh = tg.Mesh(torch.from_numpy(g["points"]), {"tetra": torch.from_numpy(g["conn"])}).to(cuda)
    topo = tg.LaplaceElementAssembler.from_mesh(mesh)._topology
    K = torch.empty(topo.nnz, dtype=torch.float64, device=cuda)
    a = _args(topo, cuda, mesh.points.contiguous(), torch.ones(mesh.n_elements, dtype=torch.float64, device=cuda),
              K, torch.empty_like(K))
    a.plan.n_partials = (64 << 20) // 16 + 1            # two forms x 8 bytes: one partial over the limit
    st = noalloc(C.byref(a), _lib.stream_handle(cuda))
    assert st == _lib.TM_ERR_TOO_LARGE
    assert b"static scratch" in lib.tm_last_error_message()
