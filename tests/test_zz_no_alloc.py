"""tm_assemble_matrix_noalloc: the assembly entry point for callers that
cannot allocate GPU memory (an FFI host holding only device pointers handed
to it by another framework, or a process confined to a fixed device pool).
It takes its partial-sum workspace from a static device array instead of a
caller-provided buffer.

Checked through the C ABI against tm_assemble_matrix on the same inputs, on
two calls in a row (the static array keeps the previous call's contents,
which must not leak into the next result), for every partial stride the
array serves: two scalar float64 forms fused (P1 tets, P2 triangles, Q2
quadrilaterals), one float32 form, and P2-tet elasticity (a 3x3 block per
partial).  Both entry points run the same kernels on the same plan, whose
reduction order is fixed, so the results must be bitwise equal.  Plus the
size limit.  This file is collected last so that a stop at the first failure
has already run every other test."""
import ctypes as C

import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import load_golden
from tensormesh_gb300 import _lib

pytestmark = pytest.mark.gpu


def _noalloc_fn():
    lib = _lib.load()
    fn = lib.tm_assemble_matrix_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(_lib.MatrixArgs), C.c_void_p]
    return lib, fn


def _args(topo, dev, pts, forms, coef, outs, block=False):
    a = _lib.MatrixArgs()
    a.dtype = _lib.dtype_code(pts.dtype)
    a.forms = forms
    a.n_points = topo.n_points
    a.points = _lib.ptr(pts)
    a.kappa_scale = a.mass_scale = a.young_scale = 1.0
    a.poisson = 0.3
    if forms & _lib.TM_FORM_ELASTICITY:
        a.young = _lib.ptr(coef)
        a.out_elasticity = _lib.ptr(outs[0])
    else:
        if forms & _lib.TM_FORM_DIFFUSION:
            a.kappa = _lib.ptr(coef)
            a.out_diffusion = _lib.ptr(outs[0])
        if forms & _lib.TM_FORM_MASS:
            a.out_mass = _lib.ptr(outs[-1])
    a.plan = topo.matrix_plan(dev, block=block, dtype=pts.dtype).struct()
    a.tables = topo.table_struct(dev)
    return a


DM = _lib.TM_FORM_DIFFUSION | _lib.TM_FORM_MASS
# name: (mesh, dtype, forms, block); each mesh spans several chunks, so
# that the plan has shared targets and the static array is used
CASES = {
    "tetra-f64-diffusion-mass": (lambda: tg.gen_unit_cube(6, jitter=0.2, seed=21), torch.float64, DM, False),
    "triangle6-f64-diffusion-mass": (lambda: tg.gen_unit_square(24, order=2, jitter=0.1, seed=22),
                                     torch.float64, DM, False),
    "quad9-f64-diffusion-mass": (lambda: tg.gen_unit_square(20, order=2, jitter=0.1, seed=24, cell="quad"),
                                 torch.float64, DM, False),
    "tetra-f32-diffusion": (lambda: tg.gen_unit_cube(6, jitter=0.2, seed=25, dtype=torch.float32),
                            torch.float32, _lib.TM_FORM_DIFFUSION, False),
    "tetra10-f64-elasticity": (lambda: tg.gen_unit_cube(4, order=2, jitter=0.1, seed=26), torch.float64,
                               _lib.TM_FORM_ELASTICITY, True),
}


def _outputs(topo, forms, dt, dev, fill):
    shape = (topo.nnz, 3, 3) if forms & _lib.TM_FORM_ELASTICITY else (topo.nnz,)
    n = 1 if forms != DM else 2
    return [torch.full(shape, fill, dtype=dt, device=dev) for _ in range(n)]


@pytest.mark.parametrize("case", list(CASES))
def test_noalloc_matches_workspace_entry_point(case, cuda):
    make, dt, forms, block = CASES[case]
    lib, noalloc = _noalloc_fn()
    mesh = make().to(cuda)
    asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    topo = asm._topology
    pts = mesh.points.contiguous()
    assert pts.dtype == dt
    coef = torch.from_numpy(np.random.default_rng(23).lognormal(0.0, 0.5, mesh.n_elements)).to(cuda, dt)
    stream = _lib.stream_handle(cuda)
    assert topo.matrix_plan(cuda, block=block, dtype=dt).n_partials > 0   # the static array is used

    for call in range(2):
        c = coef * (1.0 + call)                             # second call: different inputs
        ref = _outputs(topo, forms, dt, cuda, 0.0)
        a = _args(topo, cuda, pts, forms, c, ref, block)
        ws = torch.empty(max(1, lib.tm_matrix_workspace_bytes(C.byref(a))), dtype=torch.uint8, device=cuda)
        a.workspace = _lib.ptr(ws)
        _lib.check(lib.tm_assemble_matrix(C.byref(a), stream), "tm_assemble_matrix")

        got = _outputs(topo, forms, dt, cuda, float("nan"))
        b = _args(topo, cuda, pts, forms, c, got, block)
        _lib.check(noalloc(C.byref(b), stream), "tm_assemble_matrix_noalloc")
        torch.cuda.synchronize()
        assert lib.tm_device_fault() == 0
        for g, r in zip(got, ref):
            assert torch.isfinite(g).all()
            assert torch.equal(g, r), f"{case}, call {call}: results differ from tm_assemble_matrix"


def test_noalloc_rejects_plans_above_the_limit(cuda):
    lib, noalloc = _noalloc_fn()
    g = load_golden("tet4")
    mesh = tg.Mesh(torch.from_numpy(g["points"]), {"tetra": torch.from_numpy(g["conn"])}).to(cuda)
    topo = tg.LaplaceElementAssembler.from_mesh(mesh)._topology
    K = torch.empty(topo.nnz, dtype=torch.float64, device=cuda)
    a = _args(topo, cuda, mesh.points.contiguous(), DM, torch.ones(mesh.n_elements, dtype=torch.float64,
                                                                   device=cuda), [K, torch.empty_like(K)])
    a.plan.n_partials = (64 << 20) // 16 + 1            # two forms x 8 bytes: one partial over the limit
    st = noalloc(C.byref(a), _lib.stream_handle(cuda))
    assert st == _lib.TM_ERR_TOO_LARGE
    assert b"static scratch" in lib.tm_last_error_message()
