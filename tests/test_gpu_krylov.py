"""Jacobi-BiCGSTAB on the GPU (tm_bicgstab_*, ``bicgstab_solve``,
``SparseMatrix.solve(method="bicgstab")``) against the reference's own
solve of a non-symmetric system (golden fixture), direct solves, the CG
path on an SPD system, and its gradients against direct adjoint solves.
Tolerances: 1e-10 relative on solutions converged to a relative residual
near 1e-12; gradients 1e-9."""
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl
import torch

import tensormesh_gb300 as tg
from tensormesh_gb300.sparse import SparseMatrix
from conftest import rel_fro

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "small_krylov.npz")


def _fixture(cuda):
    d = np.load(GOLDEN)
    n = d["b"].size
    A = SparseMatrix(torch.from_numpy(d["values"]).to(cuda), torch.from_numpy(d["row"]).to(cuda),
                     torch.from_numpy(d["col"]).to(cuda), (n, n))
    As = sp.csr_matrix((d["values"], (d["row"], d["col"])), shape=(n, n))
    return d, A, As, n


def test_bicgstab_matches_reference_solve(cuda):
    d, A, As, n = _fixture(cuda)
    b = torch.from_numpy(d["b"]).to(cuda)
    x, info = tg.bicgstab_solve(A, b, atol=1e-6, max_iter=2000, return_info=True)
    assert info.converged and not info.breakdown
    xs = spl.spsolve(As.tocsc(), d["b"])
    assert np.linalg.norm(x.cpu().numpy() - xs) <= 1e-10 * np.linalg.norm(xs)
    assert np.linalg.norm(x.cpu().numpy() - d["x"]) <= 1e-10 * np.linalg.norm(d["x"])
    x2 = tg.bicgstab_solve(A, b, atol=1e-6, max_iter=2000)
    assert torch.equal(x, x2), "the solve must be bitwise reproducible"


def test_bicgstab_zero_rhs_and_relative_threshold(cuda):
    d, A, As, n = _fixture(cuda)
    x, info = tg.bicgstab_solve(A, torch.zeros(n, dtype=torch.float64, device=cuda), return_info=True)
    assert info.converged and info.iterations == 0 and float(x.abs().max()) == 0.0
    b = torch.from_numpy(d["b"]).to(cuda)
    x, info = tg.bicgstab_solve(A, b, atol=0.0, rtol=1e-10, return_info=True)
    assert info.converged and info.relative_residual <= 1e-10
    r = b - A @ x
    assert float(r.norm() / b.norm()) <= 1e-9


def test_bicgstab_on_spd_system_agrees_with_cg(cuda):
    m = tg.gen_unit_square(24, jitter=0.2, seed=81).to(cuda)
    K = tg.LaplaceElementAssembler.from_mesh(m)(m.points)
    # a right-hand side of size 1e9: the reference's absolute safeguards
    # (t . t < 1e-12 sets omega = 0 and ends the solve) stay below the
    # threshold asked for
    bvec = tg.const_node_assembler(1.0).from_mesh(m)(m.points) * 1e9
    cond = tg.Condenser(m.boundary_mask)
    Ki, bi = cond(K, bvec)
    xc = tg.pcg_solve(Ki, bi, rtol=1e-13)
    xb, info = tg.bicgstab_solve(Ki, bi, atol=1e-12 * float(bi.norm()), return_info=True)
    assert info.converged
    assert rel_fro(xb, xc) <= 1e-10


def test_bicgstab_gradients(cuda):
    d, A, As, n = _fixture(cuda)
    vals = torch.from_numpy(d["values"]).to(cuda).requires_grad_(True)
    b = torch.from_numpy(d["b"]).to(cuda).requires_grad_(True)
    w = torch.from_numpy(d["w"]).to(cuda)
    Av = A.with_values(vals)
    x = Av.solve(b, method="bicgstab", atol=1e-6, max_iter=2000)
    (x * w).sum().backward()
    xs = spl.spsolve(As.tocsc(), d["b"])
    lam = spl.spsolve(As.T.tocsc(), d["w"])
    gv = -lam[d["row"]] * xs[d["col"]]
    assert np.linalg.norm(b.grad.cpu().numpy() - lam) <= 1e-9 * np.linalg.norm(lam)
    assert np.linalg.norm(vals.grad.cpu().numpy() - gv) <= 1e-9 * np.linalg.norm(gv)


def test_bicgstab_float32(cuda):
    d, A, As, n = _fixture(cuda)
    A32 = A.with_values(A.values.float())
    b = torch.from_numpy(d["b"]).float().to(cuda)
    x, info = tg.bicgstab_solve(A32, b, atol=0.0, rtol=1e-5, return_info=True)
    assert x.dtype == torch.float32 and info.converged
    xs = spl.spsolve(As.tocsc(), d["b"])
    assert np.linalg.norm(x.double().cpu().numpy() - xs) <= 1e-4 * np.linalg.norm(xs)


def test_solve_accepts_the_inherited_keywords(cuda):
    """SparseMatrix.solve with the keywords of the solve the reference's
    SparseMatrix inherits (as its examples call it: ``K.solve(F,
    backend="scipy")``, ``method="lu"``, ``is_spd=False``)."""
    m = tg.gen_unit_square(16, jitter=0.2, seed=82).to(cuda)
    K = tg.LaplaceElementAssembler.from_mesh(m)(m.points)
    b = tg.const_node_assembler(1.0).from_mesh(m)(m.points)
    Ki, bi = tg.Condenser(m.boundary_mask)(K, b)
    ref = tg.pcg_solve(Ki, bi, rtol=1e-13)
    for kw in ({"backend": "scipy"}, {"method": "lu"}, {"method": "cholesky", "backend": "cudss"},
               {"method": "cg", "preconditioner": "jacobi", "tol": 1e-12, "verbose": True}):
        x = Ki.solve(bi, **kw)
        assert rel_fro(x, ref) <= 1e-9, kw
    d, A, As, n = _fixture(cuda)
    b2 = torch.from_numpy(d["b"]).to(cuda)
    x = A.solve(b2, is_spd=False, tol=1e-12)
    xs = spl.spsolve(As.tocsc(), d["b"])
    assert np.linalg.norm(x.cpu().numpy() - xs) <= 1e-10 * np.linalg.norm(xs)


def test_direct_solver_calls_are_differentiable(cuda):
    """pcg_solve / bicgstab_solve with a right-hand side or values that
    require grad go through the adjoint solve (as SparseMatrix.solve does):
    the same gradients, and return_info still reports the forward solve."""
    mesh = tg.gen_unit_square(10, jitter=0.2, seed=91).to(cuda)
    K = tg.LaplaceElementAssembler.from_mesh(mesh)(mesh.points)
    b = tg.const_node_assembler(1.0).from_mesh(mesh)(mesh.points)
    Kc, bc = tg.Condenser(mesh.boundary_mask)(K, b)
    w = torch.linspace(-1.0, 1.0, bc.numel(), dtype=torch.float64, device=cuda)
    grads = []
    # (BiCGSTAB keeps the reference's absolute breakdown thresholds, 1e-12:
    # its right-hand side and the loss weights are scaled up; dL/db does not
    # depend on b and is linear in the weights)
    for solve, scale in ((lambda A, r: tg.pcg_solve(A, r, rtol=1e-13, return_info=True), 1.0),
                         (lambda A, r: tg.bicgstab_solve(A, r, atol=0.0, rtol=1e-9, return_info=True), 1e6),
                         (lambda A, r: (A.solve(r, rtol=1e-13), None), 1.0)):
        r = (bc.detach() * scale).requires_grad_(True)
        x, info = solve(Kc, r)
        if info is not None:
            assert info.relative_residual <= 1e-7
        (x * w * scale).sum().backward()
        grads.append(r.grad.clone() / scale)
    assert rel_fro(grads[0], grads[2]) <= 1e-10
    assert rel_fro(grads[1], grads[2]) <= 1e-6
